// Shape preparation on the device: the poles (k_poles) and the simplification (k_simplify) of many
// shapes at once.
//
// compute_pole (fail_fast/pole.rs:52-77) is a breadth-first branch and bound over a cell tree of
// MAX_POI_TREE_DEPTH = 10 levels (pole.rs:79): each cell's centre is scored by its signed distance to
// the shape's border and to the poles found so far (POINode::new, pole.rs:90-120); the queue keeps the
// best cell seen (strict >) and splits a cell into its four quadrants while its radius plus distance
// beats that best.  The queue is FIFO, so it pops the cells level by level, each level in the order
// its parents were split; that order is kept here exactly:
//   * a level's cells are scored in parallel, G lanes per cell (G from 32 down to 1 as levels widen),
//     each lane taking every G-th edge and pole; the lanes' partial minima and crossing counts combine
//     exactly (min of correctly rounded square roots = square root of the min, sums of integers);
//   * the running best at each cell is an inclusive prefix maximum over the level's cells in queue
//     order (NaN ignored, as `>` ignores it), so every split decision is the queue's own;
//   * the best cell is the first one in queue order reaching the maximum, as strict `>` keeps it;
//   * the children of the split cells are compacted in parent order into the next level's list.
// generate_surrogate_poles (pole.rs:12-47) then repeats compute_pole with the coverage limits, one
// CTA per shape (shapes handed out by a counter), the shape's vertices and poles in shared memory.
// Every score uses the predicates of geom.cuh, compiled with the same rounding rules as the host
// preparation, so each pole is bit-identical to the host's (and the oracle's).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstdint>

#include "../../include/jcde.h"
#include "geom.cuh"

namespace jcde {
namespace {

// threads of one shape's CTA: 512 (two CTAs per SM) for batches that fill the GPU, 1024 (one per
// SM, twice the lanes on each level) for batches of at most one shape per SM
constexpr int PP_THREADS_WIDE = 1024;
constexpr uint32_t PP_LEVEL_CAP = 16384;   // cells of one level of one compute_pole
constexpr uint32_t PP_MAX_POLES = 1000;    // generate_surrogate_poles' bound (pole.rs:42-45)
constexpr int PP_DEPTH = 10;               // MAX_POI_TREE_DEPTH (pole.rs:79)
constexpr float PP_PI = 3.14159265358979323846f;
constexpr unsigned FULL = 0xffffffffu;

// per-shape status codes written to `status`
constexpr int32_t PS_OK = 0, PS_BAD_SHAPE = 1, PS_NO_POLE = 2, PS_TOO_MANY = 3, PS_LEVEL_CAP = 4, PS_OUT_CAP = 5;

struct PoleArgs {
    const float2* verts;
    const uint32_t* voff;
    uint32_t n_shapes, vmax;
    const float* area;   // nullptr: the poi of each shape (no initial poles, one pole)
    const float* poi;    // (x, y, r) per shape, the first pole
    uint32_t lim_n[3];
    float lim_cov[3];
    uint32_t n_lim;
    float* out;          // n_shapes x cap x 3
    uint32_t cap;
    uint32_t* n_out;
    int32_t* status;
    const uint32_t* order;   // processing order of the shapes (nullptr: batch order)
    float4* scratch;     // gridDim x 2 x PP_LEVEL_CAP cells
    uint32_t* next;      // shape counter
};

template <int PP_THREADS>
struct PoleShared {
    static constexpr int PP_WARPS = PP_THREADS / 32;
    float d[PP_THREADS];
    float r[PP_THREADS];
    float wmax[PP_WARPS];
    uint32_t wsum[PP_WARPS];
    Box bbox;
    Pt best_c;
    float best_r, total;
    uint32_t first2[2];   // first cell reaching a chunk's maximum, alternating between chunks
    uint32_t nv, np, shape, have, done;
    int32_t err;
};

__device__ __forceinline__ float4 box4(const Box& b) { return make_float4(b.x0, b.y0, b.x1, b.y1); }
__device__ __forceinline__ Box box_of(const float4& f) { return Box{f.x, f.y, f.z, f.w}; }

// compute_pole (pole.rs:52-77) over the shape and poles in shared memory; the result lands in
// sh.best_c / sh.best_r with sh.have, or sh.err is set.  Called by every thread of the CTA.
// The queue's state (running best, children count) is kept by every thread in registers, updated
// identically from shared values, so a chunk of cells costs three barriers: after the scores,
// after the warp maxima, after the split counts.  The first-maximum slot alternates between two
// words, so the reset of one never races with a late read of the other.
template <int PP_THREADS>
__device__ void compute_pole(PoleShared<PP_THREADS>& sh, const float2* v, const float4* poles, float4* lvl_a,
                             float4* lvl_b) {
    constexpr int PP_WARPS = PP_THREADS / 32;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t below = (1u << lane) - 1u;
    if (tid == 0) {
        lvl_a[0] = box4(box_square(sh.bbox));
        sh.first2[0] = PP_THREADS;
        sh.first2[1] = PP_THREADS;
    }
    __syncthreads();
    const uint32_t nv = sh.nv, np = sh.np;
    const Box bb = sh.bbox;
    float best_r = 0.0f;            // the queue's best so far (0 before any: pole.rs:57)
    Pt best_c{0.f, 0.f};
    bool have = false, overflow = false;
    uint32_t n = 1, parity = 0;
    for (int lev = PP_DEPTH; lev >= 0 && n > 0 && !overflow; lev--) {
        uint32_t G = 32;
        while (G > 1 && (uint32_t)PP_THREADS / G < n) G >>= 1;
        const uint32_t per = PP_THREADS / G;
        uint32_t n_child = 0;
        for (uint32_t c0 = 0; c0 < n; c0 += per, parity ^= 1u) {
            const uint32_t slot = tid / G, lig = tid % G, ci = c0 + slot;
            const bool valid = ci < n;
            Pt c{0.f, 0.f};
            Box cb{0.f, 0.f, 0.f, 0.f};
            float sq = INFINITY, psep = FLT_MAX;
            int cnt = 0;
            bool pin = false;
            if (valid) {
                cb = box_of(lvl_a[ci]);
                c = box_mid(cb);
                // POINode::new (pole.rs:90-120): edges (edge.rs:63-87), PIP (simple_polygon.rs:255-292),
                // poles (circle.rs:527-531, 551-560)
                const bool in_box = box_hits_pt(bb, c);
                const Seg ray = pip_ray(bb, c);
                for (uint32_t j = lig; j < nv; j += G) {
                    const float2 a = v[j], b = v[j + 1 == nv ? 0 : j + 1];
                    const Seg e{Pt{a.x, a.y}, Pt{b.x, b.y}};
                    sq = fmn(sq, seg_sq_dist(e, c));
                    if (in_box) cnt += pip_edge_term(ray, e, c);
                }
                for (uint32_t k = lig; k < np; k += G) {
                    const float4 p = poles[k];
                    const Disk dk{Pt{p.x, p.y}, p.z};
                    pin |= disk_hits_pt(dk, c);
                    psep = fmn(psep, disk_sep_dist(dk, c));
                }
            }
            for (uint32_t o = G >> 1; o; o >>= 1) {
                sq = fmn(sq, __shfl_xor_sync(FULL, sq, o));
                cnt += __shfl_xor_sync(FULL, cnt, o);
                pin |= __shfl_xor_sync(FULL, (int)pin, o) != 0;
                psep = fmn(psep, __shfl_xor_sync(FULL, psep, o));
            }
            if (valid && lig == 0) {
                const bool inside = (cnt & 1) && !pin;
                const float dist = fmn(fmn(FLT_MAX, sqrtf(sq)), psep);
                sh.d[slot] = inside ? dist : -dist;
                sh.r[slot] = box_diameter(cb) / 2.0f;
            }
            __syncthreads();   // A: the chunk's scores
            if (tid == 0) sh.first2[parity ^ 1u] = PP_THREADS;   // the other word, for the next chunk
            // the queue's running best at each cell of the chunk: an inclusive prefix maximum
            const uint32_t nc = min(per, n - c0);
            const bool mine = (uint32_t)tid < nc;
            const float dt = mine ? sh.d[tid] : -INFINITY;
            float m = dt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const float x = __shfl_up_sync(FULL, m, o);
                if (lane >= o) m = fmaxf(m, x);
            }
            if (lane == 31) sh.wmax[warp] = m;
            __syncthreads();   // B: the warps' maxima
            const float carry = best_r;
            float pre = carry, all = carry;
            for (int w = 0; w < PP_WARPS; w++) {
                if (w < warp) pre = fmaxf(pre, sh.wmax[w]);
                all = fmaxf(all, sh.wmax[w]);
            }
            const float incl = fmaxf(pre, m);
            // pole.rs:67-73: split while radius + distance beats the best so far (level 0 never splits)
            const bool split = mine && lev > 0 && sh.r[tid] + dt > incl;
            const uint32_t bal = __ballot_sync(FULL, split);
            if (lane == 0) sh.wsum[warp] = __popc(bal);
            // strict `>` keeps the first cell reaching the chunk's maximum
            if (mine && all > carry && dt == all) atomicMin(&sh.first2[parity], (uint32_t)tid);
            __syncthreads();   // C: the split counts and the first maximum
            uint32_t base = n_child, total = 0;
            for (int w = 0; w < PP_WARPS; w++) {
                if (w < warp) base += sh.wsum[w];
                total += sh.wsum[w];
            }
            base += __popc(bal & below);
            if (n_child + total > PP_LEVEL_CAP / 4) {
                overflow = true;
                break;
            }
            if (split) {
                const Box pb = box_of(lvl_a[c0 + tid]);
#pragma unroll
                for (int q = 0; q < 4; q++) lvl_b[4 * base + q] = box4(box_quadrant(pb, q));
            }
            if (all > carry) {
                best_r = all;
                best_c = box_mid(box_of(lvl_a[c0 + sh.first2[parity]]));
                have = true;
            }
            n_child += total;
        }
        __syncthreads();   // the next level reads the children written above
        float4* t = lvl_a;
        lvl_a = lvl_b;
        lvl_b = t;
        n = 4 * n_child;   // four quadrants per split cell
    }
    if (tid == 0) {
        if (overflow) sh.err = PS_LEVEL_CAP;
        else if (!have) sh.err = PS_NO_POLE;
        sh.best_c = best_c;
        sh.best_r = best_r;
        sh.have = have;
    }
    __syncthreads();
}

template <int PP_THREADS>
__global__ void __launch_bounds__(PP_THREADS, 1024 / PP_THREADS) k_poles(PoleArgs a) {
    extern __shared__ float4 dyn[];
    __shared__ PoleShared<PP_THREADS> sh;
    float4* poles = dyn;   // PP_MAX_POLES (poles mode) or the one result slot (poi mode)
    float2* v = reinterpret_cast<float2*>(dyn + (a.area ? PP_MAX_POLES : 1));
    float4* lvl_a = a.scratch + (size_t)blockIdx.x * 2 * PP_LEVEL_CAP;
    float4* lvl_b = lvl_a + PP_LEVEL_CAP;
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) {
            const uint32_t k = atomicAdd(a.next, 1u);
            sh.shape = k < a.n_shapes ? (a.order ? a.order[k] : k) : 0xFFFFFFFFu;
        }
        __syncthreads();
        const uint32_t s = sh.shape;
        if (s >= a.n_shapes) return;
        const uint32_t v0 = a.voff[s], nv = a.voff[s + 1] - v0;
        if (nv < 3 || nv > a.vmax) {
            if (tid == 0) {
                a.status[s] = PS_BAD_SHAPE;
                a.n_out[s] = 0;
            }
            __syncthreads();
            continue;
        }
        for (uint32_t j = tid; j < nv; j += PP_THREADS) v[j] = a.verts[v0 + j];
        if (tid == 0) {
            sh.nv = nv;
            sh.err = 0;
            sh.done = 0;
            sh.np = 0;
            sh.total = 0.0f;
            if (a.area) {   // generate_surrogate_poles starts from the poi (pole.rs:16-17)
                const float pr = a.poi[3 * s + 2];
                poles[0] = make_float4(a.poi[3 * s], a.poi[3 * s + 1], pr, 0.f);
                sh.np = 1;
                sh.total = pr * pr * PP_PI;
            }
        }
        __syncthreads();
        if (tid == 0) {   // generate_bounding_box (simple_polygon.rs:122-133), in vertex order
            float x0 = FLT_MAX, y0 = FLT_MAX, x1 = -FLT_MAX, y1 = -FLT_MAX;
            for (uint32_t j = 0; j < nv; j++) {
                x0 = fmn(x0, v[j].x);
                y0 = fmn(y0, v[j].y);
                x1 = fmx(x1, v[j].x);
                y1 = fmx(y1, v[j].y);
            }
            sh.bbox = Box{x0, y0, x1, y1};
        }
        __syncthreads();
        for (;;) {
            compute_pole(sh, v, poles, lvl_a, lvl_b);
            if (sh.err) break;
            if (!a.area) {   // the poi: one pole, no earlier ones
                if (tid == 0) {
                    poles[0] = make_float4(sh.best_c.x, sh.best_c.y, sh.best_r, 0.f);
                    sh.np = 1;
                }
                __syncthreads();
                break;
            }
            if (tid == 0) {   // pole.rs:22-45: coverage limits
                const float r = sh.best_r;
                sh.total += r * r * PP_PI;
                poles[sh.np] = make_float4(sh.best_c.x, sh.best_c.y, r, 0.f);
                sh.np++;
                const float coverage = sh.total / a.area[s];
                bool found = false;
                uint32_t lim = 0;
                for (uint32_t i = 0; i < a.n_lim; i++)
                    if (coverage > a.lim_cov[i] && (!found || a.lim_n[i] < lim)) {
                        lim = a.lim_n[i];
                        found = true;
                    }
                if (found && sh.np >= lim) sh.done = 1;
                else if (sh.np >= PP_MAX_POLES) sh.err = PS_TOO_MANY;
            }
            __syncthreads();
            if (sh.done || sh.err) break;
        }
        const uint32_t np = sh.np;
        for (uint32_t k = tid; k < np && k < a.cap; k += PP_THREADS) {
            const float4 p = poles[k];
            float* o = a.out + ((size_t)s * a.cap + k) * 3;
            o[0] = p.x;
            o[1] = p.y;
            o[2] = p.z;
        }
        if (tid == 0) {
            a.n_out[s] = sh.err ? 0u : np;
            a.status[s] = sh.err ? sh.err : (np > a.cap ? PS_OUT_CAP : PS_OK);
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------------------
// simplify_shape (geometry/shape_modification.rs:48-144), one warp per shape.
//
// Each round lists the removal candidates in corner order (Concave / Collinear corners, Convex
// after Convex pairs; shape_modification.rs:62-99), orders them by area change with ties kept in
// corner order (a stable sort, NaN last as OrderedFloat puts it), and executes the first valid one
// if the whole shape's area stays within the tolerance.  The warp takes the candidates in that
// order without sorting: the next one is the least (area change, corner position) above the last
// rejected one, found by a warp minimum over 64-bit keys; validity tests the shape's edges over
// lanes.  The new area is summed by one lane in the reference's order (simple_polygon.rs:137-150).
// ------------------------------------------------------------------------------------------
constexpr int SP_WARPS = 4;   // shapes per CTA at a time

struct SimpArgs {
    const float2* verts;
    const uint32_t* voff;
    uint32_t n_shapes, vmax;
    const float* area;   // the shape's area (SPolygon::area)
    int deflate;         // ShapeModifyMode::Deflate (else Inflate)
    float tolerance;     // max_area_change_ratio
    float2* out;         // same layout as verts
    uint32_t* n_out;
    int32_t* status;
};

enum : int { SC_CONCAVE = 0, SC_COLLINEAR = 1, SC_CONVEX = 2 };
enum : int { SK_NONE = 0, SK_CONCAVE = 1, SK_COLLINEAR = 2, SK_CONVEX_CONVEX = 3 };

struct SCorner { uint32_t a, b, c; };

// corner at position k of the corner list (shape_modification.rs:62-77): (k-1, k, k+1), or for
// Deflate the reversed list with every corner flipped
__device__ __forceinline__ SCorner corner_at(uint32_t k, uint32_t n, int deflate) {
    if (!deflate) return SCorner{k == 0 ? n - 1 : k - 1, k, k + 1 == n ? 0 : k + 1};
    const uint32_t i = n - 1 - k;
    return SCorner{i + 1 == n ? 0 : i + 1, i, i == 0 ? n - 1 : i - 1};
}

// CornerType::from (shape_modification.rs:317-327)
__device__ __forceinline__ int corner_kind(float2 p1, float2 p2, float2 p3) {
    const float ax = p2.x - p1.x, ay = p2.y - p1.y;
    const float bx = p3.x - p1.x, by = p3.y - p1.y;
    const float cross = ax * by - ay * bx;
    return cross < 0.0f ? SC_CONCAVE : (cross == 0.0f ? SC_COLLINEAR : SC_CONVEX);
}

// calculate_intersection_in_front (shape_modification.rs:248-283) of edge (p1, p2) and edge (p3, p4)
__device__ __forceinline__ bool in_front(float2 p1, float2 p2, float2 p3, float2 p4, float2* out) {
    const float x1 = p1.x, y1 = p1.y, x2 = p2.x, y2 = p2.y, x3 = p3.x, y3 = p3.y, x4 = p4.x, y4 = p4.y;
    const float t_nom = (x2 - x4) * (y4 - y3) - (y2 - y4) * (x4 - x3);
    const float t_den = (x2 - x1) * (y4 - y3) - (y2 - y1) * (x4 - x3);
    const float u_nom = (x2 - x4) * (y2 - y1) - (y2 - y4) * (x2 - x1);
    const float u_den = (x2 - x1) * (y4 - y3) - (y2 - y1) * (x4 - x3);
    const float t = t_den != 0.0f ? t_nom / t_den : 0.0f;
    const float u = u_den != 0.0f ? u_nom / u_den : 0.0f;
    if (t < 0.0f && u < 0.0f) {
        *out = make_float2(x2 + t * (x1 - x2), y2 + t * (y1 - y2));
        return true;
    }
    return false;
}

// |triangle area| of calculate_area_delta (shape_modification.rs:146-174)
__device__ __forceinline__ float tri_area(float2 p0, float2 p1, float2 p2) {
    const float x0 = p0.x, y0 = p0.y, x1 = p1.x, y1 = p1.y, x2 = p2.x, y2 = p2.y;
    return fabsf((x0 * y1 + x1 * y2 + x2 * y0 - x0 * y2 - x1 * y0 - x2 * y1) / 2.0f);
}

__device__ __forceinline__ bool same_pt(float2 a, float2 b) { return a.x == b.x && a.y == b.y; }
__device__ __forceinline__ Seg seg_of(float2 a, float2 b) { return Seg{Pt{a.x, a.y}, Pt{b.x, b.y}}; }

// the candidate at position k: its kind, sort key bits (NaN last) and, for a convex pair, the
// replacing vertex (replacing_vertex_convex_convex_candidate, shape_modification.rs:234-246)
struct SCand {
    int kind;
    uint32_t key;
    bool has_v;
    float2 v;
    SCorner c1, c2;
};

__device__ __forceinline__ SCand cand_at(const float2* P, uint32_t k, uint32_t n, int deflate) {
    SCand r{};
    r.c2 = corner_at(k, n, deflate);
    const int t = corner_kind(P[r.c2.a], P[r.c2.b], P[r.c2.c]);
    float key = 0.0f;
    if (t == SC_CONCAVE) {
        r.kind = SK_CONCAVE;
        r.c1 = r.c2;
        key = tri_area(P[r.c2.a], P[r.c2.b], P[r.c2.c]);
    } else if (t == SC_COLLINEAR) {
        r.kind = SK_COLLINEAR;
        r.c1 = r.c2;
    } else {
        r.c1 = corner_at(k == 0 ? n - 1 : k - 1, n, deflate);
        if (corner_kind(P[r.c1.a], P[r.c1.b], P[r.c1.c]) != SC_CONVEX) return r;   // SK_NONE
        r.kind = SK_CONVEX_CONVEX;
        r.has_v = in_front(P[r.c1.a], P[r.c1.b], P[r.c2.c], P[r.c2.b], &r.v);
        key = r.has_v ? tri_area(P[r.c1.b], r.v, P[r.c2.b]) : INFINITY;
    }
    r.key = key != key ? 0x7FFFFFFFu : __float_as_uint(key);
    return r;
}

__global__ void __launch_bounds__(SP_WARPS * 32) k_simplify(SimpArgs a) {
    extern __shared__ float2 sp_dyn[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float2* P = sp_dyn + (size_t)w * a.vmax;
    for (uint32_t s = blockIdx.x * SP_WARPS + w; s < a.n_shapes; s += gridDim.x * SP_WARPS) {
        const uint32_t v0 = a.voff[s], n0 = a.voff[s + 1] - v0;
        if (n0 < 3 || n0 > a.vmax) {
            if (lane == 0) {
                a.status[s] = PS_BAD_SHAPE;
                a.n_out[s] = 0;
            }
            continue;
        }
        for (uint32_t j = lane; j < n0; j += 32) P[j] = a.verts[v0 + j];
        __syncwarp();
        const float area0 = a.area[s];
        uint32_t n = n0;
        for (uint32_t it = 0; it < n0 && n >= 4; it++) {
            // candidates in (key, position) order until a valid one (shape_modification.rs:101-108)
            unsigned long long lo = 0ull;
            SCand best{};
            bool found = false;
            for (;;) {
                unsigned long long m = ~0ull;
                for (uint32_t k = lane; k < n; k += 32) {
                    const SCand c = cand_at(P, k, n, a.deflate);
                    const unsigned long long key = ((unsigned long long)c.key << 32) | k;
                    if (c.kind != SK_NONE && key >= lo && key < m) m = key;
                }
#pragma unroll
                for (int o = 16; o; o >>= 1) {
                    const unsigned long long x = __shfl_xor_sync(FULL, m, o);
                    m = x < m ? x : m;
                }
                if (m == ~0ull) break;   // no (further) candidate
                const SCand c = cand_at(P, (uint32_t)(m & 0xFFFFFFFFu), n, a.deflate);
                // candidate_is_valid (shape_modification.rs:176-207)
                bool bad = false;
                if (c.kind == SK_CONVEX_CONVEX && !c.has_v) {
                    bad = true;
                } else if (c.kind != SK_COLLINEAR) {
                    float2 af[4];
                    int n_af;
                    Seg e1, e2;
                    if (c.kind == SK_CONCAVE) {
                        af[0] = P[c.c1.a];
                        af[1] = P[c.c1.b];
                        af[2] = P[c.c1.c];
                        af[3] = af[2];
                        n_af = 3;
                        e1 = seg_of(P[c.c1.a], P[c.c1.c]);
                        e2 = e1;
                    } else {
                        af[0] = P[c.c1.b];
                        af[1] = P[c.c1.a];
                        af[2] = P[c.c2.b];
                        af[3] = P[c.c2.c];
                        n_af = 4;
                        e1 = seg_of(P[c.c1.a], c.v);
                        e2 = seg_of(c.v, P[c.c2.c]);
                    }
                    for (uint32_t i = lane; i < n && !bad; i += 32) {
                        const float2 ls = P[i], le = P[i + 1 == n ? 0 : i + 1];
                        bool touch = false;
                        for (int q = 0; q < n_af; q++) touch |= same_pt(af[q], ls) || same_pt(af[q], le);
                        if (touch) continue;
                        const Seg l = seg_of(ls, le);
                        bad = seg_hits_seg(l, e1) || (c.kind == SK_CONVEX_CONVEX && seg_hits_seg(l, e2));
                    }
                    bad = __any_sync(FULL, bad);
                }
                if (!bad) {
                    best = c;
                    found = true;
                    break;
                }
                lo = m + 1;
            }
            if (!found) break;
            // execute_candidate (shape_modification.rs:217-232): drop corner c1.b; a convex pair
            // also puts the replacing vertex in place of c2.b.  Area of the result first, in the
            // reference's order (one lane), the shape updated only if it stays within tolerance.
            const uint32_t gone = best.c1.b;
            const bool repl = best.kind == SK_CONVEX_CONVEX;
            const uint32_t at = best.c2.b;
            int keep = 0;
            if (lane == 0) {
                const uint32_t m = n - 1;
                float sigma = 0.0f;
                auto vtx = [&](uint32_t i) {   // vertex i of the new list
                    const uint32_t src = i < gone ? i : i + 1;
                    return (repl && src == at) ? best.v : P[src];
                };
                float2 cur = vtx(0), first = cur;
                for (uint32_t i = 0; i < m; i++) {
                    const float2 nx = i + 1 == m ? first : vtx(i + 1);
                    sigma += (cur.y + nx.y) * (cur.x - nx.x);
                    cur = nx;
                }
                const float new_area = 0.5f * sigma;
                keep = fabsf(new_area - area0) / area0 <= a.tolerance;
            }
            keep = __shfl_sync(FULL, keep, 0);
            if (!keep) break;
            if (repl && lane == 0) P[at] = best.v;
            __syncwarp();
            for (uint32_t base = gone; base + 1 < n; base += 32) {   // close the gap at `gone`
                const uint32_t j = base + lane;
                const float2 nx = j + 1 < n ? P[j + 1] : make_float2(0.f, 0.f);
                __syncwarp();
                if (j + 1 < n) P[j] = nx;
                __syncwarp();
            }
            n--;
        }
        for (uint32_t j = lane; j < n; j += 32) a.out[v0 + j] = P[j];
        if (lane == 0) {
            a.n_out[s] = n;
            a.status[s] = PS_OK;
        }
        __syncwarp();
    }
}

size_t pole_smem(uint32_t vmax, bool poles_mode) {
    return (poles_mode ? PP_MAX_POLES : 1) * sizeof(float4) + (size_t)vmax * sizeof(float2);
}

// CTAs of one launch: every SM's worth of resident CTAs, at most one per shape; *wide selects the
// 1024-thread CTA (batches of at most one shape per SM)
template <int T>
jcde_status pole_occupancy(size_t smem, int* per_sm) {
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_poles<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return JCDE_ERR_ARG;   // more vertices than shared memory holds
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_poles<T>, T, smem) != cudaSuccess || *per_sm < 1)
        return JCDE_ERR_ARG;
    return JCDE_OK;
}

jcde_status pole_grid(uint32_t n_shapes, uint32_t vmax, bool poles_mode, uint32_t* grid, bool* wide) {
    const size_t smem = pole_smem(vmax, poles_mode);
    int dev = 0, n_sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return JCDE_ERR_CUDA;
    *wide = n_shapes <= (uint32_t)n_sms;
    jcde_status st = *wide ? pole_occupancy<PP_THREADS_WIDE>(smem, &per_sm) : pole_occupancy<512>(smem, &per_sm);
    if (st) return st;
    *grid = std::max<uint32_t>(1u, std::min<uint32_t>(n_shapes, (uint32_t)(n_sms * per_sm)));
    return JCDE_OK;
}

// workspace: shape counter | per-shape counts of a poi batch | two level lists per CTA
size_t pole_workspace(uint32_t n_shapes, uint32_t grid) {
    return 256 + (((size_t)n_shapes * sizeof(uint32_t) + 255) & ~(size_t)255) +
           (size_t)grid * 2 * PP_LEVEL_CAP * sizeof(float4);
}

jcde_status launch_poles(PoleArgs a, void* ws, uint64_t ws_bytes, cudaStream_t s) {
    if (a.n_shapes == 0) return JCDE_OK;
    uint32_t grid = 0;
    bool wide = false;
    jcde_status st = pole_grid(a.n_shapes, a.vmax, a.area != nullptr, &grid, &wide);
    if (st) return st;
    const size_t need = pole_workspace(a.n_shapes, grid);
    void* own = nullptr;
    if (!ws) {
        if (cudaMallocAsync(&own, need, s) != cudaSuccess) return JCDE_ERR_CUDA;
        ws = own;
    } else if (ws_bytes < need || (reinterpret_cast<uintptr_t>(ws) & 255)) {
        return JCDE_ERR_ARG;
    }
    char* w = static_cast<char*>(ws);
    a.next = reinterpret_cast<uint32_t*>(w);
    if (!a.n_out) a.n_out = reinterpret_cast<uint32_t*>(w + 256);
    a.scratch = reinterpret_cast<float4*>(w + 256 + (((size_t)a.n_shapes * sizeof(uint32_t) + 255) & ~(size_t)255));
    if (cudaMemsetAsync(a.next, 0, sizeof(uint32_t), s) != cudaSuccess) st = JCDE_ERR_CUDA;
    if (!st) {
        const size_t smem = pole_smem(a.vmax, a.area != nullptr);
        if (wide) k_poles<PP_THREADS_WIDE><<<grid, PP_THREADS_WIDE, smem, s>>>(a);
        else k_poles<512><<<grid, 512, smem, s>>>(a);
        if (cudaGetLastError() != cudaSuccess) st = JCDE_ERR_CUDA;
    }
    if (own && cudaFreeAsync(own, s) != cudaSuccess) st = JCDE_ERR_CUDA;
    return st;
}

}  // namespace
}  // namespace jcde

using namespace jcde;

extern "C" jcde_status jcde_simplify_batch(const float* d_xy, const uint32_t* d_voff, uint32_t n_shapes,
                                           uint32_t max_vertices, const float* d_area, int deflate, float tolerance,
                                           float* d_xy_out, uint32_t* d_n_out, int32_t* d_status, void* stream) {
    if (n_shapes == 0) return JCDE_OK;
    if (!d_xy || !d_voff || !d_area || !d_xy_out || !d_n_out || !d_status || max_vertices < 3) return JCDE_ERR_ARG;
    SimpArgs a{reinterpret_cast<const float2*>(d_xy), d_voff, n_shapes, max_vertices, d_area, deflate != 0, tolerance,
               reinterpret_cast<float2*>(d_xy_out), d_n_out, d_status};
    const size_t smem = (size_t)SP_WARPS * max_vertices * sizeof(float2);
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_simplify, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return JCDE_ERR_ARG;   // more vertices than shared memory holds
    int dev = 0, n_sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return JCDE_ERR_CUDA;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_simplify, SP_WARPS * 32, smem) != cudaSuccess || per_sm < 1)
        return JCDE_ERR_ARG;
    const uint32_t grid = std::min<uint32_t>((n_shapes + SP_WARPS - 1) / SP_WARPS, (uint32_t)(n_sms * per_sm));
    k_simplify<<<grid, SP_WARPS * 32, smem, (cudaStream_t)stream>>>(a);
    return cudaGetLastError() == cudaSuccess ? JCDE_OK : JCDE_ERR_CUDA;
}

extern "C" uint64_t jcde_poles_workspace_bytes(uint32_t n_shapes, uint32_t max_vertices, int with_poles) {
    uint32_t grid = 0;
    bool wide = false;
    if (n_shapes == 0 || pole_grid(n_shapes, max_vertices, with_poles != 0, &grid, &wide)) return 0;
    return pole_workspace(n_shapes, grid);
}

extern "C" jcde_status jcde_poi_batch(const float* d_xy, const uint32_t* d_voff, uint32_t n_shapes, uint32_t max_vertices,
                                      float* d_poi, int32_t* d_status, const uint32_t* d_order, void* d_workspace,
                                      uint64_t workspace_bytes, void* stream) {
    if (n_shapes && (!d_xy || !d_voff || !d_poi || !d_status || max_vertices < 3)) return JCDE_ERR_ARG;
    PoleArgs a{};
    a.verts = reinterpret_cast<const float2*>(d_xy);
    a.voff = d_voff;
    a.n_shapes = n_shapes;
    a.vmax = max_vertices;
    a.out = d_poi;
    a.cap = 1;
    a.status = d_status;
    a.order = d_order;
    return launch_poles(a, d_workspace, workspace_bytes, (cudaStream_t)stream);
}

extern "C" jcde_status jcde_surrogate_poles_batch(const float* d_xy, const uint32_t* d_voff, uint32_t n_shapes,
                                                  uint32_t max_vertices, const float* d_area, const float* d_poi,
                                                  const jcde_config* cfg, float* d_poles, uint32_t cap,
                                                  uint32_t* d_n_out, int32_t* d_status, const uint32_t* d_order,
                                                  void* d_workspace, uint64_t workspace_bytes, void* stream) {
    if (!cfg || cfg->n_pole_limits > 3) return JCDE_ERR_ARG;
    if (n_shapes && (!d_xy || !d_voff || !d_area || !d_poi || !d_poles || !cap || !d_n_out || !d_status ||
                     max_vertices < 3))
        return JCDE_ERR_ARG;
    PoleArgs a{};
    a.verts = reinterpret_cast<const float2*>(d_xy);
    a.voff = d_voff;
    a.n_shapes = n_shapes;
    a.vmax = max_vertices;
    a.area = d_area;
    a.poi = d_poi;
    for (uint32_t i = 0; i < cfg->n_pole_limits; i++) {
        a.lim_n[i] = cfg->pole_limit_n[i];
        a.lim_cov[i] = cfg->pole_limit_coverage[i];
    }
    a.n_lim = cfg->n_pole_limits;
    a.out = d_poles;
    a.cap = cap;
    a.n_out = d_n_out;
    a.status = d_status;
    a.order = d_order;
    return launch_poles(a, d_workspace, workspace_bytes, (cudaStream_t)stream);
}
