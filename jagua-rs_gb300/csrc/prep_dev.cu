// Shape preparation on the device: the poles of many shapes at once.
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
// restatement, so each pole is bit-identical to the host's and to the reference's.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstdint>

#include "../../include/jcde.h"
#include "geom.cuh"

namespace jcde {
namespace {

constexpr int PP_THREADS = 512;
constexpr int PP_WARPS = PP_THREADS / 32;
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

struct PoleShared {
    float d[PP_THREADS];
    float r[PP_THREADS];
    float wmax[PP_WARPS];
    uint32_t wsum[PP_WARPS];
    Box bbox;
    Pt best_c;
    float best_r, total;
    uint32_t nv, np, n_cells, n_child, first, shape, have, done;
    int32_t err;
};

__device__ __forceinline__ float4 box4(const Box& b) { return make_float4(b.x0, b.y0, b.x1, b.y1); }
__device__ __forceinline__ Box box_of(const float4& f) { return Box{f.x, f.y, f.z, f.w}; }

// compute_pole (pole.rs:52-77) over the shape and poles in shared memory; the result lands in
// sh.best_c / sh.best_r with sh.have, or sh.err is set.  Called by every thread of the CTA.
__device__ void compute_pole(PoleShared& sh, const float2* v, const float4* poles, float4* lvl_a, float4* lvl_b) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t below = (1u << lane) - 1u;
    if (tid == 0) {
        lvl_a[0] = box4(box_square(sh.bbox));
        sh.n_cells = 1;
        sh.best_r = 0.0f;
        sh.have = 0;
        sh.first = PP_THREADS;
    }
    __syncthreads();
    const uint32_t nv = sh.nv, np = sh.np;
    const Box bb = sh.bbox;
    for (int lev = PP_DEPTH; lev >= 0; lev--) {
        const uint32_t n = sh.n_cells;
        if (n == 0 || sh.err) break;
        uint32_t G = 32;
        while (G > 1 && (uint32_t)PP_THREADS / G < n) G >>= 1;
        const uint32_t per = PP_THREADS / G;
        if (tid == 0) sh.n_child = 0;
        for (uint32_t c0 = 0; c0 < n; c0 += per) {
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
            __syncthreads();
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
            const float carry = sh.best_r;
            __syncthreads();
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
            if (mine && all > carry && dt == all) atomicMin(&sh.first, (uint32_t)tid);
            __syncthreads();
            uint32_t base = sh.n_child, total = 0;
            for (int w = 0; w < PP_WARPS; w++) {
                if (w < warp) base += sh.wsum[w];
                total += sh.wsum[w];
            }
            base += __popc(bal & below);
            const bool room = sh.n_child + total <= PP_LEVEL_CAP / 4;
            if (split && room) {
                const Box pb = box_of(lvl_a[c0 + tid]);
#pragma unroll
                for (int q = 0; q < 4; q++) lvl_b[4 * base + q] = box4(box_quadrant(pb, q));
            }
            __syncthreads();
            if (tid == 0) {
                if (!room) sh.err = PS_LEVEL_CAP;
                if (all > carry) {
                    sh.best_r = all;
                    sh.best_c = box_mid(box_of(lvl_a[c0 + sh.first]));
                    sh.have = 1;
                }
                sh.first = PP_THREADS;
                sh.n_child += total;
            }
            __syncthreads();
            if (sh.err) break;
        }
        float4* t = lvl_a;
        lvl_a = lvl_b;
        lvl_b = t;
        if (tid == 0) sh.n_cells = 4 * sh.n_child;   // four quadrants per split cell
        __syncthreads();
    }
    if (tid == 0 && !sh.err && !sh.have) sh.err = PS_NO_POLE;
    __syncthreads();
}

__global__ void __launch_bounds__(PP_THREADS, 2) k_poles(PoleArgs a) {
    extern __shared__ float4 dyn[];
    __shared__ PoleShared sh;
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
            sh.first = PP_THREADS;
        }
        __syncthreads();
    }
}

size_t pole_smem(uint32_t vmax, bool poles_mode) {
    return (poles_mode ? PP_MAX_POLES : 1) * sizeof(float4) + (size_t)vmax * sizeof(float2);
}

// CTAs of one launch: every SM's worth of resident CTAs, at most one per shape
jcde_status pole_grid(uint32_t n_shapes, uint32_t vmax, bool poles_mode, uint32_t* grid) {
    const size_t smem = pole_smem(vmax, poles_mode);
    int dev = 0, n_sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return JCDE_ERR_CUDA;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_poles, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return JCDE_ERR_ARG;   // more vertices than shared memory holds
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_poles, PP_THREADS, smem) != cudaSuccess || per_sm < 1)
        return JCDE_ERR_ARG;
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
    jcde_status st = pole_grid(a.n_shapes, a.vmax, a.area != nullptr, &grid);
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
        k_poles<<<grid, PP_THREADS, pole_smem(a.vmax, a.area != nullptr), s>>>(a);
        if (cudaGetLastError() != cudaSuccess) st = JCDE_ERR_CUDA;
    }
    if (own && cudaFreeAsync(own, s) != cudaSuccess) st = JCDE_ERR_CUDA;
    return st;
}

}  // namespace
}  // namespace jcde

using namespace jcde;

extern "C" uint64_t jcde_poles_workspace_bytes(uint32_t n_shapes, uint32_t max_vertices, int with_poles) {
    uint32_t grid = 0;
    if (n_shapes == 0 || pole_grid(n_shapes, max_vertices, with_poles != 0, &grid)) return 0;
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
