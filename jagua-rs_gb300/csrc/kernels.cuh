// sm_103a kernels of the CDE query path.
//
// One warp resolves one candidate placement (item, transformation).  The reference answers a query
// sequentially (lbf/benches/ci_bench.rs:107-121): the fail-fast poles of the surrogate are walked
// down the quadtree from the root (cd_engine.rs:204-223), then every edge of the transformed item
// is walked down from the virtual root (cd_engine.rs:160-173), then the partially present hazards of
// the virtual root are tested for containment (cd_engine.rs:176-193).  Its answer is the OR of all
// those tests, so the warp spreads them over lanes:
//   * probes (poles, piers, item edges) — each lane walks one probe's descent with a 4-bit
//     pending-children mask per level packed into one 64-bit register (no stack memory).  Probes
//     are handed to lanes dynamically (ballot rank) as their previous walk ends, each loop
//     iteration is one node visit per lane, and a hit anywhere ends the query at once;
//   * containment — lanes evaluate the FPA bounding-box relation of one hazard each, then the
//     warp runs each needed ray-cast point-in-polygon test cooperatively (edges over lanes,
//     crossing counts by ballot + popc).
// Collect queries (cd_engine.rs:261-310) walk the same probes with the collect rule of
// qt_node.rs:151-191 and gather hazard keys in a per-warp shared-memory bitset, which is emitted
// in ascending key order after one warp-aggregated atomicAdd reserves the output range.
#pragma once
#include <cfloat>
#include <cstdint>
#include <type_traits>

#include "geom.cuh"
#include "qtree.hpp"

namespace jcde {

constexpr uint32_t FULL = 0xffffffffu;
constexpr int MAX_DEPTH = 15;   // 4 pending bits per level in a 64-bit register

// Work counters of the polygon pass, compiled in only with -DJCDE_POLY_STATS (a measurement build;
// every count is an atomic add, so such a build is not for timing).  Slots: 0 loop iterations,
// 1 active lanes summed over iterations, 2 iterations with <= 8 active lanes, 3 internal-node
// visits, 4 leaf visits, 5 leaf entries scanned, 6 edge groups tested, 7 hazard edges tested,
// 8 queries, 9 queries decided by the edge loop, 10 containment tests run as a warp, 11 jobs
// (edges, or listed edge walks below the virtual root), 12 visits ending at Entire/None nodes.
#ifdef JCDE_POLY_STATS
static __device__ unsigned long long g_poly_stats[16];
#define PSTAT(i, v) atomicAdd(&g_poly_stats[i], (unsigned long long)(v))
#else
#define PSTAT(i, v) ((void)0)
#endif

struct View {
    const DNode* __restrict__ nodes;
    const DEntry* __restrict__ entries;
    const float4* __restrict__ edges;
    const DHaz* __restrict__ haz;
    const float2* __restrict__ hverts;
    const DItem* __restrict__ items;
    const float2* __restrict__ iverts;
    const float4* __restrict__ poles;
    const float4* __restrict__ piers;
    const uint8_t* __restrict__ strength;   // strongest unfiltered presence per node
    const uint32_t* __restrict__ mask;      // ignored-key bitmask, nullptr = NoFilter
    const uint32_t* __restrict__ nedges;    // active edges per node (collect)
    const float4* __restrict__ cbox;        // box of each tile of 1 << eg_shift edges (nullptr: not kept)
    uint32_t eg_shift = 3;                  // log2 of the edge tile (2, 3 or 4)
    // nodes [0, n_staged) (the top levels, breadth-first) and their strengths kept in shared memory by
    // a staging kernel instance (read only where the code is compiled for staging)
    const DNode* snode = nullptr;
    const uint8_t* sstr = nullptr;
    uint32_t n_staged = 0;
    Box cde;
    float coord_max;   // the largest coordinate magnitude of the CDE box (every hazard lies inside it)
    uint32_t n_items, n_slots, cd_threshold;
    int32_t exterior;
    // hazard poles binned in a uniform grid over the CDE box (overlap proxy)
    const float4* __restrict__ hpoles;      // x, y, r, hazard key (bits)
    const uint32_t* __restrict__ hp_start;  // cell c holds hpoles[hp_start[c], hp_start[c+1])
    float hp_x0, hp_y0, hp_inv_cs, hp_rmax;
    int32_t hp_g;
    const float4* __restrict__ hpoles_c;      // the same poles binned in a coarse grid (cells 8x larger)
    const uint32_t* __restrict__ hp_start_c;
    float hp_inv_cs_c;
    int32_t hp_g_c;
};

// A raw (already transformed) query shape for the single-polygon entry points.
struct RawShape {
    const float2* verts;   // nullptr: shapes come from items + transformations
    uint32_t nv;
    float poi_x, poi_y, poi_r;
};

__device__ __forceinline__ bool filtered(const View& v, uint32_t k) {
    return v.mask != nullptr && ((__ldg(&v.mask[k >> 5]) >> (k & 31)) & 1u);
}
__device__ __forceinline__ Box ld_box(const float4* p) {
    float4 f = __ldg(p);
    return Box{f.x, f.y, f.z, f.w};
}
__device__ __forceinline__ DNode ld_node(const View& v, int i) {
    const float4* p = reinterpret_cast<const float4*>(v.nodes + i);
    float4 a = __ldg(p);
    int4 b = __ldg(reinterpret_cast<const int4*>(p + 1));
    DNode d;
    d.box = Box{a.x, a.y, a.z, a.w};
    d.child = b.x;
    d.parent = b.y;
    d.hz_off = (uint32_t)b.z;
    d.hz_cnt = (uint32_t)b.w;
    return d;
}
__device__ __forceinline__ int4 ld_node_links(const View& v, int i) {
    return __ldg(reinterpret_cast<const int4*>(v.nodes + i) + 1);
}
constexpr uint32_t MAX_STAGING_DEPTH = 4;
// Node, strength and parent of node i: from shared memory when staged (S and i < n_staged).
template <bool S>
__device__ __forceinline__ DNode node_at(const View& v, int i) {
    if constexpr (S) {
        if (i < (int)v.n_staged) return v.snode[i];
    }
    return ld_node(v, i);
}
template <bool S>
__device__ __forceinline__ uint32_t strength_at(const View& v, int i) {
    if constexpr (S) {
        if (i < (int)v.n_staged) return v.sstr[i];
    }
    return __ldg(&v.strength[i]);
}
template <bool S>
__device__ __forceinline__ int parent_at(const View& v, int i) {
    if constexpr (S) {
        if (i < (int)v.n_staged) return v.snode[i].parent;
    }
    return __ldg(&v.nodes[i].parent);
}
__device__ __forceinline__ DEntry ld_entry(const View& v, uint32_t i) {
    const float4* p = reinterpret_cast<const float4*>(v.entries + i);
    float4 a = __ldg(p);
    uint4 b = __ldg(reinterpret_cast<const uint4*>(p + 1));
    DEntry e;
    e.ff = Box{a.x, a.y, a.z, a.w};
    e.hkey = b.x;
    e.edge_off = b.y;
    e.edge_cnt = b.z;
    e.presence = b.w;
    return e;
}
__device__ __forceinline__ Seg ld_edge(const View& v, uint32_t i) {
    float4 f = __ldg(&v.edges[i]);
    return Seg{Pt{f.x, f.y}, Pt{f.z, f.w}};
}

// Probe-type dispatch: the queryable entities of qt_traits.rs (Circle for poles, Edge otherwise).
__device__ __forceinline__ bool p_hits_box(const Disk& d, const Box& b) { return disk_hits_box(d, b); }
__device__ __forceinline__ bool p_hits_box(const Seg& s, const Box& b) { return box_hits_seg(b, s); }
__device__ __forceinline__ bool p_hits_seg(const Disk& d, const Seg& e) { return disk_hits_seg(d, e); }
__device__ __forceinline__ bool p_hits_seg(const Seg& s, const Seg& e) { return seg_hits_seg(s, e); }
// The lane groups of the small-batch surrogate pass keep the pole-edge test with its division: its
// end-point branches cost the groups' lockstep leaf loops more than the division they save.
__device__ __forceinline__ bool p_hits_seg_group(const Disk& d, const Seg& e) { return disk_hits_seg_div(d, e); }
__device__ __forceinline__ bool p_hits_seg_group(const Seg& s, const Seg& e) { return seg_hits_seg(s, e); }
__device__ __forceinline__ uint32_t p_quad_mask(const Disk& d, const Box& b) { return disk_quadrant_mask(d, b); }
__device__ __forceinline__ uint32_t p_quad_mask(const Seg& s, const Box& b) { return seg_quadrant_mask(s, b); }
// The collect walks' form (each lane walks its probe to the end): the one-quadrant shortcut for edges.
__device__ __forceinline__ uint32_t p_quad_mask_walk(const Disk& d, const Box& b) { return disk_quadrant_mask(d, b); }
__device__ __forceinline__ uint32_t p_quad_mask_walk(const Seg& s, const Box& b) { return seg_quadrant_mask_short(s, b); }

// Breadth-first flattening stores the children of every node as one quartet, and quartets fill
// indices 1, 5, 9, ... in order, so the quartet holding node i >= 1 starts at quartet_base(i).
__device__ __forceinline__ int quartet_base(int i) { return 1 + ((i - 1) & ~3); }

// One lane's (or thread's) walk of the quadtree below a start node.  `pend` keeps 4 pending-child
// bits per level below the start (32 bits cover 8 levels, 64 bits 16); `qb` is the quartet of
// the deepest pending level, so moving to a sibling costs no memory access.
template <typename PendT>
struct WalkT {
    int node;    // node to visit next; -1 = idle (needs a probe), -2 = no probe left
    int depth;   // levels with pending children below the start node
    int qb;      // quartet base of level depth-1
    PendT pend;
};

// Next node of the walk in depth-first order, or -1 when the walk is finished.
template <typename PendT, bool S = false>
__device__ __forceinline__ int walk_next(const View& v, WalkT<PendT>& w) {
    while (w.depth > 0) {
        const int sh = 4 * (w.depth - 1);
        const uint32_t m = (uint32_t)(w.pend >> sh) & 0xFu;
        if (m) {
            const int i = __ffs(m) - 1;
            w.pend &= ~((PendT)1 << (sh + i));
            return w.qb + i;
        }
        if (--w.depth > 0) w.qb = quartet_base(parent_at<S>(v, w.qb));
    }
    return -1;
}

// Children mask m of node nd is pending below the current level (its slot is empty: every deeper
// slot is consumed before the walk moves on at a level).
template <typename PendT>
__device__ __forceinline__ void walk_push(WalkT<PendT>& w, uint32_t m, int child) {
    w.pend |= (PendT)m << (4 * w.depth);
    w.qb = child;
    w.depth++;
}

#ifndef JCDE_EDGE_GROUPS
#define JCDE_EDGE_GROUPS 1
#endif
// Leaf test of QTNode::collides (qt_node.rs:126-142): unfiltered Partial hazards, ff box first.
// `stop` (shared memory, may be null) is raised by the lane that finds a hit; the other lanes of
// the warp leave their leaf loops at the next check instead of finishing them.
template <class P>
__device__ __forceinline__ bool leaf_hits(const View& v, const P& p, const DNode& nd, volatile int* stop) {
    for (uint32_t k = 0; k < nd.hz_cnt; k++) {
        if (stop && *stop) return false;
        DEntry e = ld_entry(v, nd.hz_off + k);
        PSTAT(5, 1);
        // (the filter lookup, a dependent load, comes last: the tests commute)
        if (e.presence != PRES_PARTIAL || !p_hits_box(p, e.ff)) continue;   // qt_partial_hazard.rs:67-71
        if (filtered(v, e.hkey)) continue;
        if constexpr (std::is_same<P, Seg>::value) {
            if (JCDE_EDGE_GROUPS && v.cbox) {
                // groups of edges whose box misses the probe's box are skipped: edge_intersection
                // rejects every edge of such a group on the boxes' overlap (edge.rs:188-199)
                const float px0 = fmn(p.s.x, p.e.x), px1 = fmx(p.s.x, p.e.x);
                const float py0 = fmn(p.s.y, p.e.y), py1 = fmx(p.s.y, p.e.y);
                const uint32_t eg = 1u << v.eg_shift;
                for (uint32_t g = 0; g * eg < e.edge_cnt; g++) {
                    const float4 c = __ldg(&v.cbox[(e.edge_off >> v.eg_shift) + g]);
                    PSTAT(6, 1);
                    if (fmx(px0, c.x) > fmn(px1, c.z) || fmx(py0, c.y) > fmn(py1, c.w)) continue;
                    const uint32_t end = min(e.edge_cnt, g * eg + eg);
                    PSTAT(7, end - g * eg);
                    for (uint32_t j = g * eg; j < end; j++)
                        if (p_hits_seg(p, ld_edge(v, e.edge_off + j))) {
                            if (stop) *stop = 1;
                            return true;
                        }
                    if (stop && *stop) return false;
                }
                continue;
            }
        }
        if constexpr (std::is_same<P, Disk>::value) {
            if (JCDE_EDGE_GROUPS && v.cbox) {
                // a pole skips the groups farther than its radius plus a margin of 2^-14 of the
                // CDE box's coordinate magnitude, far above the rounding of the distance test
                // (circle.rs:506-510 with edge.rs:63-87), so no skipped edge could count as hit
                const float reach = p.r + v.coord_max * 0x1p-14f;
                const uint32_t eg = 1u << v.eg_shift;
                for (uint32_t g = 0; g * eg < e.edge_cnt; g++) {
                    const float4 c = __ldg(&v.cbox[(e.edge_off >> v.eg_shift) + g]);
                    if (c.x - p.c.x > reach || p.c.x - c.z > reach || c.y - p.c.y > reach || p.c.y - c.w > reach)
                        continue;
                    const uint32_t end = min(e.edge_cnt, g * eg + eg);
                    for (uint32_t j = g * eg; j < end; j++)
                        if (p_hits_seg(p, ld_edge(v, e.edge_off + j))) {
                            if (stop) *stop = 1;
                            return true;
                        }
                    if (stop && *stop) return false;
                }
                continue;
            }
        }
        for (uint32_t j = 0; j < e.edge_cnt; j++) {
            if (p_hits_seg(p, ld_edge(v, e.edge_off + j))) {
                if (stop) *stop = 1;
                return true;
            }
            if (stop && (j & 7) == 7 && *stop) return false;
        }
    }
    return false;
}

// Visit w.node for probe p (qt_node.rs:104-146) and advance the walk.  Returns true on a hit.
template <class P, typename PendT, bool S = false>
__device__ __forceinline__ bool walk_step(const View& v, const P& p, WalkT<PendT>& w, volatile int* stop) {
    const uint32_t st = strength_at<S>(v, w.node);
    if (st == PRES_ENTIRE) {
        PSTAT(12, 1);
        return true;
    }
    if (st == PRES_PARTIAL) {
        DNode nd = node_at<S>(v, w.node);
        if (nd.child >= 0) {
            PSTAT(3, 1);
            const uint32_t m = p_quad_mask(p, nd.box);
            if (m) walk_push(w, m, nd.child);
        } else {
            PSTAT(4, 1);
            if (leaf_hits(v, p, nd, stop)) return true;
        }
    } else {
        PSTAT(12, 1);
    }
    w.node = walk_next<PendT, S>(v, w);
    return false;
}

__device__ __forceinline__ void bit_set(uint32_t* bits, uint32_t k) { atomicOr(&bits[k >> 5], 1u << (k & 31)); }
__device__ __forceinline__ bool bit_get(const uint32_t* bits, uint32_t k) {
    return (((volatile const uint32_t*)bits)[k >> 5] >> (k & 31)) & 1u;
}

// Any edge of entry e hit by probe p; for an edge probe the edge groups whose box misses the
// probe's box are skipped (see leaf_hits).
template <class P>
__device__ __forceinline__ bool seg_group_hits(const View& v, const P& p, const DEntry& e) {
    if constexpr (std::is_same<P, Seg>::value) {
        if (JCDE_EDGE_GROUPS && v.cbox) {
            const float px0 = fmn(p.s.x, p.e.x), px1 = fmx(p.s.x, p.e.x);
            const float py0 = fmn(p.s.y, p.e.y), py1 = fmx(p.s.y, p.e.y);
            const uint32_t eg = 1u << v.eg_shift;
            for (uint32_t g = 0; g * eg < e.edge_cnt; g++) {
                const float4 c = __ldg(&v.cbox[(e.edge_off >> v.eg_shift) + g]);
                if (fmx(px0, c.x) > fmn(px1, c.z) || fmx(py0, c.y) > fmn(py1, c.w)) continue;
                const uint32_t end = min(e.edge_cnt, g * eg + eg);
                for (uint32_t j = g * eg; j < end; j++)
                    if (p_hits_seg(p, ld_edge(v, e.edge_off + j))) return true;
            }
            return false;
        }
    }
    if constexpr (std::is_same<P, Disk>::value) {
        if (JCDE_EDGE_GROUPS && v.cbox) {   // the margin of leaf_hits
            const float reach = p.r + v.coord_max * 0x1p-14f;
            const uint32_t eg = 1u << v.eg_shift;
            for (uint32_t g = 0; g * eg < e.edge_cnt; g++) {
                const float4 c = __ldg(&v.cbox[(e.edge_off >> v.eg_shift) + g]);
                if (c.x - p.c.x > reach || p.c.x - c.z > reach || c.y - p.c.y > reach || p.c.y - c.w > reach) continue;
                const uint32_t end = min(e.edge_cnt, g * eg + eg);
                for (uint32_t j = g * eg; j < end; j++)
                    if (p_hits_seg(p, ld_edge(v, e.edge_off + j))) return true;
            }
            return false;
        }
    }
    for (uint32_t j = 0; j < e.edge_cnt; j++)
        if (p_hits_seg(p, ld_edge(v, e.edge_off + j))) return true;
    return false;
}

// QTNode::collect_collisions (qt_node.rs:151-191) for one probe, continuing walk `w`.
template <class P, typename PendT>
__device__ void collect_walk_w(const View& v, const P& p, WalkT<PendT>& w, uint32_t* bits) {
    while (w.node >= 0) {
        DNode nd = ld_node(v, w.node);
        const bool now = __ldg(&v.nedges[w.node]) <= v.cd_threshold;
        if (nd.child >= 0 && !now) {
            const uint32_t m = p_quad_mask_walk(p, nd.box);
            if (m) walk_push(w, m, nd.child);
        } else {
            for (uint32_t k = 0; k < nd.hz_cnt; k++) {
                DEntry e = ld_entry(v, nd.hz_off + k);
                if (bit_get(bits, e.hkey)) continue;
                if (e.presence == PRES_ENTIRE) {
                    bit_set(bits, e.hkey);
                } else if (e.presence == PRES_PARTIAL && p_hits_box(p, e.ff)) {
                    if (seg_group_hits(v, p, e)) bit_set(bits, e.hkey);
                }
            }
        }
        w.node = walk_next(v, w);
    }
}
// ... for one probe from node `start`.
template <class P, typename PendT>
__device__ __forceinline__ void collect_walk(const View& v, const P& p, int start, uint32_t* bits) {
    WalkT<PendT> w{start, 0, 0, (PendT)0};
    collect_walk_w(v, p, w, bits);
}

// Float bits mapped to unsigned integers of the same order (for 64-bit atomicMin of (cost, index)).
__device__ __forceinline__ uint32_t orderable(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// Per-query shape: item vertices under the query's transformation, or a raw polygon.
struct QShape {
    const float2* verts;
    uint32_t nv;
    float c, s, tx, ty;
    bool raw;
    __device__ __forceinline__ Pt vtx(uint32_t k) const {
        float2 f = __ldg(&verts[k]);
        Pt p{f.x, f.y};
        return raw ? p : xform(p, c, s, tx, ty);
    }
    __device__ __forceinline__ Seg edge(uint32_t k) const { return Seg{vtx(k), vtx(k + 1 == nv ? 0 : k + 1)}; }
};

// SPolygon::generate_bounding_box (simple_polygon.rs:122-133) as a warp reduction.
__device__ __forceinline__ Box warp_bbox(const QShape& sh, int lane) {
    float x0 = FLT_MAX, y0 = FLT_MAX, x1 = -FLT_MAX, y1 = -FLT_MAX;
    for (uint32_t k = lane; k < sh.nv; k += 32) {
        Pt p = sh.vtx(k);
        x0 = fminf(x0, p.x);
        y0 = fminf(y0, p.y);
        x1 = fmaxf(x1, p.x);
        y1 = fmaxf(y1, p.y);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        x0 = fminf(x0, __shfl_xor_sync(FULL, x0, o));
        y0 = fminf(y0, __shfl_xor_sync(FULL, y0, o));
        x1 = fmaxf(x1, __shfl_xor_sync(FULL, x1, o));
        y1 = fmaxf(y1, __shfl_xor_sync(FULL, y1, o));
    }
    return Box{x0, y0, x1, y1};
}

// CDEngine::get_virtual_root (cd_engine.rs:314-327); children boxes are Rect::quadrants of the parent.
__device__ __forceinline__ int virtual_root(const View& v, const Box& sb) {
    int n = 0;
    for (;;) {
        DNode nd = ld_node(v, n);
        if (nd.child < 0) return n;
        int next = -1;
#pragma unroll
        for (int i = 0; i < 4; i++)
            if (next < 0 && box_surrounds(box_quadrant(nd.box, i), sb)) next = nd.child + i;
        if (next < 0) return n;
        n = next;
    }
}

// get_virtual_root with the four children of a level tested by lanes 0-3 at once; the first
// surrounding child in quadrant order is the one `find` takes (cd_engine.rs:318-321).
template <bool S = false>
__device__ __forceinline__ int virtual_root_warp(const View& v, const Box& sb, int lane) {
    int n = 0;
    for (;;) {
        const DNode nd = node_at<S>(v, n);
        if (nd.child < 0) return n;
        const bool ok = lane < 4 && box_surrounds(box_quadrant(nd.box, lane), sb);
        const uint32_t m = __ballot_sync(FULL, ok);
        if (!m) return n;
        n = nd.child + __ffs(m) - 1;
    }
}

// Ray-cast point-in-polygon (simple_polygon.rs:255-292) with the polygon's edges over the lanes.
__device__ __forceinline__ bool warp_pip_hazard(const View& v, const DHaz& h, Pt p, int lane) {
    if (!box_hits_pt(h.box, p)) return false;
    const Seg ray = pip_ray(h.box, p);
    const uint32_t nv = h.v_cnt_scope & 0x7fffffffu;
    uint32_t n = 0;
    for (uint32_t base = 0; base < nv; base += 32) {
        uint32_t k = base + lane;
        int t = 0;
        if (k < nv) {
            float2 a = __ldg(&v.hverts[h.v_off + k]);
            float2 b = __ldg(&v.hverts[h.v_off + (k + 1 == nv ? 0 : k + 1)]);
            t = pip_edge_term(ray, Seg{Pt{a.x, a.y}, Pt{b.x, b.y}}, p);
        }
        n += __popc(__ballot_sync(FULL, t));
    }
    return (n & 1u) == 1u;
}
__device__ __forceinline__ bool warp_pip_shape(const QShape& sh, const Box& sb, Pt p, int lane) {
    if (!box_hits_pt(sb, p)) return false;
    const Seg ray = pip_ray(sb, p);
    uint32_t n = 0;
    for (uint32_t base = 0; base < sh.nv; base += 32) {
        uint32_t k = base + lane;
        int t = 0;
        if (k < sh.nv) t = pip_edge_term(ray, sh.edge(k), p);
        n += __popc(__ballot_sync(FULL, t));
    }
    return (n & 1u) == 1u;
}

// CDEngine::detect_containment_collision (cd_engine.rs:231-255) for a hazard whose FPA bbox
// relation needs a point-in-polygon test: 1 = Surrounding, 2 = Enclosed.
__device__ __forceinline__ bool warp_containment(const View& v, const QShape& sh, const Box& sb, Pt spoi,
                                                 uint32_t hkey, int need, int lane) {
    DHaz h;
    {
        const float4* p = reinterpret_cast<const float4*>(v.haz + hkey);
        float4 a = __ldg(p), b = __ldg(p + 1);
        h.box = Box{a.x, a.y, a.z, a.w};
        h.poi_x = b.x;
        h.poi_y = b.y;
        h.v_off = __float_as_uint(b.z);
        h.v_cnt_scope = __float_as_uint(b.w);
    }
    bool contained = need == 1 ? warp_pip_hazard(v, h, spoi, lane) : warp_pip_shape(sh, sb, Pt{h.poi_x, h.poi_y}, lane);
    bool ext = (h.v_cnt_scope >> 31) != 0;
    return ext ? !contained : contained;
}

// Shape of query `qi`, loaded by 5 lanes and broadcast.
struct QueryHead {
    uint32_t item;
    float c, s, tx, ty;
};
__device__ __forceinline__ QueryHead load_query_words(const uint32_t* __restrict__ w5, int lane) {
    uint32_t w = lane < 5 ? __ldg(&w5[lane]) : 0u;
    QueryHead h;
    h.item = __shfl_sync(FULL, w, 0);
    h.c = __uint_as_float(__shfl_sync(FULL, w, 1));
    h.s = __uint_as_float(__shfl_sync(FULL, w, 2));
    h.tx = __uint_as_float(__shfl_sync(FULL, w, 3));
    h.ty = __uint_as_float(__shfl_sync(FULL, w, 4));
    return h;
}
__device__ __forceinline__ QueryHead load_query(const uint32_t* __restrict__ q, uint32_t qi, int lane) {
    return load_query_words(q + (size_t)qi * 5, lane);
}

// Undecided queries of the surrogate pass, compacted for the polygon pass: record k is 6 words
// (query index, then the query's 5 words) at rec + 6 k, appended with one atomic per warp; the
// polygon pass then reads the records in order instead of re-reading every query's verdict slot.
struct PendList {
    uint32_t* rec;     // nullptr: no list
    uint32_t* count;   // records written (zeroed before the surrogate pass)
};
constexpr uint32_t PEND_WORDS = 6;

constexpr int MODE_SURROGATE = 1;
constexpr int MODE_POLY = 2;
constexpr int POLY_WARPS = 8;
constexpr int SURR_THREADS = 256;
// Blocks per SM the surrogate passes are compiled for (the register budget): 0 leaves it to ptxas.
// Six (40 registers, 48 warps per SM) suit the memory-latency-bound thread-per-query pass: 0.153 ->
// 0.149 ms per 1M batch against ptxas's own 48 registers, the warp pass unchanged.
#ifndef JCDE_SURR_MIN_BLOCKS
#define JCDE_SURR_MIN_BLOCKS 6
#endif
#if JCDE_SURR_MIN_BLOCKS > 0
#define JCDE_SURR_BOUNDS __launch_bounds__(SURR_THREADS, JCDE_SURR_MIN_BLOCKS)
#else
#define JCDE_SURR_BOUNDS __launch_bounds__(SURR_THREADS)
#endif
constexpr uint8_t PENDING = 0xFFu;   // verdict slot of a query the surrogate pass left undecided

// Surrogate pass — CDEngine::detect_surrogate_collision (cd_engine.rs:204-223), one thread per
// query: the fail-fast poles, then the piers, each walked down from the root in the reference's
// order, stopping at the first hit.  A hit writes JCDE_COLLIDES; a miss writes `miss` (JCDE_FREE
// for a surrogate-only batch, PENDING when the polygon pass follows).
// Views of one or several layouts: a kernel reads the View of the layout a query belongs to.
struct MultiSrc {
    const View* __restrict__ views;     // one per layout
    const uint32_t* __restrict__ offs;  // layout l owns queries [offs[l], offs[l+1])
    uint32_t n_layouts;
    __device__ __forceinline__ uint32_t layout_of(uint32_t qi) const {
        uint32_t lo = 0, hi = n_layouts - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (__ldg(&offs[mid]) <= qi) lo = mid;
            else hi = mid - 1;
        }
        return lo;
    }
};

// With `n_pending`, every query the pass leaves undecided (miss = PENDING) is counted there.
// Returns true when the query is left undecided (PENDING).
template <typename PendT>
__device__ __forceinline__ bool surrogate_query(const View& v, const uint32_t* __restrict__ q, uint32_t qi,
                                                uint8_t* __restrict__ out, uint8_t miss,
                                                uint32_t* __restrict__ n_pending = nullptr) {
    const uint32_t* w5 = q + (size_t)qi * 5;
    const uint32_t item = __ldg(&w5[0]);
    const float c = __uint_as_float(__ldg(&w5[1])), s = __uint_as_float(__ldg(&w5[2]));
    const float tx = __uint_as_float(__ldg(&w5[3])), ty = __uint_as_float(__ldg(&w5[4]));
    if (item >= v.n_items) {
        out[qi] = 2;
        return false;
    }
    const DItem it = v.items[item];
    bool hit = false;
    for (uint32_t p = 0; p < it.n_ff_poles && !hit; p++) {
        const float4 pl = __ldg(&v.poles[it.pole_off + p]);
        const Disk d{xform(Pt{pl.x, pl.y}, c, s, tx, ty), pl.z};
        WalkT<PendT> w{0, 0, 0, (PendT)0};
        while (w.node >= 0 && !hit) hit = walk_step(v, d, w, nullptr);
    }
    for (uint32_t p = 0; p < it.n_piers && !hit; p++) {
        const float4 pr = __ldg(&v.piers[it.pier_off + p]);
        const Seg sg{xform(Pt{pr.x, pr.y}, c, s, tx, ty), xform(Pt{pr.z, pr.w}, c, s, tx, ty)};
        WalkT<PendT> w{0, 0, 0, (PendT)0};
        while (w.node >= 0 && !hit) hit = walk_step(v, sg, w, nullptr);
    }
    out[qi] = hit ? (uint8_t)1 : miss;
    if (n_pending && !hit && miss == PENDING) atomicAdd(n_pending, 1u);
    return !hit && miss == PENDING;
}

template <typename PendT, bool MULTI>
__global__ void JCDE_SURR_BOUNDS k_surrogate(View v, MultiSrc ms, const uint32_t* __restrict__ q,
                                                            uint32_t n, uint8_t* __restrict__ out, uint8_t miss,
                                                            const uint32_t* __restrict__ order,
                                                            uint32_t* __restrict__ next,
                                                            uint32_t* __restrict__ n_pending = nullptr,
                                                            PendList pend = PendList{nullptr, nullptr}) {
    if (next) {   // each warp takes the next 32 queries from the counter as it finishes
        const int lane = threadIdx.x & 31;
        for (;;) {
            uint32_t t = 0;
            if (lane == 0) t = atomicAdd(next, 32u);
            const uint32_t base = __shfl_sync(FULL, t, 0);
            if (base >= n) break;
            const uint32_t i = base + lane;
            bool undecided = false;
            uint32_t qi = 0;
            if (i < n) {
                qi = order ? __ldg(&order[i]) : i;
                if constexpr (MULTI) undecided = surrogate_query<PendT>(ms.views[ms.layout_of(qi)], q, qi, out, miss);
                else undecided = surrogate_query<PendT>(v, q, qi, out, miss, n_pending);
            }
            if (pend.rec) {
                const uint32_t bal = __ballot_sync(FULL, undecided);
                uint32_t at = 0;
                if (lane == 0 && bal) at = atomicAdd(pend.count, (uint32_t)__popc(bal));
                at = __shfl_sync(FULL, at, 0) + __popc(bal & ((1u << lane) - 1u));
                if (undecided) {
                    uint32_t* r = pend.rec + (size_t)at * PEND_WORDS;
                    const uint32_t* w5 = q + (size_t)qi * 5;
                    r[0] = qi;
                    #pragma unroll
                    for (int k = 0; k < 5; k++) r[1 + k] = __ldg(&w5[k]);
                }
            }
        }
        return;
    }
    const uint32_t stride = gridDim.x * SURR_THREADS;
    for (uint32_t i = blockIdx.x * SURR_THREADS + threadIdx.x; i < n; i += stride) {
        const uint32_t qi = order ? __ldg(&order[i]) : i;
        if constexpr (MULTI) surrogate_query<PendT>(ms.views[ms.layout_of(qi)], q, qi, out, miss);
        else surrogate_query<PendT>(v, q, qi, out, miss, n_pending);
    }
}

// The surrogate pass with a group of G lanes per query (a warp at G = 32), for batches too small to
// fill the GPU with one thread per query (each query's walk then sets the batch's latency).  The
// group follows each probe's walk together; at a leaf its lanes test the node's hazards' ff boxes
// G at a time, then the edges of every hazard whose box the probe hits, G at a time.  Same tests,
// same verdict.  Groups of one warp run their own queries independently (group-masked votes).
#ifndef JCDE_SURR_GROUP
#define JCDE_SURR_GROUP 32   // lanes per query in the small-batch surrogate pass
#endif
template <int G>
struct LaneGroup {
    static_assert(G == 1 || G == 2 || G == 4 || G == 8 || G == 16 || G == 32, "group sizes divide a warp");
    uint32_t lig, base;
    unsigned mask;
    __device__ __forceinline__ explicit LaneGroup(int lane)
        : lig((uint32_t)lane % G), base((uint32_t)lane - (uint32_t)lane % G),
          mask(G == 32 ? FULL : (((1u << (G & 31)) - 1u) << ((uint32_t)lane - (uint32_t)lane % G))) {}
};

template <class P, int G>
__device__ __forceinline__ bool leaf_hits_group(const View& v, const P& p, const DNode& nd, const LaneGroup<G>& g) {
    for (uint32_t b = 0; b < nd.hz_cnt; b += G) {
        const uint32_t k = b + g.lig;
        uint32_t eo = 0, ec = 0;
        bool cand = false;
        if (k < nd.hz_cnt) {
            const DEntry e = ld_entry(v, nd.hz_off + k);
            cand = e.presence == PRES_PARTIAL && p_hits_box(p, e.ff) && !filtered(v, e.hkey);
            eo = e.edge_off;
            ec = e.edge_cnt;
        }
        uint32_t m = __ballot_sync(g.mask, cand) >> g.base;   // the group's lanes, from bit 0
        while (m) {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            const uint32_t off = __shfl_sync(g.mask, eo, (int)g.base + src);
            const uint32_t cnt = __shfl_sync(g.mask, ec, (int)g.base + src);
            for (uint32_t jb = 0; jb < cnt; jb += G) {
                const uint32_t j = jb + g.lig;
                if (__any_sync(g.mask, j < cnt && p_hits_seg_group(p, ld_edge(v, off + j)))) return true;
            }
        }
    }
    return false;
}

template <class P, typename PendT, int G>
__device__ __forceinline__ bool walk_group(const View& v, const P& p, const LaneGroup<G>& g) {
    WalkT<PendT> w{0, 0, 0, (PendT)0};
    while (w.node >= 0) {
        const uint32_t st = __ldg(&v.strength[w.node]);
        if (st == PRES_ENTIRE) return true;
        if (st == PRES_PARTIAL) {
            const DNode nd = ld_node(v, w.node);
            if (nd.child >= 0) {
                const uint32_t m = p_quad_mask(p, nd.box);
                if (m) walk_push(w, m, nd.child);
            } else if (leaf_hits_group<P, G>(v, p, nd, g)) {
                return true;
            }
        }
        w.node = walk_next(v, w);
    }
    return false;
}

template <typename PendT, int G = JCDE_SURR_GROUP>
__global__ void JCDE_SURR_BOUNDS k_surrogate_warp(View v, const uint32_t* __restrict__ q, uint32_t n,
                                                                 uint8_t* __restrict__ out, uint8_t miss,
                                                                 const uint32_t* __restrict__ order,
                                                                 uint32_t* __restrict__ n_pending = nullptr,
                                                                 uint32_t* __restrict__ zero = nullptr) {
    pdl_wait();
    // `zero`: the polygon pass's work counter, cleared here (the polygon pass runs after this one on
    // the stream) instead of by a memset of its own
    if (zero && blockIdx.x == 0 && threadIdx.x == 0) *zero = 0u;
    const LaneGroup<G> g(threadIdx.x & 31);
    constexpr uint32_t gpb = SURR_THREADS / G;   // groups per block
    for (uint32_t i = blockIdx.x * gpb + threadIdx.x / G; i < n; i += gridDim.x * gpb) {
        const uint32_t qi = order ? __ldg(&order[i]) : i;
        const uint32_t* w5 = q + (size_t)qi * 5;
        const uint32_t item = __ldg(&w5[0]);
        if (item >= v.n_items) {
            if (g.lig == 0) out[qi] = 2;
            continue;
        }
        const float c = __uint_as_float(__ldg(&w5[1])), s = __uint_as_float(__ldg(&w5[2]));
        const float tx = __uint_as_float(__ldg(&w5[3])), ty = __uint_as_float(__ldg(&w5[4]));
        const DItem it = v.items[item];
        bool hit = false;
        for (uint32_t p = 0; p < it.n_ff_poles && !hit; p++) {
            const float4 pl = __ldg(&v.poles[it.pole_off + p]);
            hit = walk_group<Disk, PendT, G>(v, Disk{xform(Pt{pl.x, pl.y}, c, s, tx, ty), pl.z}, g);
        }
        for (uint32_t p = 0; p < it.n_piers && !hit; p++) {
            const float4 pr = __ldg(&v.piers[it.pier_off + p]);
            hit = walk_group<Seg, PendT, G>(v, Seg{xform(Pt{pr.x, pr.y}, c, s, tx, ty), xform(Pt{pr.z, pr.w}, c, s, tx, ty)},
                                            g);
        }
        if (g.lig == 0) {
            out[qi] = hit ? (uint8_t)1 : miss;
            if (n_pending && !hit && miss == PENDING) atomicAdd(n_pending, 1u);
        }
    }
}

// Per-warp table of the Partial leaves a query's bounding box reaches, each with its Partial,
// unfiltered hazards whose ff box meets that bounding box.  Every edge of the shape lies inside the
// shape's bounding box, and box_hits_seg rejects an edge whose box misses the rectangle first
// (rect.rs:301-345), so a hazard whose ff box misses the bounding box is missed by every edge:
// testing only the tabled hazards of a leaf gives the full leaf loop's answer.  A leaf that is not
// in the table (no room, or not reached by the box walk) falls back to the full loop.
// The table costs a walk and a scan of the reached leaves per query; it is built in the
// latency-bound regime of small batches (k_poly's `leaf_tab`), where it shortens the slowest
// queries' leaf loops.
// The table also keeps, per tabled hazard, the edges whose box meets the shape's box: an edge
// whose box misses the shape's box misses the box of every edge of the shape, and
// edge_intersection rejects on those boxes first (edge.rs:188-199), so the other edges cannot be hit.
#ifndef JCDE_LT_LEAVES
#define JCDE_LT_LEAVES 8
#endif
#ifndef JCDE_LT_ENTS
#define JCDE_LT_ENTS 64
#endif
#ifndef JCDE_LT_EDGES
#define JCDE_LT_EDGES 96
#endif
constexpr int LT_LEAVES = JCDE_LT_LEAVES, LT_ENTS = JCDE_LT_ENTS, LT_EDGES = JCDE_LT_EDGES;
struct LeafTab {
    float4 ff[LT_ENTS];
    uint2 ec[LT_ENTS];   // edge offset, edge count; offset | LT_LOCAL: into `edges` below
    int32_t node[LT_LEAVES];
    uint32_t start[LT_LEAVES + 1];
    uint32_t n_leaves;
    float4 edges[LT_EDGES];
};
constexpr uint32_t LT_LOCAL = 0x80000000u;

template <typename PendT>
__device__ __forceinline__ void build_leaf_tab(const View& v, int vr, const Box& sb, LeafTab* lt, int lane) {
    uint32_t nl = 0, ne = 0;
    const uint32_t below = (1u << lane) - 1u;
    WalkT<PendT> w{vr, 0, 0, (PendT)0};
    while (w.node >= 0) {
        if (__ldg(&v.strength[w.node]) == PRES_PARTIAL) {
            const DNode nd = ld_node(v, w.node);
            if (nd.child >= 0) {
                const Pt m = box_mid(nd.box);
                uint32_t msk = 0;
                JCDE_UNROLL
                for (int i = 0; i < 4; i++)
                    if (box_hits_box(quad_box(nd.box, m, i), sb)) msk |= 1u << i;
                if (msk) walk_push(w, msk, nd.child);
            } else if (nl < LT_LEAVES) {
                const uint32_t e0 = ne;
                bool fits = true;
                for (uint32_t b = 0; b < nd.hz_cnt; b += 32) {
                    const uint32_t k = b + lane;
                    bool c = false;
                    DEntry e{};
                    if (k < nd.hz_cnt) {
                        e = ld_entry(v, nd.hz_off + k);
                        c = e.presence == PRES_PARTIAL && box_hits_box(e.ff, sb) && !filtered(v, e.hkey);
                    }
                    const uint32_t bal = __ballot_sync(FULL, c);
                    if (ne + __popc(bal) > (uint32_t)LT_ENTS) {
                        fits = false;
                        break;
                    }
                    if (c) {
                        const uint32_t at = ne + __popc(bal & below);
                        lt->ff[at] = make_float4(e.ff.x0, e.ff.y0, e.ff.x1, e.ff.y1);
                        lt->ec[at] = make_uint2(e.edge_off, e.edge_cnt);
                    }
                    ne += __popc(bal);
                }
                if (fits) {
                    if (lane == 0) {
                        lt->node[nl] = w.node;
                        lt->start[nl] = e0;
                    }
                    nl++;
                } else {
                    ne = e0;
                }
            }
        }
        w.node = walk_next(v, w);
    }
    if (lane == 0) {
        lt->start[nl] = ne;
        lt->n_leaves = nl;
    }
    __syncwarp();
    uint32_t nx = 0;
    for (uint32_t k = 0; k < ne; k++) {
        const uint2 ec = lt->ec[k];
        const uint32_t x0 = nx;
        bool fits = true;
        for (uint32_t b = 0; b < ec.y; b += 32) {
            const uint32_t j = b + lane;
            bool keep = false;
            float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
            if (j < ec.y) {
                f = __ldg(&v.edges[ec.x + j]);
                keep = !(fmx(fmn(f.x, f.z), sb.x0) > fmn(fmx(f.x, f.z), sb.x1)) &&
                       !(fmx(fmn(f.y, f.w), sb.y0) > fmn(fmx(f.y, f.w), sb.y1));
            }
            const uint32_t bal = __ballot_sync(FULL, keep);
            if (nx + __popc(bal) > (uint32_t)LT_EDGES) {
                fits = false;
                break;
            }
            if (keep) lt->edges[nx + __popc(bal & below)] = f;
            nx += __popc(bal);
        }
        if (fits) {
            if (lane == 0) lt->ec[k] = make_uint2(x0 | LT_LOCAL, nx - x0);
        } else {
            nx = x0;   // this hazard keeps its full edge list
        }
    }
    __syncwarp();
}

template <class P>
__device__ __forceinline__ bool leaf_hits_tab(const View& v, const P& p, int node, const DNode& nd, const LeafTab* lt,
                                              volatile int* stop) {
    const uint32_t nl = lt->n_leaves;
    for (uint32_t t = 0; t < nl; t++) {
        if (lt->node[t] != node) continue;
        const uint32_t end = lt->start[t + 1];
        for (uint32_t k = lt->start[t]; k < end; k++) {
            if (*stop) return false;
            const float4 f = lt->ff[k];
            if (!p_hits_box(p, Box{f.x, f.y, f.z, f.w})) continue;   // qt_partial_hazard.rs:67-71
            const uint2 ec = lt->ec[k];
            if (ec.x & LT_LOCAL) {
                const float4* es = lt->edges + (ec.x & ~LT_LOCAL);
                for (uint32_t j = 0; j < ec.y; j++) {
                    const float4 f = es[j];
                    if (p_hits_seg(p, Seg{Pt{f.x, f.y}, Pt{f.z, f.w}})) {
                        *stop = 1;
                        return true;
                    }
                }
                continue;
            }
            for (uint32_t j = 0; j < ec.y; j++) {
                if (p_hits_seg(p, ld_edge(v, ec.x + j))) {
                    *stop = 1;
                    return true;
                }
                if ((j & 7) == 7 && *stop) return false;
            }
        }
        return false;
    }
    return leaf_hits(v, p, nd, stop);
}

// walk_step with the leaf test answered from the warp's leaf table.
template <class P, typename PendT>
__device__ __forceinline__ bool walk_step_tab(const View& v, const P& p, WalkT<PendT>& w, volatile int* stop,
                                              const LeafTab* lt) {
    const uint32_t st = __ldg(&v.strength[w.node]);
    if (st == PRES_ENTIRE) return true;
    if (st == PRES_PARTIAL) {
        DNode nd = ld_node(v, w.node);
        if (nd.child >= 0) {
            const uint32_t m = p_quad_mask(p, nd.box);
            if (m) walk_push(w, m, nd.child);
        } else if (lt ? leaf_hits_tab(v, p, w.node, nd, lt, stop) : leaf_hits(v, p, nd, stop)) {
            return true;
        }
    }
    w.node = walk_next(v, w);
    return false;
}

// Polygon pass — CDEngine::detect_poly_collision (cd_engine.rs:160-197), one warp per query.
// With `only_pending`, queries whose slot is not PENDING were decided by the surrogate pass and
// are skipped.  Writes JCDE_FREE / JCDE_COLLIDES.
#ifndef JCDE_POLY_MIN_BLOCKS
#define JCDE_POLY_MIN_BLOCKS 4   // 64 registers: four 256-thread blocks per SM
#endif
constexpr uint32_t POLY_MAXV = 256;   // items with more vertices transform edges on the fly
template <typename PendT, bool TAB, bool S = false>
__device__ __forceinline__ void poly_query(const View& v, const uint32_t* __restrict__ qw, uint32_t qi,
                                           uint8_t* __restrict__ out, const RawShape& raw, volatile int* stop,
                                           float2* tv, uint32_t* jobsw, LeafTab* ltab, int lane,
                                           unsigned long long* best = nullptr, bool skip = false) {
    QShape sh;
    Pt spoi;
    if (raw.verts) {
        sh = QShape{raw.verts, raw.nv, 1.0f, 0.0f, 0.0f, 0.0f, true};
        spoi = Pt{raw.poi_x, raw.poi_y};
    } else {
        QueryHead qh = load_query_words(qw, lane);
        if (qh.item >= v.n_items) {
            if (lane == 0) out[qi] = 2;
            return;
        }
        const DItem it = v.items[qh.item];
        sh = QShape{v.iverts + it.v_off, it.v_cnt, qh.c, qh.s, qh.tx, qh.ty, false};
        spoi = xform(Pt{it.poi_x, it.poi_y}, qh.c, qh.s, qh.tx, qh.ty);
    }
    if (lane == 0) *stop = 0;
    // the transformed vertices are kept in shared memory (items up to POLY_MAXV vertices)
    const bool cached = sh.nv <= POLY_MAXV;
    Box sb;
    {
        float x0 = FLT_MAX, y0 = FLT_MAX, x1 = -FLT_MAX, y1 = -FLT_MAX;
        for (uint32_t k = lane; k < sh.nv; k += 32) {
            const Pt p = sh.vtx(k);
            if (cached) tv[k] = make_float2(p.x, p.y);
            x0 = fminf(x0, p.x);
            y0 = fminf(y0, p.y);
            x1 = fmaxf(x1, p.x);
            y1 = fmaxf(y1, p.y);
        }
        JCDE_UNROLL
        for (int o = 16; o; o >>= 1) {
            x0 = fminf(x0, __shfl_xor_sync(FULL, x0, o));
            y0 = fminf(y0, __shfl_xor_sync(FULL, y0, o));
            x1 = fmaxf(x1, __shfl_xor_sync(FULL, x1, o));
            y1 = fmaxf(y1, __shfl_xor_sync(FULL, y1, o));
        }
        sb = Box{x0, y0, x1, y1};   // SPolygon::generate_bounding_box (simple_polygon.rs:122-133)
    }
    __syncwarp();
    // lbf's search tests a sample's polygon only if it could still beat the best free sample
    // (search.rs:52-56): with `skip`, a query whose (cost, index) exceeds the batch's best so far
    // is left unjudged (3); the best only falls, so no skipped query could have been the choice.
    unsigned long long skip_key = ~0ull;
    if (skip && best && !raw.verts) {
        skip_key = ((unsigned long long)orderable(sb.x1 * 10.0f + sb.y1) << 32) | qi;
        if (skip_key > *(volatile unsigned long long*)best) {
            if (lane == 0) out[qi] = 3;
            return;
        }
    }
    // the same test while the query is judged (before its leaf table, then every 4 iterations of the
    // edge loop, then before the containment scan): a query whose key falls behind a best found since
    // can no longer be the choice, so its judgment stops there (unjudged, 3)
    auto overtaken = [&]() -> bool {
        return skip_key != ~0ull && skip_key > *(volatile unsigned long long*)best;
    };
    auto edge_of = [&](uint32_t k) -> Seg {
        if (!cached) return sh.edge(k);
        const float2 a = tv[k], b = tv[k + 1 == sh.nv ? 0 : k + 1];
        return Seg{Pt{a.x, a.y}, Pt{b.x, b.y}};
    };
    // a shape not surrounded by the CDE box collides (cd_engine.rs:161-163)
    bool hit = !box_surrounds(v.cde, sb);
    const int vr = hit ? 0 : virtual_root_warp<S>(v, sb, lane);
    const uint32_t lt = (1u << lane) - 1u;
    // Every edge's walk starts with a visit of the virtual root.  When the root of the walk is a
    // Partial internal node, that first visit is done here for all edges at once (uniform work,
    // 32 edges per round): edges whose quadrant mask is empty are dropped and the others are
    // listed with their mask, so the walks below start one level down.
    uint32_t n_jobs = sh.nv;   // without the list, job k is edge k starting at the virtual root
    bool listed = false;
    int vr_child = -1;
    if (!hit) {
        const uint32_t st = strength_at<S>(v, vr);
        if (st == PRES_ENTIRE) {
            hit = true;
        } else if (st == PRES_NONE) {
            n_jobs = 0;   // nothing to hit below; containment still runs
        } else {
            const DNode vn = node_at<S>(v, vr);
            if (vn.child >= 0 && cached) {
                listed = true;
                vr_child = vn.child;
                uint32_t cnt = 0;
                for (uint32_t base = 0; base < sh.nv; base += 32) {
                    const uint32_t k = base + lane;
                    const uint32_t m = k < sh.nv ? seg_quadrant_mask(edge_of(k), vn.box) : 0u;
                    const uint32_t bal = __ballot_sync(FULL, m != 0);
                    if (m) jobsw[cnt + __popc(bal & lt)] = k | (m << 16);
                    cnt += __popc(bal);
                }
                n_jobs = cnt;
                __syncwarp();
            }
        }
    }
    const LeafTab* tab = nullptr;
    if constexpr (TAB) {
        if (!hit && n_jobs > 0 && overtaken()) {
            if (lane == 0) out[qi] = 3;
            return;
        }
        if (!hit && n_jobs > 0) {
            build_leaf_tab<PendT>(v, vr, sb, ltab, lane);
            tab = ltab;
        }
    }
    // Jobs are handed out dynamically: a lane whose walk is over takes the next unassigned job
    // (ballot rank), so no lane waits for the slowest walk of a fixed round.  Every loop
    // iteration is one node visit per active lane; a hit anywhere ends the query.
    uint32_t next = 0;
    WalkT<PendT> w{-1, 0, 0, (PendT)0};
    Seg e{};
    uint32_t iter = 0;
    while (!hit) {
        if (((++iter & 3) == 0) && overtaken()) {
            if (lane == 0) out[qi] = 3;
            return;
        }
        const bool want = w.node == -1;
        const uint32_t need = __ballot_sync(FULL, want);
        if (want) {
            const uint32_t p = next + __popc(need & lt);
            if (p < n_jobs) {
                if (listed) {
                    const uint32_t job = jobsw[p];
                    e = edge_of(job & 0xFFFFu);
                    w = WalkT<PendT>{-1, 1, vr_child, (PendT)(job >> 16)};
                    w.node = walk_next<PendT, S>(v, w);
                } else {
                    e = edge_of(p);
                    w = WalkT<PendT>{vr, 0, 0, (PendT)0};
                }
            } else {
                w.node = -2;
            }
        }
        next += __popc(need);
        const bool active = w.node >= 0;
        if (!__any_sync(FULL, active)) break;
#ifdef JCDE_POLY_STATS
        {
            const uint32_t na = __popc(__ballot_sync(FULL, active));
            if (lane == 0) {
                PSTAT(0, 1);
                PSTAT(1, na);
                if (na <= 8) PSTAT(2, 1);
            }
        }
#endif
        bool h = false;
        if (active) {
            if constexpr (TAB) h = walk_step_tab(v, e, w, stop, tab);
            else h = walk_step<Seg, PendT, S>(v, e, w, stop);
            if (!h && w.node < 0) w.node = -1;
        }
        hit = __any_sync(FULL, h);
    }
    if (lane == 0) {
        PSTAT(8, 1);
        PSTAT(9, hit ? 1 : 0);
        PSTAT(11, n_jobs);
    }
    if (!hit && overtaken()) {
        if (lane == 0) out[qi] = 3;
        return;
    }
    if (!hit) {
        // containment of the shape in (or of) the partially present hazards of the virtual root
        DNode vn = node_at<S>(v, vr);
        for (uint32_t base = 0; !hit && base < vn.hz_cnt; base += 32) {
            const uint32_t k = base + lane;
            int need = 0;
            bool res = false;
            uint32_t hk = 0;
            if (k < vn.hz_cnt) {
                DEntry en = ld_entry(v, vn.hz_off + k);
                // an Entire entry here is an ignored one (qt_node.rs:104), and is skipped
                if (en.presence == PRES_PARTIAL && !filtered(v, en.hkey)) {
                    hk = en.hkey;
                    const float4* hp = reinterpret_cast<const float4*>(v.haz + hk);
                    float4 a = __ldg(hp), b = __ldg(hp + 1);
                    int rel = box_almost_relation(Box{a.x, a.y, a.z, a.w}, sb);
                    if (rel == REL_SURROUNDING) need = 1;
                    else if (rel == REL_ENCLOSED) need = 2;
                    else res = (__float_as_uint(b.w) >> 31) != 0;   // not contained: exterior scope collides
                }
            }
            if (__any_sync(FULL, res)) {
                hit = true;
                break;
            }
            uint32_t todo = __ballot_sync(FULL, need != 0);
            while (todo && !hit) {
                const int src = __ffs(todo) - 1;
                todo &= todo - 1;
                const int nd = __shfl_sync(FULL, need, src);
                const uint32_t hkk = __shfl_sync(FULL, hk, src);
                if (lane == 0) PSTAT(10, 1);
                hit = warp_containment(v, sh, sb, spoi, hkk, nd, lane);
            }
        }
    }
    if (lane == 0) {
        out[qi] = hit ? 1 : 0;
        // the LBF choice of a free candidate (k_lbf_select's rule) while its box is at hand
        if (best && !hit && !raw.verts)
            atomicMin(best, ((unsigned long long)orderable(sb.x1 * 10.0f + sb.y1) << 32) | qi);
    }
}

template <typename PendT, bool MULTI, bool STAGE = false>
__global__ void __launch_bounds__(POLY_WARPS * 32, JCDE_POLY_MIN_BLOCKS)
    k_poly(View v, MultiSrc ms, const uint32_t* __restrict__ q, uint32_t n, uint8_t* __restrict__ out,
           RawShape raw, bool only_pending, const uint32_t* __restrict__ order, uint32_t* __restrict__ next,
           uint32_t chunk, const uint32_t* __restrict__ pend_rec = nullptr,
           const uint32_t* __restrict__ pend_count = nullptr) {
    __shared__ int stops[POLY_WARPS];
    __shared__ float2 tverts[POLY_WARPS][POLY_MAXV];   // transformed item vertices
    __shared__ uint32_t jobs[POLY_WARPS][POLY_MAXV];   // edge index | children mask below the virtual root << 16
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    volatile int* stop = &stops[warp];
    uint32_t* jobsw = jobs[warp];
    if constexpr (STAGE) {
        // the top levels of the tree (v.n_staged nodes, breadth-first) and their strengths under
        // this batch's filter, copied into dynamic shared memory once per block
        extern __shared__ float4 staged[];
        DNode* sn = reinterpret_cast<DNode*>(staged);
        uint8_t* ss = reinterpret_cast<uint8_t*>(sn + v.n_staged);
        for (uint32_t k = threadIdx.x; k < v.n_staged; k += blockDim.x) {
            sn[k] = ld_node(v, (int)k);
            ss[k] = __ldg(&v.strength[k]);
        }
        __syncthreads();
        v.snode = sn;
        v.sstr = ss;
    }
    const uint32_t stride = gridDim.x * POLY_WARPS;
    // with a pending list: its records, in the order the surrogate pass wrote them
    if (pend_rec) n = *(volatile const uint32_t*)pend_count;
    // queries in grid-stride order, or `chunk` consecutive ones at a time from the counter `next`
    uint32_t i = 0, end = 0, gs = blockIdx.x * POLY_WARPS + warp;
    for (;;) {
        if (i >= end) {
            if (next) {
                uint32_t t = 0;
                if (lane == 0) t = atomicAdd(next, chunk);
                i = __shfl_sync(FULL, t, 0);
                end = min(i + chunk, n);
            } else {
                i = gs;
                end = gs + 1;
                gs += stride;
            }
            if (i >= n) break;
        }
        if (pend_rec) {
            const uint32_t* r = pend_rec + (size_t)i * PEND_WORDS;
            i++;
            const uint32_t qi = __ldg(&r[0]);
            if constexpr (MULTI)
                poly_query<PendT, false>(ms.views[ms.layout_of(qi)], r + 1, qi, out, raw, stop, tverts[warp], jobsw,
                                         nullptr, lane);
            else
                poly_query<PendT, false, STAGE>(v, r + 1, qi, out, raw, stop, tverts[warp], jobsw, nullptr, lane);
            continue;
        }
        const uint32_t qi = order ? __ldg(&order[i]) : i;
        i++;
        if (only_pending && out[qi] != PENDING) continue;
        if constexpr (MULTI)
            poly_query<PendT, false>(ms.views[ms.layout_of(qi)], q + (size_t)qi * 5, qi, out, raw, stop, tverts[warp],
                                     jobsw, nullptr, lane);
        else
            poly_query<PendT, false, STAGE>(v, q + (size_t)qi * 5, qi, out, raw, stop, tverts[warp], jobsw, nullptr,
                                            lane);
    }
}

// The polygon pass of small batches (latency-bound): leaf tables in dynamic shared memory, queries
// one at a time from the counter `next`, and a register budget of its own (fewer, longer-lived warps).
// With `best`, every query found free also enters the LBF choice (as k_lbf_select would), and with
// `skip` the queries that can no longer win it are left unjudged (see poly_query).
#ifndef JCDE_POLY_TAB_MIN_BLOCKS
#define JCDE_POLY_TAB_MIN_BLOCKS 2
#endif
template <typename PendT>
__global__ void __launch_bounds__(POLY_WARPS * 32, JCDE_POLY_TAB_MIN_BLOCKS)
    k_poly_tab(View v, const uint32_t* __restrict__ q, uint32_t n, uint8_t* __restrict__ out, RawShape raw,
               bool only_pending, const uint32_t* __restrict__ order, uint32_t* __restrict__ next,
               unsigned long long* __restrict__ best, bool skip) {
    __shared__ int stops[POLY_WARPS];
    __shared__ float2 tverts[POLY_WARPS][POLY_MAXV];
    __shared__ uint32_t jobs[POLY_WARPS][POLY_MAXV];
    extern __shared__ LeafTab ltabs[];   // one per warp
    pdl_wait();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    volatile int* stop = &stops[warp];
    const uint32_t stride = gridDim.x * POLY_WARPS;
    for (uint32_t i = next ? 0u : blockIdx.x * POLY_WARPS + warp;; i += stride) {
        if (next) {
            uint32_t t = 0;
            if (lane == 0) t = atomicAdd(next, 1u);
            i = __shfl_sync(FULL, t, 0);
        }
        if (i >= n) break;
        const uint32_t qi = order ? __ldg(&order[i]) : i;
        if (only_pending && out[qi] != PENDING) continue;
        poly_query<PendT, true>(v, q + (size_t)qi * 5, qi, out, raw, stop, tverts[warp], jobs[warp], &ltabs[warp], lane,
                                best, skip);
    }
}

constexpr int COLLECT_WARPS = 4;
#ifndef JCDE_COLLECT_MIN_BLOCKS
#define JCDE_COLLECT_MIN_BLOCKS 6   // blocks per SM the collect pass is compiled for (0: ptxas decides)
#endif
#if JCDE_COLLECT_MIN_BLOCKS > 0
#define JCDE_COLLECT_BOUNDS __launch_bounds__(COLLECT_WARPS * 32, JCDE_COLLECT_MIN_BLOCKS)
#else
#define JCDE_COLLECT_BOUNDS __launch_bounds__(COLLECT_WARPS * 32)
#endif

// Collect: sorted colliding hazard keys per query, compacted with one atomicAdd per query.
// Dynamic shared memory: COLLECT_WARPS bitsets of `words` words, then per warp the item's
// transformed vertices (POLY_MAXV float2).  (Listing the virtual root's first visit for all edges
// at once, as the detect pass does, made this pass 30% slower: measured and left out.)
template <int MODE, typename PendT>
__global__ void JCDE_COLLECT_BOUNDS k_collect(View v, const uint32_t* __restrict__ q, uint32_t n,
                                                                uint32_t words, uint32_t* __restrict__ offsets,
                                                                uint32_t* __restrict__ counts, uint32_t* __restrict__ ids,
                                                                uint32_t cap, uint32_t* __restrict__ total, RawShape raw,
                                                                const uint32_t* __restrict__ order,
                                                                uint32_t* __restrict__ next) {
    extern __shared__ uint32_t smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t* bits = smem + (size_t)warp * words;
    float2* tv = reinterpret_cast<float2*>(smem + (size_t)COLLECT_WARPS * words) + (size_t)warp * POLY_MAXV;
    const uint32_t stride = gridDim.x * COLLECT_WARPS;
    // queries in grid-stride order, or two at a time from the counter `next`
    uint32_t i = 0, end = 0, gs = blockIdx.x * COLLECT_WARPS + warp;
    for (;;) {
        if (i >= end) {
            if (next) {
                uint32_t t = 0;
                if (lane == 0) t = atomicAdd(next, 2u);
                i = __shfl_sync(FULL, t, 0);
                end = min(i + 2u, n);
            } else {
                i = gs;
                end = gs + 1;
                gs += stride;
            }
            if (i >= n) break;
        }
        const uint32_t qi = order ? __ldg(&order[i]) : i;
        i++;
        QShape sh;
        DItem it{};
        Pt spoi;
        bool valid = true;
        if (raw.verts) {
            sh = QShape{raw.verts, raw.nv, 1.0f, 0.0f, 0.0f, 0.0f, true};
            spoi = Pt{raw.poi_x, raw.poi_y};
        } else {
            QueryHead qh = load_query(q, qi, lane);
            valid = qh.item < v.n_items;
            if (valid) {
                it = v.items[qh.item];
                sh = QShape{v.iverts + it.v_off, it.v_cnt, qh.c, qh.s, qh.tx, qh.ty, false};
                spoi = xform(Pt{it.poi_x, it.poi_y}, qh.c, qh.s, qh.tx, qh.ty);
            } else {
                sh = QShape{v.iverts, 0, 1.0f, 0.0f, 0.0f, 0.0f, true};
                spoi = Pt{0, 0};
            }
        }
        // the ignored keys are pre-seeded into the collector (hazards/filter.rs:69-76)
        for (uint32_t w = lane; w < words; w += 32) bits[w] = v.mask ? __ldg(&v.mask[w]) : 0u;
        // the transformed vertices (kept for items up to POLY_MAXV vertices) and the shape's bbox
        // (SPolygon::generate_bounding_box, simple_polygon.rs:122-133)
        const bool cached = (MODE & MODE_POLY) && valid && sh.nv <= POLY_MAXV;
        Box sb{0, 0, 0, 0};
        if ((MODE & MODE_POLY) && valid) {
            float x0 = FLT_MAX, y0 = FLT_MAX, x1 = -FLT_MAX, y1 = -FLT_MAX;
            for (uint32_t k = lane; k < sh.nv; k += 32) {
                const Pt p = sh.vtx(k);
                if (cached) tv[k] = make_float2(p.x, p.y);
                x0 = fminf(x0, p.x);
                y0 = fminf(y0, p.y);
                x1 = fmaxf(x1, p.x);
                y1 = fmaxf(y1, p.y);
            }
            JCDE_UNROLL
            for (int o = 16; o; o >>= 1) {
                x0 = fminf(x0, __shfl_xor_sync(FULL, x0, o));
                y0 = fminf(y0, __shfl_xor_sync(FULL, y0, o));
                x1 = fmaxf(x1, __shfl_xor_sync(FULL, x1, o));
                y1 = fmaxf(y1, __shfl_xor_sync(FULL, y1, o));
            }
            sb = Box{x0, y0, x1, y1};
        }
        __syncwarp();
        auto edge_of = [&](uint32_t k) -> Seg {
            if (!cached) return sh.edge(k);
            const float2 a = tv[k], b = tv[k + 1 == sh.nv ? 0 : k + 1];
            return Seg{Pt{a.x, a.y}, Pt{b.x, b.y}};
        };
        if (valid) {
            int vr = 0;
            if (MODE & MODE_POLY) {
                if (!box_surrounds(v.cde, sb) && v.exterior >= 0 && lane == 0) bit_set(bits, (uint32_t)v.exterior);
                vr = virtual_root_warp(v, sb, lane);
            }
            const uint32_t n_pole = (MODE & MODE_SURROGATE) ? it.n_ff_poles : 0u;
            const uint32_t n_pier = (MODE & MODE_SURROGATE) ? it.n_piers : 0u;
            const uint32_t n_sp = n_pole + n_pier;
            const uint32_t n_edge = (MODE & MODE_POLY) ? sh.nv : 0u;
            const uint32_t np = n_sp + n_edge;
            for (uint32_t p = lane; p < np; p += 32) {   // lane l walks probes l, l+32, ...
                if (p < n_pole) {
                    const float4 pl = __ldg(&v.poles[it.pole_off + p]);
                    collect_walk<Disk, PendT>(v, Disk{xform(Pt{pl.x, pl.y}, sh.c, sh.s, sh.tx, sh.ty), pl.z}, 0, bits);
                } else if (p < n_sp) {
                    const float4 pr = __ldg(&v.piers[it.pier_off + (p - n_pole)]);
                    collect_walk<Seg, PendT>(v, Seg{xform(Pt{pr.x, pr.y}, sh.c, sh.s, sh.tx, sh.ty),
                                                    xform(Pt{pr.z, pr.w}, sh.c, sh.s, sh.tx, sh.ty)}, 0, bits);
                } else {
                    collect_walk<Seg, PendT>(v, edge_of(p - n_sp), vr, bits);
                }
            }
            __syncwarp();
            if (MODE & MODE_POLY) {
                DNode vn = ld_node(v, vr);
                for (uint32_t base = 0; base < vn.hz_cnt; base += 32) {
                    const uint32_t k = base + lane;
                    int need = 0;
                    uint32_t hk = 0;
                    if (k < vn.hz_cnt) {
                        DEntry e = ld_entry(v, vn.hz_off + k);
                        if (e.presence == PRES_PARTIAL && !bit_get(bits, e.hkey)) {
                            hk = e.hkey;
                            const float4* hp = reinterpret_cast<const float4*>(v.haz + hk);
                            float4 a = __ldg(hp), b = __ldg(hp + 1);
                            int rel = box_almost_relation(Box{a.x, a.y, a.z, a.w}, sb);
                            if (rel == REL_SURROUNDING) need = 1;
                            else if (rel == REL_ENCLOSED) need = 2;
                            else if ((__float_as_uint(b.w) >> 31) != 0) bit_set(bits, hk);
                        }
                    }
                    uint32_t todo = __ballot_sync(FULL, need != 0);
                    while (todo) {
                        const int src = __ffs(todo) - 1;
                        todo &= todo - 1;
                        const int nd = __shfl_sync(FULL, need, src);
                        const uint32_t hkk = __shfl_sync(FULL, hk, src);
                        if (warp_containment(v, sh, sb, spoi, hkk, nd, lane) && lane == 0) bit_set(bits, hkk);
                    }
                }
            }
        }
        __syncwarp();
        // emit keys in ascending order: bits minus the pre-seeded ignored keys
        uint32_t cnt = 0;
        for (uint32_t w = lane; w < words; w += 32) cnt += __popc(bits[w] & ~(v.mask ? __ldg(&v.mask[w]) : 0u));
#pragma unroll
        for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(FULL, cnt, o);
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(total, cnt);
        base = __shfl_sync(FULL, base, 0);
        if (lane == 0) {
            offsets[qi] = base;
            counts[qi] = valid ? cnt : 0xffffffffu;
        }
        if ((uint64_t)base + cnt <= cap) {
            uint32_t run = base;
            for (uint32_t w0 = 0; w0 < words; w0 += 32) {
                const uint32_t w = w0 + lane;
                uint32_t m = w < words ? (bits[w] & ~(v.mask ? __ldg(&v.mask[w]) : 0u)) : 0u;
                uint32_t c = __popc(m), incl = c;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    uint32_t t = __shfl_up_sync(FULL, incl, o);
                    if (lane >= o) incl += t;
                }
                uint32_t pos = run + incl - c;
                while (m) {
                    int b = __ffs(m) - 1;
                    m &= m - 1;
                    ids[pos++] = w * 32 + b;
                }
                run += __shfl_sync(FULL, incl, 31);
            }
        }
        __syncwarp();
    }
}

// Spatial ordering of a batch: queries are counted into a BUCKET_GRID x BUCKET_GRID grid over the
// CDE box by translation (Morton order of the cells), and the passes visit them cell by cell, so
// the threads of a warp walk neighbouring parts of the quadtree.  Only the visiting order changes;
// every query still writes its own verdict slot.
constexpr uint32_t BUCKET_BITS = 6;
constexpr uint32_t BUCKET_GRID = 1u << BUCKET_BITS;
constexpr uint32_t N_BUCKETS = BUCKET_GRID * BUCKET_GRID;

__device__ __forceinline__ uint32_t spread_bits(uint32_t x) {   // up to 8 bits -> even positions
    x &= 0xFFu;
    x = (x | (x << 4)) & 0x0F0Fu;
    x = (x | (x << 2)) & 0x3333u;
    x = (x | (x << 1)) & 0x5555u;
    return x;
}
__device__ __forceinline__ uint32_t bucket_of(const uint32_t* __restrict__ q, uint32_t qi, const Box& b) {
    const float tx = __uint_as_float(__ldg(&q[(size_t)qi * 5 + 3]));
    const float ty = __uint_as_float(__ldg(&q[(size_t)qi * 5 + 4]));
    const float g = (float)BUCKET_GRID;
    const float fx = fmaxf(0.0f, fminf((tx - b.x0) / (b.x1 - b.x0) * g, g - 1.0f));
    const float fy = fmaxf(0.0f, fminf((ty - b.y0) / (b.y1 - b.y0) * g, g - 1.0f));
    return spread_bits((uint32_t)fx) | (spread_bits((uint32_t)fy) << 1);
}
// The same ordering in two kernels with the histogram in shared memory: one atomic per query to
// shared memory and one per non-empty cell and block to global memory (global atomics on 4,096
// counters were most of the three-kernel version's time).  ORDER_BITS bits per axis.
#ifndef JCDE_ORDER_BITS
#define JCDE_ORDER_BITS 6
#endif
constexpr uint32_t ORDER_BITS = JCDE_ORDER_BITS;
constexpr uint32_t ORDER_CELLS = 1u << (2 * ORDER_BITS);
constexpr uint32_t ORDER_HIST_WORDS = ORDER_CELLS + 32;   // the cells' counts, then the blocks-done counter
constexpr uint32_t ORDER_THREADS = 1024;
constexpr uint32_t ORDER_PER_THREAD = 8;                  // queries per thread and tile of the scatter
constexpr uint32_t ORDER_TILE = ORDER_THREADS * ORDER_PER_THREAD;
constexpr size_t ORDER_SMEM = ORDER_CELLS * 4;             // the block's histogram (dynamic shared memory)
static_assert(ORDER_BITS <= 7, "the scan takes up to 16 cells per thread");

__device__ __forceinline__ uint32_t order_cell(const uint32_t* __restrict__ q, uint32_t qi, const Box& b) {
    const float tx = __uint_as_float(__ldg(&q[(size_t)qi * 5 + 3]));
    const float ty = __uint_as_float(__ldg(&q[(size_t)qi * 5 + 4]));
    const float g = (float)(1u << ORDER_BITS);
    const float fx = fmaxf(0.0f, fminf((tx - b.x0) / (b.x1 - b.x0) * g, g - 1.0f));
    const float fy = fmaxf(0.0f, fminf((ty - b.y0) / (b.y1 - b.y0) * g, g - 1.0f));
    return spread_bits((uint32_t)fx) | (spread_bits((uint32_t)fy) << 1);
}

// Counts per cell (hist, zeroed by the caller, ORDER_HIST_WORDS words); the last block to finish
// turns them into exclusive offsets and clears the blocks-done counter.
__global__ void __launch_bounds__(ORDER_THREADS) k_order_count(const uint32_t* __restrict__ q, uint32_t n, Box b,
                                                               uint32_t* __restrict__ hist) {
    extern __shared__ uint32_t h[];   // ORDER_CELLS
    __shared__ uint32_t warp_sums[32];
    __shared__ bool is_last;
    const uint32_t t = threadIdx.x;
    for (uint32_t k = t; k < ORDER_CELLS; k += ORDER_THREADS) h[k] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * ORDER_THREADS + t; i < n; i += gridDim.x * ORDER_THREADS)
        atomicAdd(&h[order_cell(q, i, b)], 1u);
    __syncthreads();
    for (uint32_t k = t; k < ORDER_CELLS; k += ORDER_THREADS)
        if (h[k]) atomicAdd(&hist[k], h[k]);
    __threadfence();
    __syncthreads();
    if (t == 0) is_last = atomicAdd(&hist[ORDER_CELLS], 1u) == gridDim.x - 1;
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    // exclusive scan of consecutive cells per thread (the counts are read from L2)
    constexpr uint32_t PER = (ORDER_CELLS + ORDER_THREADS - 1) / ORDER_THREADS;
    const uint32_t lane = t & 31, warp = t >> 5;
    uint32_t c[PER], s = 0;
    JCDE_UNROLL
    for (uint32_t k = 0; k < PER; k++) {
        const uint32_t j = t * PER + k;
        c[k] = j < ORDER_CELLS ? __ldcg(&hist[j]) : 0u;
        s += c[k];
    }
    uint32_t incl = s;
    JCDE_UNROLL
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = warp_sums[lane];
        uint32_t wi = w;
        JCDE_UNROLL
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, wi, o);
            if (lane >= (uint32_t)o) wi += y;
        }
        warp_sums[lane] = wi - w;
    }
    __syncthreads();
    uint32_t run = warp_sums[warp] + incl - s;
    JCDE_UNROLL
    for (uint32_t k = 0; k < PER; k++) {
        const uint32_t j = t * PER + k;
        if (j < ORDER_CELLS) hist[j] = run;
        run += c[k];
    }
    if (t == 0) hist[ORDER_CELLS] = 0u;
}

// Places every query at its cell's offset: per tile of ORDER_TILE queries the block ranks them in
// shared memory, reserves one range per non-empty cell from the global offsets, then writes.
__global__ void __launch_bounds__(ORDER_THREADS) k_order_scatter(const uint32_t* __restrict__ q, uint32_t n, Box b,
                                                                 uint32_t* __restrict__ offs,
                                                                 uint32_t* __restrict__ order) {
    extern __shared__ uint32_t h[];   // ORDER_CELLS
    const uint32_t t = threadIdx.x;
    for (uint32_t tile = blockIdx.x; (size_t)tile * ORDER_TILE < n; tile += gridDim.x) {
        for (uint32_t k = t; k < ORDER_CELLS; k += ORDER_THREADS) h[k] = 0;
        __syncthreads();
        const uint32_t i0 = tile * ORDER_TILE + t;
        uint32_t cell[ORDER_PER_THREAD], rank[ORDER_PER_THREAD];
        JCDE_UNROLL
        for (uint32_t j = 0; j < ORDER_PER_THREAD; j++) {
            const uint32_t i = i0 + j * ORDER_THREADS;
            cell[j] = i < n ? order_cell(q, i, b) : 0u;
            rank[j] = i < n ? atomicAdd(&h[cell[j]], 1u) : 0u;
        }
        __syncthreads();
        for (uint32_t k = t; k < ORDER_CELLS; k += ORDER_THREADS) {
            const uint32_t c = h[k];
            if (c) h[k] = atomicAdd(&offs[k], c);
        }
        __syncthreads();
        JCDE_UNROLL
        for (uint32_t j = 0; j < ORDER_PER_THREAD; j++) {
            const uint32_t i = i0 + j * ORDER_THREADS;
            if (i < n) order[h[cell[j]] + rank[j]] = i;
        }
        __syncthreads();
    }
}

// Several layouts in one batch: the bucket key is (layout, Morton cell of the layout's CDE box).
__global__ void k_mbucket_count(const uint32_t* __restrict__ q, uint32_t n, MultiSrc ms, uint32_t* __restrict__ hist) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t l = ms.layout_of(i);
        atomicAdd(&hist[l * N_BUCKETS + bucket_of(q, i, ms.views[l].cde)], 1u);
    }
}
__global__ void k_mbucket_scatter(const uint32_t* __restrict__ q, uint32_t n, MultiSrc ms, uint32_t* __restrict__ offs,
                                  uint32_t* __restrict__ order) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t l = ms.layout_of(i);
        order[atomicAdd(&offs[l * N_BUCKETS + bucket_of(q, i, ms.views[l].cde)], 1u)] = i;
    }
}
// exclusive scan of `total` counts in place, one block of 1024 threads, a contiguous run per thread
__global__ void __launch_bounds__(1024) k_scan_counts(uint32_t* __restrict__ c, uint32_t total) {
    __shared__ uint32_t warp_sums[32];
    const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t per = (total + 1023) / 1024, a = min(total, t * per), b = min(total, a + per);
    uint32_t s = 0;
    for (uint32_t k = a; k < b; k++) s += c[k];
    uint32_t incl = s;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(FULL, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_sums[lane], wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(FULL, wi, o);
            if (lane >= (uint32_t)o) wi += y;
        }
        warp_sums[lane] = wi - w;
    }
    __syncthreads();
    uint32_t run = warp_sums[warp] + incl - s;
    for (uint32_t k = a; k < b; k++) {
        const uint32_t v = c[k];
        c[k] = run;
        run += v;
    }
}

// ---------------------------------------------------------------------------------------------
// Differentiable pole-overlap proxy (no counterpart in the reference).  For a candidate placement
// (theta, tx, ty) of an item, with the item's surrogate poles p_i (circle.rs:95-107 as circles,
// sp_surrogate.rs:19) placed at c_i = R(theta) p_i + t and the hazards' poles (c_j, r_j):
//     P = sum_ij max(0, r_i + r_j - |c_i - c_j|)^2
//     dP/dt = sum -2 pen_ij (c_i - c_j) / |c_i - c_j|
//     dP/dtheta = sum -2 pen_ij (c_i - c_j) . R'(theta) p_i / |c_i - c_j|,  R'(theta) p = (-ry, rx)
// with (rx, ry) = R(theta) p.  Differences are formed as (t - c_j) + R p to keep float32 precision.
// One warp per candidate, lanes over the item's poles, FP32 accumulation, warp-reduced.
// ---------------------------------------------------------------------------------------------
struct ProxyOut {
    float p, gx, gy, gth;
};

// Neumaier-compensated float32 accumulation (sum + running correction)
struct KSum {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        const float t = s + x;
        c += fabsf(s) >= fabsf(x) ? (s - t) + x : (x - t) + s;
        s = t;
    }
    __device__ __forceinline__ float get() const { return s + c; }
};

__device__ __forceinline__ int pole_cell(float x, float o, float inv, int g) {
    return max(0, min(g - 1, (int)floorf((x - o) * inv)));
}

// `lane` counts within a group of `nsub` lanes (32 or 16) whose member mask is `mask`; hazard pole
// radii are grown by `clear` (0 for the proxy itself).
__device__ __forceinline__ ProxyOut proxy_eval(const View& v, const DItem& it, float c, float s, float tx, float ty,
                                               int lane, int nsub, uint32_t mask, float clear) {
    KSum p, gx, gy, gth;
    const int g = v.hp_g;
    for (uint32_t k = lane; k < it.n_poles; k += nsub) {
        const float4 pl = __ldg(&v.poles[it.pole_off + k]);
        const float rx = c * pl.x - s * pl.y, ry = s * pl.x + c * pl.y;
        const float cx = rx + tx, cy = ry + ty;
        const float rc = pl.z + clear;   // reach: a hazard pole's box grown by `clear` must overlap this one
        const float bx0 = cx - rc, by0 = cy - rc, bx1 = cx + rc, by1 = cy + rc;
        const int ix0 = pole_cell(bx0, v.hp_x0, v.hp_inv_cs, g), ix1 = pole_cell(bx1, v.hp_x0, v.hp_inv_cs, g);
        const int iy0 = pole_cell(by0, v.hp_y0, v.hp_inv_cs, g), iy1 = pole_cell(by1, v.hp_y0, v.hp_inv_cs, g);
        for (int iy = iy0; iy <= iy1; iy++)
            for (int ix = ix0; ix <= ix1; ix++) {
                const uint32_t cell = (uint32_t)iy * (uint32_t)g + (uint32_t)ix;
                const uint32_t a = __ldg(&v.hp_start[cell]), b = __ldg(&v.hp_start[cell + 1]);
                for (uint32_t j = a; j < b; j++) {
                    const float4 h = __ldg(&v.hpoles[j]);
                    // the pair belongs to the cell of the low corner of the two boxes' overlap
                    const float mx = fmaxf(bx0, h.x - h.z), my = fmaxf(by0, h.y - h.z);
                    if (mx > fminf(bx1, h.x + h.z) || my > fminf(by1, h.y + h.z)) continue;
                    // (the item box carries the clearance, so every grown overlap is still found, and
                    // the low corner lies in a cell both boxes reach: each pair is counted once)
                    if (pole_cell(mx, v.hp_x0, v.hp_inv_cs, g) != ix || pole_cell(my, v.hp_y0, v.hp_inv_cs, g) != iy)
                        continue;
                    if (filtered(v, __float_as_uint(h.w))) continue;
                    const float dx = (tx - h.x) + rx, dy = (ty - h.y) + ry;
                    const float d2 = dx * dx + dy * dy;
                    const float rr = pl.z + h.z + clear;
                    if (d2 >= rr * rr) continue;
                    const float d = sqrtf(d2), pen = rr - d;
                    p.add(pen * pen);
                    if (d > 0.0f) {
                        const float f = -2.0f * pen / d;
                        gx.add(f * dx);
                        gy.add(f * dy);
                        gth.add(f * (dy * rx - dx * ry));
                    }
                }
            }
    }
    ProxyOut o{p.get(), gx.get(), gy.get(), gth.get()};
    for (int sh = nsub >> 1; sh; sh >>= 1) {
        o.p += __shfl_xor_sync(mask, o.p, sh);
        o.gx += __shfl_xor_sync(mask, o.gx, sh);
        o.gy += __shfl_xor_sync(mask, o.gy, sh);
        o.gth += __shfl_xor_sync(mask, o.gth, sh);
    }
    return o;
}

// ---------------------------------------------------------------------------------------------
// Float-float ("double-single") arithmetic for the proxy's forward / adjoint: a value is hi + lo
// with |lo| <= ulp(hi) / 2, about 48 significant bits.  Built from the error-free transforms
// TwoSum (Knuth) and FMA-based TwoProduct (Dekker 1971; Ogita, Rump and Oishi 2005).  The file is
// compiled with -fmad=false, so only the explicit __fmaf_rn below is fused.
//
// Why: the penetration depth r_i + r_j - |c_i - c_j| of a shallow contact cancels most of its
// digits (coordinates ~2000, depths ~0.01-1), so a plain float32 depth carries a relative error
// of up to ~1e-3; float-float keeps it near 1e-10 and the gradient then agrees with a float64
// evaluation of the same float32 inputs to far better than 1e-4.
// ---------------------------------------------------------------------------------------------
struct FF {
    float hi, lo;
};
__device__ __forceinline__ FF ff_two_sum(float a, float b) {
    const float s = a + b, bb = s - a;
    return FF{s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ FF ff_fast_sum(float a, float b) {   // |a| >= |b|
    const float s = a + b;
    return FF{s, b - (s - a)};
}
__device__ __forceinline__ FF ff_two_prod(float a, float b) {
    const float p = a * b;
    return FF{p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
    FF s = ff_two_sum(a.hi, b.hi);
    const FF t = ff_two_sum(a.lo, b.lo);
    s = ff_fast_sum(s.hi, s.lo + t.hi);
    return ff_fast_sum(s.hi, s.lo + t.lo);
}
__device__ __forceinline__ FF ff_neg(FF a) { return FF{-a.hi, -a.lo}; }
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
    const FF p = ff_two_prod(a.hi, b.hi);
    return ff_fast_sum(p.hi, p.lo + (a.hi * b.lo + a.lo * b.hi));
}
__device__ __forceinline__ FF ff_mul_f(FF a, float b) {
    const FF p = ff_two_prod(a.hi, b);
    return ff_fast_sum(p.hi, p.lo + a.lo * b);
}
// square root of a > 0: one Newton correction of the float32 root
__device__ __forceinline__ FF ff_sqrt(FF a) {
    const float x = sqrtf(a.hi);
    const FF r = ff_add(a, ff_neg(ff_two_prod(x, x)));
    return ff_fast_sum(x, r.hi / (2.0f * x));
}
// a / b: quotient digits by long division (three float32 partial quotients)
__device__ __forceinline__ FF ff_div(FF a, FF b) {
    const float q1 = a.hi / b.hi;
    FF r = ff_add(a, ff_neg(ff_mul_f(b, q1)));
    const float q2 = r.hi / b.hi;
    r = ff_add(r, ff_neg(ff_mul_f(b, q2)));
    const float q3 = r.hi / b.hi;
    return ff_add(ff_fast_sum(q1, q2), FF{q3, 0.0f});
}
__device__ __forceinline__ float ff_f(FF a) { return a.hi + a.lo; }

// cos and sin of a float32 angle in float-float: Cody-Waite reduction by pi/2 (split into three
// float32 parts, the first with 8 significant bits so that k * part is exact for |k| < 2^16, the
// other two products taken exactly by TwoProduct), then the Taylor series of sin and cos of the
// reduced argument (|r| <= ~pi/4 + rounding) in Horner form, to the term where it stops changing
// float-float digits (sin to r^17, cos to r^18).  Coefficients are 1/n! split into hi + lo.
__constant__ float c_inv_fact[19][2] = {
    {0x1p+0f, 0.0f}, {0x1p+0f, 0.0f}, {0x1p-1f, 0.0f},
    {0x1.555556p-3f, -0x1.555556p-28f}, {0x1.555556p-5f, -0x1.555556p-30f},
    {0x1.111112p-7f, -0x1.ddddde0p-32f}, {0x1.6c16c2p-10f, -0x1.27d27ep-35f},
    {0x1.a01a02p-13f, -0x1.7f97fap-39f}, {0x1.a01a02p-16f, -0x1.7f97fap-42f},
    {0x1.71de3ap-19f, 0x1.55b1ccp-45f}, {0x1.27e4fcp-22f, -0x1.10ec14p-47f},
    {0x1.ae6456p-26f, 0x1.fd5138p-52f}, {0x1.1eed8ep-29f, 0x1.ff1b12p-54f},
    {0x1.612462p-33f, -0x1.8af25ep-58f}, {0x1.93974ap-37f, 0x1.180f94p-62f},
    {0x1.ae7f3ep-41f, 0x1.ccee08p-67f}, {0x1.ae7f3ep-45f, 0x1.ccee08p-71f},
    {0x1.952c78p-49f, -0x1.f9ea56p-74f}, {0x1.682786p-53f, 0x1.dcbeccp-80f}};

__device__ __forceinline__ void ff_sincos(float theta, FF& s_out, FF& c_out) {
    const float P1 = 0x1.92p+0f, P2 = 0x1.fb5444p-12f, P3 = 0x1.68c234p-39f;   // pi/2 = P1 + P2 + P3 + O(1e-19)
    const float k = rintf(theta * 0x1.45f306p-1f);                               // theta * 2/pi
    FF r = ff_two_sum(theta, -(k * P1));
    r = ff_add(r, ff_neg(ff_two_prod(k, P2)));
    r = ff_add(r, ff_neg(ff_two_prod(k, P3)));
    const FF r2 = ff_mul(r, r);
    // sin r = r (1 - r^2/3! + r^4/5! - ...), cos r = 1 - r^2/2! + r^4/4! - ...
    FF ps = FF{c_inv_fact[17][0], c_inv_fact[17][1]};
    for (int n = 15; n >= 1; n -= 2) {
        ps = ff_add(FF{c_inv_fact[n][0], c_inv_fact[n][1]}, ff_neg(ff_mul(ps, r2)));
    }
    FF pc = FF{c_inv_fact[18][0], c_inv_fact[18][1]};
    for (int n = 16; n >= 0; n -= 2) {
        pc = ff_add(FF{c_inv_fact[n][0], c_inv_fact[n][1]}, ff_neg(ff_mul(pc, r2)));
    }
    const FF sr = ff_mul(ps, r), cr = pc;
    const int q = ((int)k) & 3;
    s_out = q == 0 ? sr : q == 1 ? cr : q == 2 ? ff_neg(sr) : ff_neg(cr);
    c_out = q == 0 ? cr : q == 1 ? ff_neg(sr) : q == 2 ? ff_neg(cr) : sr;
}

// The proxy and its adjoint for one candidate, every contact pair in float-float.  Pairs are first
// screened in float32 with a margin far above float32's rounding of the distance (so no contact is
// lost), then the depth and the gradient terms are formed and summed in float-float.
__device__ __forceinline__ ProxyOut proxy_eval_ff(const View& v, const DItem& it, FF c, FF s, float tx, float ty,
                                                  int lane) {
    FF p{0.0f, 0.0f}, gx{0.0f, 0.0f}, gy{0.0f, 0.0f}, gth{0.0f, 0.0f};
    const int g = v.hp_g;
    const float cf = ff_f(c), sf = ff_f(s);
    for (uint32_t k = lane; k < it.n_poles; k += 32) {
        const float4 pl = __ldg(&v.poles[it.pole_off + k]);
        const float rxf = cf * pl.x - sf * pl.y, ryf = sf * pl.x + cf * pl.y;
        const FF rx = ff_add(ff_mul_f(c, pl.x), ff_neg(ff_mul_f(s, pl.y)));
        const FF ry = ff_add(ff_mul_f(s, pl.x), ff_mul_f(c, pl.y));
        const float cx = rxf + tx, cy = ryf + ty;
        const float reach = pl.z * 1.00001f + 1e-3f;   // the pole's box, grown by the screening margin
        const float bx0 = cx - reach, by0 = cy - reach, bx1 = cx + reach, by1 = cy + reach;
        const int ix0 = pole_cell(bx0, v.hp_x0, v.hp_inv_cs, g), ix1 = pole_cell(bx1, v.hp_x0, v.hp_inv_cs, g);
        const int iy0 = pole_cell(by0, v.hp_y0, v.hp_inv_cs, g), iy1 = pole_cell(by1, v.hp_y0, v.hp_inv_cs, g);
        for (int iy = iy0; iy <= iy1; iy++)
            for (int ix = ix0; ix <= ix1; ix++) {
                const uint32_t cell = (uint32_t)iy * (uint32_t)g + (uint32_t)ix;
                const uint32_t a = __ldg(&v.hp_start[cell]), b = __ldg(&v.hp_start[cell + 1]);
                for (uint32_t j = a; j < b; j++) {
                    const float4 h = __ldg(&v.hpoles[j]);
                    // each pair once: in the cell of the low corner of the two boxes' overlap
                    const float mx = fmaxf(bx0, h.x - h.z), my = fmaxf(by0, h.y - h.z);
                    if (mx > fminf(bx1, h.x + h.z) || my > fminf(by1, h.y + h.z)) continue;
                    if (pole_cell(mx, v.hp_x0, v.hp_inv_cs, g) != ix || pole_cell(my, v.hp_y0, v.hp_inv_cs, g) != iy)
                        continue;
                    if (filtered(v, __float_as_uint(h.w))) continue;
                    const float dxf = (tx - h.x) + rxf, dyf = (ty - h.y) + ryf;
                    const float rm = (pl.z + h.z) * 1.00001f + 1e-3f;
                    if (dxf * dxf + dyf * dyf >= rm * rm) continue;
                    const FF dx = ff_add(ff_two_sum(tx, -h.x), rx), dy = ff_add(ff_two_sum(ty, -h.y), ry);
                    const FF d2 = ff_add(ff_mul(dx, dx), ff_mul(dy, dy));
                    const FF rr = ff_two_sum(pl.z, h.z);
                    if (d2.hi <= 0.0f) {   // coincident centres: depth rr, no direction
                        p = ff_add(p, ff_mul(rr, rr));
                        continue;
                    }
                    const FF d = ff_sqrt(d2);
                    const FF pen = ff_add(rr, ff_neg(d));
                    if (pen.hi <= 0.0f) continue;
                    p = ff_add(p, ff_mul(pen, pen));
                    const FF f = ff_div(ff_mul_f(pen, -2.0f), d);
                    gx = ff_add(gx, ff_mul(f, dx));
                    gy = ff_add(gy, ff_mul(f, dy));
                    gth = ff_add(gth, ff_mul(f, ff_add(ff_mul(dy, rx), ff_neg(ff_mul(dx, ry)))));
                }
            }
    }
    for (int sh = 16; sh; sh >>= 1) {
        p = ff_add(p, FF{__shfl_xor_sync(FULL, p.hi, sh), __shfl_xor_sync(FULL, p.lo, sh)});
        gx = ff_add(gx, FF{__shfl_xor_sync(FULL, gx.hi, sh), __shfl_xor_sync(FULL, gx.lo, sh)});
        gy = ff_add(gy, FF{__shfl_xor_sync(FULL, gy.hi, sh), __shfl_xor_sync(FULL, gy.lo, sh)});
        gth = ff_add(gth, FF{__shfl_xor_sync(FULL, gth.hi, sh), __shfl_xor_sync(FULL, gth.lo, sh)});
    }
    return ProxyOut{ff_f(p), ff_f(gx), ff_f(gy), ff_f(gth)};
}

constexpr int PROXY_WARPS = 8;

// Forward and/or adjoint for a batch: params are (theta, tx, ty) per candidate.  `value` (may be
// null) receives P; `grad` (may be null) receives dP/d(theta, tx, ty), times gscale[i] when
// `gscale` is given (the backward of a loss L with dL/dP = gscale).  A warp takes 32 consecutive
// candidates: each lane evaluates the float-float cos / sin of one of them, then the warp works
// through the 32 together, lanes over the item's poles.
__global__ void __launch_bounds__(PROXY_WARPS * 32) k_proxy(View v, const float* __restrict__ params,
                                                            const uint32_t* __restrict__ items, uint32_t n,
                                                            float* __restrict__ value, float* __restrict__ grad,
                                                            const float* __restrict__ gscale) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (uint32_t base = (blockIdx.x * PROXY_WARPS + warp) * 32u; base < n; base += gridDim.x * PROXY_WARPS * 32u) {
        FF my_s{0.0f, 0.0f}, my_c{1.0f, 0.0f};
        if (base + lane < n) ff_sincos(__ldg(&params[3 * (base + lane)]), my_s, my_c);
        const uint32_t m = min(32u, n - base);
        for (uint32_t l = 0; l < m; l++) {
            const uint32_t i = base + l;
            const FF s{__shfl_sync(FULL, my_s.hi, l), __shfl_sync(FULL, my_s.lo, l)};
            const FF c{__shfl_sync(FULL, my_c.hi, l), __shfl_sync(FULL, my_c.lo, l)};
            const uint32_t item = __ldg(&items[i]);
            if (item >= v.n_items) {
                if (lane == 0) {
                    if (value) value[i] = -1.0f;
                    if (grad) grad[3 * i] = grad[3 * i + 1] = grad[3 * i + 2] = 0.0f;
                }
                continue;
            }
            const DItem it = v.items[item];
            const ProxyOut o = proxy_eval_ff(v, it, c, s, __ldg(&params[3 * i + 1]), __ldg(&params[3 * i + 2]), lane);
            if (lane == 0) {
                if (value) value[i] = o.p;
                if (grad) {
                    const float gs = gscale ? __ldg(&gscale[i]) : 1.0f;
                    grad[3 * i] = gscale ? o.gth * gs : o.gth;
                    grad[3 * i + 1] = gscale ? o.gx * gs : o.gx;
                    grad[3 * i + 2] = gscale ? o.gy * gs : o.gy;
                }
            }
        }
    }
}

// Gradient-descent separation: `steps` descent steps on the proxy per candidate (state in
// registers).  Each step tries x - eta * D grad (D scales translation by step_t and rotation by
// step_th / max|p_i|^2); the trial is kept when it lowers the proxy (eta grows x1.5, up to 4) and
// dropped otherwise (eta halves), so the proxy never increases.  Stops when the proxy reaches 0.
// Writes the final params and the query record (item, cos, sin, tx, ty) for the exact verdict.
#ifndef JCDE_SEP_LANES
#define JCDE_SEP_LANES 32       // lanes per candidate in k_separate (measured faster than 8 or 16)
#endif
#ifndef JCDE_SEP_MARGIN
#define JCDE_SEP_MARGIN 0.25f   // motion (in item bounds) allowed before a candidate's list is gathered again
#endif
constexpr uint32_t SEP_LOCAL = 96;   // hazard poles kept per candidate for its descent

// The hazard poles a candidate at (cx, cy) can meet while it moves less than `margin`: every
// pole box overlapping the square of half-size `reach` around it, gathered once from the coarse
// grid (a pole is taken from the cell holding the low corner of its box's overlap with the square).
// Radii are stored grown by `clear`.  Returns the count, or SEP_LOCAL + 1 when they do not fit.
__device__ __forceinline__ uint32_t gather_poles(const View& v, float cx, float cy, float reach, float rdisk,
                                                 float clear, float4* list, int lane, int nsub, uint32_t mask) {
    const int g = v.hp_g_c;
    const float gx0 = cx - reach, gy0 = cy - reach, gx1 = cx + reach, gy1 = cy + reach;
    const int ix0 = pole_cell(gx0, v.hp_x0, v.hp_inv_cs_c, g), ix1 = pole_cell(gx1, v.hp_x0, v.hp_inv_cs_c, g);
    const int iy0 = pole_cell(gy0, v.hp_y0, v.hp_inv_cs_c, g), iy1 = pole_cell(gy1, v.hp_y0, v.hp_inv_cs_c, g);
    const uint32_t below = mask & ((1u << (threadIdx.x & 31)) - 1u);
    uint32_t cnt = 0;
    for (int iy = iy0; iy <= iy1; iy++)
        for (int ix = ix0; ix <= ix1; ix++) {   // the coarse cells of the square, lanes over each cell's poles
            const uint32_t cell = (uint32_t)iy * (uint32_t)g + (uint32_t)ix;
            const uint32_t a = __ldg(&v.hp_start_c[cell]), b = __ldg(&v.hp_start_c[cell + 1]);
            for (uint32_t j0 = a; j0 < b; j0 += nsub) {
                const uint32_t j = j0 + lane;
                bool take = false;
                float4 h = make_float4(0.f, 0.f, 0.f, 0.f);
                if (j < b) {
                    h = __ldg(&v.hpoles_c[j]);
                    const float mx = fmaxf(gx0, h.x - h.z), my = fmaxf(gy0, h.y - h.z);
                    const float dx = h.x - cx, dy = h.y - cy, rr = rdisk + h.z;
                    take = mx <= fminf(gx1, h.x + h.z) && my <= fminf(gy1, h.y + h.z) &&
                           pole_cell(mx, v.hp_x0, v.hp_inv_cs_c, g) == ix && pole_cell(my, v.hp_y0, v.hp_inv_cs_c, g) == iy &&
                           dx * dx + dy * dy <= rr * rr && !filtered(v, __float_as_uint(h.w));
                }
                const uint32_t bal = __ballot_sync(mask, take);
                if (take) {
                    const uint32_t pos = cnt + __popc(bal & below);
                    if (pos < SEP_LOCAL) list[pos] = make_float4(h.x, h.y, h.z + clear, 0.0f);
                }
                cnt += __popc(bal & mask);
            }
        }
    __syncwarp(mask);
    return cnt <= SEP_LOCAL ? cnt : SEP_LOCAL + 1;
}

// The proxy against a gathered list (radii already grown): lanes over the item's poles.
__device__ __forceinline__ ProxyOut proxy_local(const View& v, const DItem& it, float c, float s, float tx, float ty,
                                                const float4* list, uint32_t m, int lane, int nsub, uint32_t mask) {
    KSum p, gx, gy, gth;
    for (uint32_t k = lane; k < it.n_poles; k += nsub) {
        const float4 pl = __ldg(&v.poles[it.pole_off + k]);
        const float rx = c * pl.x - s * pl.y, ry = s * pl.x + c * pl.y;
        for (uint32_t j = 0; j < m; j++) {
            const float4 h = list[j];
            const float dx = (tx - h.x) + rx, dy = (ty - h.y) + ry;
            const float d2 = dx * dx + dy * dy;
            const float rr = pl.z + h.z;
            if (d2 >= rr * rr) continue;
            const float d = sqrtf(d2), pen = rr - d;
            p.add(pen * pen);
            if (d > 0.0f) {
                const float f = -2.0f * pen / d;
                gx.add(f * dx);
                gy.add(f * dy);
                gth.add(f * (dy * rx - dx * ry));
            }
        }
    }
    ProxyOut o{p.get(), gx.get(), gy.get(), gth.get()};
    for (int sh = nsub >> 1; sh; sh >>= 1) {
        o.p += __shfl_xor_sync(mask, o.p, sh);
        o.gx += __shfl_xor_sync(mask, o.gx, sh);
        o.gy += __shfl_xor_sync(mask, o.gy, sh);
        o.gth += __shfl_xor_sync(mask, o.gth, sh);
    }
    return o;
}

__global__ void __launch_bounds__(PROXY_WARPS * 32) k_separate(View v, float* __restrict__ params,
                                                               const uint32_t* __restrict__ items, uint32_t n,
                                                               uint32_t steps, float step_t, float step_th, float clear,
                                                               uint32_t* __restrict__ qout, float* __restrict__ value,
                                                               uint32_t* __restrict__ next) {
    constexpr int L = JCDE_SEP_LANES, PER_WARP = 32 / L;
    __shared__ float4 local[PROXY_WARPS * PER_WARP][SEP_LOCAL];
    // PER_WARP candidates per warp, L lanes each; candidates are taken from the counter `next` (the
    // descent stops early for candidates that separate, so the work per candidate varies widely)
    const int grp = (threadIdx.x & 31) / L, hl = threadIdx.x % L;
    const uint32_t mask = (L == 32 ? FULL : ((1u << L) - 1u)) << (L * grp);
    float4* list = local[(threadIdx.x >> 5) * PER_WARP + grp];
    const uint32_t groups = gridDim.x * PROXY_WARPS * PER_WARP;
    for (uint32_t i = next ? 0u : (blockIdx.x * PROXY_WARPS + (threadIdx.x >> 5)) * PER_WARP + grp;; i += groups) {
        if (next) {
            uint32_t t = 0;
            if (hl == 0) t = atomicAdd(next, 1u);
            i = __shfl_sync(mask, t, L * grp);
        }
        if (i >= n) break;
        const uint32_t item = __ldg(&items[i]);
        float th = params[3 * i], tx = params[3 * i + 1], ty = params[3 * i + 2];
        float p = -1.0f;
        if (item < v.n_items) {
            const DItem it = v.items[item];
            const float kth = step_th / fmaxf(it.pole_r2max, 1.0f);
            const float margin = JCDE_SEP_MARGIN * it.pole_bound;   // motion allowed before gathering again
            const float reach = it.pole_bound + clear + margin;
            // a hazard pole can meet an item pole only within pole_bound + clear of the item's
            // origin, and the origin moves at most margin * sqrt(2) before the list is gathered again
            const float rdisk = it.pole_bound + clear + 1.4143f * margin;
            float ox = tx, oy = ty;
            uint32_t m = gather_poles(v, ox, oy, reach, rdisk, clear, list, hl, L, mask);
            auto eval = [&](float c, float s, float x, float y) -> ProxyOut {
                if (fabsf(x - ox) > margin || fabsf(y - oy) > margin) {
                    ox = x;
                    oy = y;
                    m = gather_poles(v, ox, oy, reach, rdisk, clear, list, hl, L, mask);
                }
                return m <= SEP_LOCAL ? proxy_local(v, it, c, s, x, y, list, m, hl, L, mask)
                                      : proxy_eval(v, it, c, s, x, y, hl, L, mask, clear);
            };
            float s, c;
            sincosf(th, &s, &c);
            ProxyOut cur = eval(c, s, tx, ty);
            float eta = 1.0f;
            for (uint32_t k = 0; k < steps && cur.p > 0.0f; k++) {
                const float th2 = th - eta * kth * cur.gth;
                const float tx2 = tx - eta * step_t * cur.gx, ty2 = ty - eta * step_t * cur.gy;
                sincosf(th2, &s, &c);
                const ProxyOut trial = eval(c, s, tx2, ty2);
                if (trial.p < cur.p) {
                    th = th2;
                    tx = tx2;
                    ty = ty2;
                    cur = trial;
                    eta = fminf(eta * 1.5f, 4.0f);
                } else {
                    eta *= 0.5f;
                }
            }
            p = cur.p;
        }
        if (hl == 0) {
            params[3 * i] = th;
            params[3 * i + 1] = tx;
            params[3 * i + 2] = ty;
            value[i] = p;
            float s, c;
            sincosf(th, &s, &c);
            uint32_t* r = qout + (size_t)i * 5;
            r[0] = item;
            r[1] = __float_as_uint(c);
            r[2] = __float_as_uint(s);
            r[3] = __float_as_uint(tx);
            r[4] = __float_as_uint(ty);
        }
        __syncwarp(mask);
    }
}

// Random-resampling baseline: `k` perturbed copies of each candidate (Gaussian in translation and
// rotation, counter-based hash RNG), written as query records for the exact verdict.
__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}
__device__ __forceinline__ float gauss(uint32_t a, uint32_t b) {   // Box-Muller from two hashes
    const float u1 = ((hash32(a) >> 8) + 1u) * (1.0f / 16777217.0f);
    const float u2 = (hash32(b) >> 8) * (1.0f / 16777216.0f);
    return sqrtf(-2.0f * __logf(u1)) * __cosf(6.2831853f * u2);
}
__global__ void k_resample(const float* __restrict__ params, const uint32_t* __restrict__ items, uint32_t n, uint32_t k,
                           float sigma_t, float sigma_th, uint32_t seed, uint32_t* __restrict__ qout) {
    const uint64_t total = (uint64_t)n * k;
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < total; j += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t i = (uint32_t)(j / k);
        const uint32_t h = hash32((uint32_t)j * 4u + seed);
        const float th = params[3 * i] + sigma_th * gauss(h, h ^ 0x9e3779b9u);
        const float tx = params[3 * i + 1] + sigma_t * gauss(h + 1u, h ^ 0x85ebca6bu);
        const float ty = params[3 * i + 2] + sigma_t * gauss(h + 2u, h ^ 0xc2b2ae35u);
        float s, c;
        sincosf(th, &s, &c);
        uint32_t* r = qout + j * 5;
        r[0] = items[i];
        r[1] = __float_as_uint(c);
        r[2] = __float_as_uint(s);
        r[3] = __float_as_uint(tx);
        r[4] = __float_as_uint(ty);
    }
}

// LBF choice over a candidate batch (lbf/src/opt/search.rs:44-66 with LBFLoss, lbf/src/opt/loss.rs):
// among candidates whose verdict is JCDE_FREE, the smallest cost x_max * 10 + y_max of the
// transformed shape's bounding box, the lowest index among equal costs (the strict `<` of
// search.rs:52 keeps the first best).  Costs are mapped to order-preserving integers and
// packed with the index into one 64-bit atomicMin.
// With a grid of several rows (blockIdx.y), row y chooses among its own segment of n queries
// (queries, verdicts and the result word offset by y): one launch for several batches.
__global__ void k_lbf_select(View v, const uint32_t* __restrict__ q, const uint8_t* __restrict__ verdicts, uint32_t n,
                             unsigned long long* __restrict__ best, uint32_t* __restrict__ n_free) {
    q += (size_t)blockIdx.y * n * 5;
    verdicts += (size_t)blockIdx.y * n;
    best += blockIdx.y;
    if (n_free) n_free += blockIdx.y;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t wpb = blockDim.x >> 5;
    __shared__ unsigned long long s_best;
    __shared__ uint32_t s_free;
    if (threadIdx.x == 0) {
        s_best = ~0ull;
        s_free = 0;
    }
    __syncthreads();
    unsigned long long mine = ~0ull;   // the warp's best (lane-uniform)
    uint32_t nfree = 0;
    for (uint32_t qi = blockIdx.x * wpb + warp; qi < n; qi += gridDim.x * wpb) {
        if (verdicts[qi] != 0) continue;
        const QueryHead qh = load_query(q, qi, lane);
        if (qh.item >= v.n_items) continue;
        const DItem it = v.items[qh.item];
        const QShape sh{v.iverts + it.v_off, it.v_cnt, qh.c, qh.s, qh.tx, qh.ty, false};
        const Box b = warp_bbox(sh, lane);
        const float cost = b.x1 * 10.0f + b.y1;   // LBFLoss::cost (loss.rs:29-31)
        mine = min(mine, ((unsigned long long)orderable(cost) << 32) | qi);
        nfree++;
    }
    if (lane == 0) {
        if (mine != ~0ull) atomicMin(&s_best, mine);
        if (nfree) atomicAdd(&s_free, nfree);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_best != ~0ull) atomicMin(best, s_best);
        if (n_free && s_free) atomicAdd(n_free, s_free);
    }
}

// Strongest presence per node under a filter (QTHazardVec::strongest, qt_hazard_vec.rs:60-63).
__global__ void k_strength(View v, uint32_t n_nodes, uint8_t* __restrict__ out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_nodes) return;
    DNode nd = ld_node(v, i);
    uint8_t s = PRES_NONE;
    for (uint32_t k = 0; k < nd.hz_cnt; k++) {
        DEntry e = ld_entry(v, nd.hz_off + k);
        if (!filtered(v, e.hkey)) {
            s = (uint8_t)e.presence;
            break;
        }
    }
    out[i] = s;
}

}  // namespace jcde
