// Device-resident quadtree updates and the on-device LBF-style build (see resident.cuh).
//
// Every update kernel runs as one warp: the tree mutations of one registration form a short chain
// of dependent steps (descend, split, clip, append), and the data-parallel parts of each step
// (clipping a hazard's edges against a quadrant, the ray-cast point-in-polygon test of a quadrant
// centre, searching a node's entries) spread over the 32 lanes.  Control values are warp-uniform:
// every lane computes them, lane 0 alone writes shared state, and __syncwarp orders the writes
// before the next read.
#include "resident.cuh"

#include <algorithm>

#ifndef JCDE_UNROLL
#define JCDE_UNROLL _Pragma("unroll")
#endif

namespace jcde {

constexpr uint32_t FULL = 0xffffffffu;

enum : uint32_t { RT_REG = 0, RT_CONSTRICT = 1, RT_DEREG = 2, RT_FREE = 3 };

struct RState {
    uint32_t n_nodes, n_qfree, entry_top, edge_top, hvert_top, n_slots, n_kfree, error, not_found, n_live;
};

__device__ __forceinline__ RState r_load(const RCtl* c) {
    const volatile RCtl* v = c;
    return RState{v->n_nodes,   v->n_qfree, v->entry_top, v->edge_top,  v->hvert_top,
                  v->n_slots,   v->n_kfree, v->error,     v->not_found, v->n_live};
}
__device__ __forceinline__ void r_store(RCtl* c, const RState& s, int lane) {
    __syncwarp();
    if (lane == 0) {
        c->n_nodes = s.n_nodes;
        c->n_qfree = s.n_qfree;
        c->entry_top = s.entry_top;
        c->edge_top = s.edge_top;
        c->hvert_top = s.hvert_top;
        c->n_slots = s.n_slots;
        c->n_kfree = s.n_kfree;
        c->error = s.error;
        c->not_found = s.not_found;
        c->n_live = s.n_live;
    }
    __syncwarp();
}
__device__ __forceinline__ void r_fail(RState& s, uint32_t code) {
    if (!s.error) s.error = code;
}

__device__ __forceinline__ RTask* r_task(const RTree& t, uint32_t i) {
    return (t.stasks && i < RT_SMEM_TASKS) ? &t.stasks[i] : &t.tasks[i];
}

__device__ __forceinline__ bool r_push(const RTree& t, RState& s, uint32_t& top, int32_t node, uint32_t kind,
                                       const DEntry& e, int lane) {
    if (top >= t.task_cap) {
        r_fail(s, RES_ERR_TASKS);
        return false;
    }
    if (lane == 0) {
        RTask* k = r_task(t, top);
        k->node = node;
        k->kind = kind;
        k->e = e;
    }
    top++;
    return true;
}

// A new quartet of children under `parent` (QTNode::register_hazard's child creation,
// qt_node.rs:44-55); children boxes are Rect::quadrants of the parent (rect.rs:141-151).
__device__ int32_t r_alloc_quartet(const RTree& t, RState& s, int32_t parent, int lane) {
    int32_t c;
    bool fresh = false;
    if (s.n_qfree) {
        c = t.qfree[s.n_qfree - 1];
        s.n_qfree--;
    } else {
        if (s.n_nodes + 4 > t.node_cap) {
            r_fail(s, RES_ERR_NODES);
            return -1;
        }
        c = (int32_t)s.n_nodes;
        s.n_nodes += 4;
        fresh = true;
    }
    const Box pb = t.nodes[parent].box;
    const uint8_t pl = t.level[parent];
    __syncwarp();
    if (lane < 4) {
        DNode* n = &t.nodes[c + lane];
        n->box = box_quadrant(pb, lane);
        n->child = -1;
        n->parent = parent;
        n->hz_cnt = 0;
        if (fresh) {
            n->hz_off = 0;
            t.ncap[c + lane] = 0;
        }
        t.level[c + lane] = (uint8_t)(pl - 1);
        t.strength[c + lane] = 0;
        t.nedges[c + lane] = 0;
    }
    if (lane == 0) t.nodes[parent].child = c;
    __syncwarp();
    return c;
}

// QTHazardVec::add (qt_hazard_vec.rs:24-43) as an unordered set, with the node's caches.
__device__ bool r_append(const RTree& t, RState& s, int32_t n, const DEntry& h, int lane) {
    const uint32_t cnt = t.nodes[n].hz_cnt;
    uint32_t off = t.nodes[n].hz_off;
    const uint32_t cap = t.ncap[n];
    if (cnt == cap) {
        const uint32_t ncap = cap ? cap * 2 : 4;
        if (s.entry_top + ncap > t.entry_cap) {
            r_fail(s, RES_ERR_ENTRIES);
            return false;
        }
        const uint32_t noff = s.entry_top;
        s.entry_top += ncap;
        for (uint32_t k = lane; k < cnt; k += 32) t.entries[noff + k] = t.entries[off + k];
        off = noff;
        __syncwarp();
        if (lane == 0) {
            t.nodes[n].hz_off = off;
            t.ncap[n] = ncap;
        }
    }
    if (lane == 0) {
        t.entries[off + cnt] = h;
        t.nodes[n].hz_cnt = cnt + 1;
        if (h.presence == PRES_PARTIAL) t.nedges[n] += h.edge_cnt;
        if (t.strength[n] < h.presence) t.strength[n] = (uint8_t)h.presence;
    }
    __syncwarp();
    return true;
}

// SPolygon::collides_with(&Point) (simple_polygon.rs:255-292) for a hazard, edges over lanes.
__device__ bool r_pip(const RTree& t, const DHaz& hz, Pt p, int lane) {
    if (!box_hits_pt(hz.box, p)) return false;
    const Seg ray = pip_ray(hz.box, p);
    const uint32_t nv = hz.v_cnt_scope & 0x7FFFFFFFu;
    int n = 0;
    for (uint32_t k = lane; k < nv; k += 32) {
        const float2 a = t.hverts[hz.v_off + k], b = t.hverts[hz.v_off + (k + 1 == nv ? 0 : k + 1)];
        n += pip_edge_term(ray, Seg{Pt{a.x, a.y}, Pt{b.x, b.y}}, p);
    }
    return (__reduce_add_sync(FULL, (uint32_t)n) & 1u) == 1u;
}

// QTHazard::constrict (qt_hazard.rs:48-167) of entry h into the children of node n, followed by
// the registration of every present child entry (qt_node.rs:66-79).
__device__ void r_constrict(const RTree& t, RState& s, uint32_t& top, int32_t n, const DEntry& h, int lane) {
    const int32_t c = t.nodes[n].child;
    Box q[4];
    for (int i = 0; i < 4; i++) q[i] = t.nodes[c + i].box;
    DEntry out[4];
    if (h.presence == PRES_ENTIRE) {
        for (int i = 0; i < 4; i++) out[i] = h;
    } else {
        const DHaz hz = t.haz[h.hkey];
        int enc = -1;
        for (int i = 0; i < 4 && enc < 0; i++)
            if (box_relation(hz.box, q[i]) == REL_ENCLOSED) enc = i;
        if (enc >= 0) {   // the whole shape lies in one quadrant (qt_hazard.rs:63-80)
            for (int i = 0; i < 4; i++) {
                out[i] = h;
                if (i != enc) out[i].presence = PRES_NONE;
            }
        } else {
            bool resolved[4];
            const uint32_t lt = (1u << lane) - 1u;
            constexpr uint32_t HELD = 4;   // edges per lane kept in registers by the one-pass clip
            if (h.edge_cnt <= 32 * HELD) {
                // one pass: every lane loads its edges once and tests them against the four
                // quadrants; exact-size lists are then written from registers
                float4 f[HELD];
                uint32_t qm[HELD];
                JCDE_UNROLL
                for (uint32_t r = 0; r < HELD; r++) {
                    const uint32_t k = r * 32 + lane;
                    f[r] = make_float4(0.f, 0.f, 0.f, 0.f);
                    qm[r] = 0;
                    if (k < h.edge_cnt) {
                        f[r] = t.edges[h.edge_off + k];
                        const Seg sg{Pt{f[r].x, f[r].y}, Pt{f[r].z, f[r].w}};
                        for (int i = 0; i < 4; i++)
                            if (box_hits_seg(q[i], sg)) qm[r] |= 1u << i;
                    }
                }
                uint32_t need = 0, cnt[4];
                for (int i = 0; i < 4; i++) {
                    cnt[i] = 0;
                    JCDE_UNROLL
                    for (uint32_t r = 0; r < HELD; r++) cnt[i] += __popc(__ballot_sync(FULL, (qm[r] >> i) & 1u));
                    if (cnt[i] && cnt[i] != h.edge_cnt) need += cnt[i];
                }
                if (s.edge_top + need > t.edge_cap) {
                    r_fail(s, RES_ERR_EDGES);
                    return;
                }
                for (int i = 0; i < 4; i++) {
                    resolved[i] = cnt[i] > 0;
                    out[i] = DEntry{Box{0.f, 0.f, 0.f, 0.f}, h.hkey, 0u, 0u, PRES_NONE};
                    if (cnt[i] == 0) continue;
                    if (cnt[i] == h.edge_cnt) {   // every edge: the parent's list and ff box
                        out[i] = h;
                        continue;
                    }
                    const uint32_t dst = s.edge_top;
                    s.edge_top += cnt[i];
                    float x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
                    uint32_t pos = 0;
                    JCDE_UNROLL
                    for (uint32_t r = 0; r < HELD; r++) {
                        const bool hit = (qm[r] >> i) & 1u;
                        const uint32_t bal = __ballot_sync(FULL, hit);
                        if (hit) {
                            t.edges[dst + pos + __popc(bal & lt)] = f[r];
                            x0 = fmn(fmn(x0, f[r].x), f[r].z);
                            y0 = fmn(fmn(y0, f[r].y), f[r].w);
                            x1 = fmx(fmx(x1, f[r].x), f[r].z);
                            y1 = fmx(fmx(y1, f[r].y), f[r].w);
                        }
                        pos += __popc(bal);
                    }
#pragma unroll
                    for (int o = 16; o; o >>= 1) {
                        x0 = fmn(x0, __shfl_xor_sync(FULL, x0, o));
                        y0 = fmn(y0, __shfl_xor_sync(FULL, y0, o));
                        x1 = fmx(x1, __shfl_xor_sync(FULL, x1, o));
                        y1 = fmx(y1, __shfl_xor_sync(FULL, y1, o));
                    }
                    // QTHazPartial::from_parent (qt_partial_hazard.rs:25-59)
                    const Box ff = (x0 < x1 && y0 < y1) ? Box{x0, y0, x1, y1} : h.ff;
                    out[i] = DEntry{ff, h.hkey, dst, cnt[i], PRES_PARTIAL};
                }
            } else
            for (int i = 0; i < 4; i++) {
                // the edges hitting quadrant i, compacted in order at the top of the edge pool
                if (s.edge_top + h.edge_cnt > t.edge_cap) {
                    r_fail(s, RES_ERR_EDGES);
                    return;
                }
                const uint32_t dst = s.edge_top;
                uint32_t cnt = 0;
                float x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
                for (uint32_t b = 0; b < h.edge_cnt; b += 32) {
                    const uint32_t k = b + lane;
                    bool hit = false;
                    float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (k < h.edge_cnt) {
                        f = t.edges[h.edge_off + k];
                        hit = box_hits_seg(q[i], Seg{Pt{f.x, f.y}, Pt{f.z, f.w}});
                    }
                    const uint32_t bal = __ballot_sync(FULL, hit);
                    if (hit) {
                        t.edges[dst + cnt + __popc(bal & lt)] = f;
                        x0 = fmn(fmn(x0, f.x), f.z);
                        y0 = fmn(fmn(y0, f.y), f.w);
                        x1 = fmx(fmx(x1, f.x), f.z);
                        y1 = fmx(fmx(y1, f.y), f.w);
                    }
                    cnt += __popc(bal);
                }
                resolved[i] = cnt > 0;
                out[i] = DEntry{Box{0.f, 0.f, 0.f, 0.f}, h.hkey, 0u, 0u, PRES_NONE};
                if (cnt == 0) continue;
                if (cnt == h.edge_cnt) {   // every edge: the parent's list and ff box
                    out[i] = h;
                    continue;
                }
#pragma unroll
                for (int o = 16; o; o >>= 1) {
                    x0 = fmn(x0, __shfl_xor_sync(FULL, x0, o));
                    y0 = fmn(y0, __shfl_xor_sync(FULL, y0, o));
                    x1 = fmx(x1, __shfl_xor_sync(FULL, x1, o));
                    y1 = fmx(y1, __shfl_xor_sync(FULL, y1, o));
                }
                s.edge_top += cnt;
                // QTHazPartial::from_parent (qt_partial_hazard.rs:25-59)
                const Box ff = (x0 < x1 && y0 < y1) ? Box{x0, y0, x1, y1} : h.ff;
                out[i] = DEntry{ff, h.hkey, dst, cnt, PRES_PARTIAL};
            }
            // quadrants without edges: presence from resolved neighbours, else the centre's PIP
            // (qt_hazard.rs:110-160; neighbours of Rect::QUADRANT_NEIGHBOR_LAYOUT, rect.rs:136)
            const int NB[4][2] = {{1, 3}, {0, 2}, {1, 3}, {0, 2}};
            const bool ext = (hz.v_cnt_scope >> 31) != 0;
            for (int i = 0; i < 4; i++) {
                if (resolved[i]) continue;
                bool none_nb = false, entire_nb = false;
                for (int k = 0; k < 2; k++) {
                    const int nb = NB[i][k];
                    if (!resolved[nb]) continue;
                    none_nb |= out[nb].presence == PRES_NONE;
                    entire_nb |= out[nb].presence == PRES_ENTIRE;
                }
                uint32_t p;
                if (none_nb && !entire_nb) p = PRES_NONE;
                else if (entire_nb && !none_nb) p = PRES_ENTIRE;
                else {
                    const bool inside = r_pip(t, hz, box_mid(q[i]), lane);
                    p = (!ext && inside) || (ext && !inside) ? PRES_ENTIRE : PRES_NONE;
                }
                out[i] = DEntry{Box{0.f, 0.f, 0.f, 0.f}, h.hkey, 0u, 0u, p};
                resolved[i] = true;
            }
        }
    }
    for (int i = 3; i >= 0; i--)
        if (out[i].presence != PRES_NONE && !r_push(t, s, top, c + i, RT_REG, out[i], lane)) return;
}

// Works off the task stack: QTNode::register_hazard (qt_node.rs:38-81).  A leaf above level 0
// that receives a Partial hazard grows children and pushes its present hazards down first.
// Entries are sets and every constricted entry ends in the same nodes whatever the order the
// tasks run in, so the stack order is free.
__device__ void r_run_register(const RTree& t, RState& s, uint32_t top, int lane) {
    while (top > 0 && !s.error) {
        __syncwarp();
        const RTask tk = *r_task(t, --top);
        __syncwarp();
        const int32_t n = tk.node;
        if (tk.kind == RT_CONSTRICT) {
            r_constrict(t, s, top, n, tk.e, lane);
            continue;
        }
        int32_t child = t.nodes[n].child;
        if (child < 0 && t.level[n] > 0 && tk.e.presence == PRES_PARTIAL) {
            const uint32_t cnt = t.nodes[n].hz_cnt, off = t.nodes[n].hz_off;
            child = r_alloc_quartet(t, s, n, lane);
            if (child < 0) return;
            for (uint32_t k = 0; k < cnt; k++)
                if (!r_push(t, s, top, n, RT_CONSTRICT, t.entries[off + k], lane)) return;
        }
        if (child >= 0 && !r_push(t, s, top, n, RT_CONSTRICT, tk.e, lane)) return;
        if (!r_append(t, s, n, tk.e, lane)) return;
    }
}

// CDEngine::register_hazard (cd_engine.rs:59-70) of a polygon: its vertices (transformed by the
// matrix (c, sn, tx, ty) when `xf`) enter the hazard vertex pool, its full edge list the edge pool
// (QTHazard::from_root, qt_hazard.rs:36-43), then the root registration runs.  Returns the key.
__device__ uint32_t r_insert(const RTree& t, RState& s, const float2* verts, uint32_t nv, bool xf, float c, float sn,
                             float tx, float ty, Pt poi, bool exterior, int64_t forced_key, int lane) {
    uint32_t key;
    if (forced_key >= 0) {
        key = (uint32_t)forced_key;
    } else if (s.n_kfree) {
        key = t.kfree[s.n_kfree - 1];
        s.n_kfree--;
    } else {
        if (s.n_slots >= t.key_cap) {
            r_fail(s, RES_ERR_KEYS);
            return ~0u;
        }
        key = s.n_slots++;
    }
    if (s.hvert_top + nv > t.hvert_cap) {
        r_fail(s, RES_ERR_HVERTS);
        return ~0u;
    }
    if (s.edge_top + nv > t.edge_cap) {
        r_fail(s, RES_ERR_EDGES);
        return ~0u;
    }
    const uint32_t voff = s.hvert_top;
    s.hvert_top += nv;
    float x0 = FLT_MAX, y0 = FLT_MAX, x1 = -FLT_MAX, y1 = -FLT_MAX;
    for (uint32_t k = lane; k < nv; k += 32) {
        const float2 f = verts[k];
        const Pt p = xf ? xform(Pt{f.x, f.y}, c, sn, tx, ty) : Pt{f.x, f.y};
        t.hverts[voff + k] = make_float2(p.x, p.y);
        x0 = fmn(x0, p.x);
        y0 = fmn(y0, p.y);
        x1 = fmx(x1, p.x);
        y1 = fmx(y1, p.y);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        x0 = fmn(x0, __shfl_xor_sync(FULL, x0, o));
        y0 = fmn(y0, __shfl_xor_sync(FULL, y0, o));
        x1 = fmx(x1, __shfl_xor_sync(FULL, x1, o));
        y1 = fmx(y1, __shfl_xor_sync(FULL, y1, o));
    }
    const Box bb{x0, y0, x1, y1};   // SPolygon::generate_bounding_box (simple_polygon.rs:122-133)
    __syncwarp();
    const uint32_t eoff = s.edge_top;
    s.edge_top += nv;
    for (uint32_t k = lane; k < nv; k += 32) {
        const float2 a = t.hverts[voff + k], b = t.hverts[voff + (k + 1 == nv ? 0 : k + 1)];
        t.edges[eoff + k] = make_float4(a.x, a.y, b.x, b.y);
    }
    if (lane == 0) {
        t.haz[key] = DHaz{bb, poi.x, poi.y, voff, nv | (exterior ? 0x80000000u : 0u)};
        t.alive[key] = 1;
    }
    s.n_live++;
    __syncwarp();
    uint32_t top = 0;
    if (r_push(t, s, top, 0, RT_REG, DEntry{bb, key, eoff, nv, PRES_PARTIAL}, lane)) r_run_register(t, s, top, lane);
    return key;
}

// CDEngine::deregister_hazard_by_key (cd_engine.rs:87-96) with QTNode::deregister_hazard
// (qt_node.rs:83-94): a node that keeps no Partial hazard drops its children.
__device__ bool r_remove(const RTree& t, RState& s, uint32_t key, int lane) {
    if (key >= s.n_slots || !t.alive[key]) {
        s.not_found++;
        return false;
    }
    uint32_t top = 0;
    const DEntry none{};
    if (!r_push(t, s, top, 0, RT_DEREG, none, lane)) return false;
    const uint32_t lt_all = FULL;
    while (top > 0 && !s.error) {
        __syncwarp();
        const RTask tk = *r_task(t, --top);
        __syncwarp();
        const int32_t n = tk.node;
        if (tk.kind == RT_FREE) {   // free a quartet and, below it, every descendant quartet
            for (int i = 3; i >= 0; i--) {
                const int32_t ch = t.nodes[n + i].child;
                if (ch >= 0 && !r_push(t, s, top, ch, RT_FREE, none, lane)) return false;
            }
            __syncwarp();
            if (lane < 4) {
                t.nodes[n + lane].child = -1;
                t.nodes[n + lane].hz_cnt = 0;
                t.nedges[n + lane] = 0;
                t.strength[n + lane] = 0;
            }
            if (lane == 0) t.qfree[s.n_qfree] = n;
            s.n_qfree++;
            continue;
        }
        const uint32_t cnt = t.nodes[n].hz_cnt, off = t.nodes[n].hz_off;
        int32_t idx = -1;
        for (uint32_t b = 0; b < cnt && idx < 0; b += 32) {
            const uint32_t k = b + lane;
            const uint32_t bal = __ballot_sync(lt_all, k < cnt && t.entries[off + k].hkey == key);
            if (bal) idx = (int32_t)(b + __ffs(bal) - 1);
        }
        if (idx < 0) continue;
        const DEntry e = t.entries[off + idx];
        const DEntry last = t.entries[off + cnt - 1];
        __syncwarp();
        if (lane == 0) {
            t.entries[off + idx] = last;
            t.nodes[n].hz_cnt = cnt - 1;
            if (e.presence == PRES_PARTIAL) t.nedges[n] -= e.edge_cnt;
        }
        __syncwarp();
        uint32_t mx = 0;
        bool partial = false;
        for (uint32_t k = lane; k < cnt - 1; k += 32) {
            const uint32_t p = t.entries[off + k].presence;
            mx = max(mx, p);
            partial |= p == PRES_PARTIAL;
        }
        mx = __reduce_max_sync(FULL, mx);
        partial = __any_sync(FULL, partial);
        if (lane == 0) t.strength[n] = (uint8_t)mx;
        const int32_t child = t.nodes[n].child;
        __syncwarp();
        if (child < 0) continue;
        if (!partial) {
            if (lane == 0) t.nodes[n].child = -1;
            if (!r_push(t, s, top, child, RT_FREE, none, lane)) return false;
        } else {
            for (int i = 3; i >= 0; i--)
                if (!r_push(t, s, top, child + i, RT_DEREG, none, lane)) return false;
        }
    }
    __syncwarp();
    if (lane == 0) {
        t.alive[key] = 0;
        t.kfree[s.n_kfree] = key;
    }
    s.n_kfree++;
    s.n_live--;
    __syncwarp();
    return true;
}

// ---------------------------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------------------------

// Copy of a host tree: the root node, then every live hazard registered under its own key.
__global__ void __launch_bounds__(32) k_res_init(RTree tg, const float2* __restrict__ verts, const uint4* __restrict__ recs,
                                                 const float2* __restrict__ pois, uint32_t n, uint32_t n_slots,
                                                 const uint32_t* __restrict__ kfree, uint32_t n_kfree) {
    __shared__ RTask stasks[RT_SMEM_TASKS];
    RTree t = tg;
    t.stasks = stasks;
    const int lane = threadIdx.x;
    RState s{};
    s.n_nodes = 1;
    if (lane == 0) {
        t.nodes[0] = DNode{t.cde, -1, -1, 0u, 0u};
        t.ncap[0] = 0;
        t.level[0] = (uint8_t)t.depth;
        t.strength[0] = 0;
        t.nedges[0] = 0;
    }
    __syncwarp();
    for (uint32_t i = 0; i < n && !s.error; i++) {
        const uint4 r = recs[i];   // key, kind, vertex offset, vertex count
        const float2 p = pois[i];
        r_insert(t, s, verts + r.z, r.w, false, 1.f, 0.f, 0.f, 0.f, Pt{p.x, p.y}, r.y == KIND_EXTERIOR, (int64_t)r.x,
                 lane);
    }
    s.n_slots = n_slots;
    if (n_kfree > t.key_cap) r_fail(s, RES_ERR_KEYS);
    else {
        for (uint32_t k = lane; k < n_kfree; k += 32) t.kfree[k] = kfree[k];
        s.n_kfree = n_kfree;
    }
    r_store(t.ctl, s, lane);
    if (lane == 0) t.ctl->last_key = ~0u;
}

struct RQuery {
    uint32_t item;
    float c, s, tx, ty;
};
__device__ __forceinline__ RQuery r_query(const uint32_t* q, uint32_t i) {
    const uint32_t* p = q + (size_t)i * 5;
    return RQuery{p[0], __uint_as_float(p[1]), __uint_as_float(p[2]), __uint_as_float(p[3]), __uint_as_float(p[4])};
}

// PlacedItem::new (entities/placed_item.rs:27-36) + register: the item's shape and reference
// point under the query's transformation become a placed-item hazard.
__device__ uint32_t r_insert_item(const RTree& t, RState& s, const DItem* items, const float2* iverts, const RQuery& q,
                                  int lane) {
    const DItem it = items[q.item];
    const Pt poi = xform(Pt{it.poi_x, it.poi_y}, q.c, q.s, q.tx, q.ty);
    return r_insert(t, s, iverts + it.v_off, it.v_cnt, true, q.c, q.s, q.tx, q.ty, poi, false, -1, lane);
}

__global__ void __launch_bounds__(32) k_res_insert_placed(RTree tg, const DItem* __restrict__ items,
                                                          const float2* __restrict__ iverts, uint32_t n_items,
                                                          const uint32_t* __restrict__ q, uint32_t* __restrict__ out_key) {
    __shared__ RTask stasks[RT_SMEM_TASKS];
    RTree t = tg;
    t.stasks = stasks;
    const int lane = threadIdx.x;
    RState s = r_load(t.ctl);
    uint32_t key = ~0u;
    const RQuery rq = r_query(q, 0);
    if (!s.error) {
        if (rq.item >= n_items) s.not_found++;
        else key = r_insert_item(t, s, items, iverts, rq, lane);
        if (s.error) key = ~0u;
    }
    r_store(t.ctl, s, lane);
    if (lane == 0) {
        t.ctl->last_key = key;
        if (out_key) *out_key = key;
    }
}

__global__ void __launch_bounds__(32) k_res_remove(RTree tg, const uint32_t* __restrict__ key) {
    __shared__ RTask stasks[RT_SMEM_TASKS];
    RTree t = tg;
    t.stasks = stasks;
    const int lane = threadIdx.x;
    RState s = r_load(t.ctl);
    if (!s.error) r_remove(t, s, *key, lane);
    r_store(t.ctl, s, lane);
}

// --- counter-based random streams (the seeded generator of the synthetic workloads) ------------
__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
__device__ __forceinline__ unsigned long long draw(unsigned long long key, unsigned long long i) {
    return mix64(mix64(i) ^ key);
}
__device__ __forceinline__ unsigned long long stream_key(unsigned long long seed, unsigned long long sid) {
    return mix64(seed * 0x100000001B3ull + sid * 0x9E3779B97F4A7C15ull);
}

// (cos, sin) of 2*pi*u, u in [0, 1): quadrant reduction and Taylor series in Horner form, float64
// additions and multiplications only (each separately rounded), then rounded to float32.
__constant__ double SIN_TAYLOR[13] = {
    0x1.0000000000000p+0,   -0x1.5555555555555p-3,  0x1.1111111111111p-7,  -0x1.a01a01a01a01ap-13,
    0x1.71de3a556c734p-19,  -0x1.ae64567f544e4p-26, 0x1.6124613a86d09p-33, -0x1.ae7f3e733b81fp-41,
    0x1.952c77030ad4ap-49,  -0x1.2f49b46814157p-57, 0x1.71b8ef6dcf572p-66, -0x1.761b413163819p-75,
    0x1.3f3ccdd165fa9p-84};
__constant__ double COS_TAYLOR[13] = {
    0x1.0000000000000p+0,   -0x1.0000000000000p-1,  0x1.5555555555555p-5,  -0x1.6c16c16c16c17p-10,
    0x1.a01a01a01a01ap-16,  -0x1.27e4fb7789f5cp-22, 0x1.1eed8eff8d898p-29, -0x1.93974a8c07c9dp-37,
    0x1.ae7f3e733b81fp-45,  -0x1.6827863b97d97p-53, 0x1.e542ba4020225p-62, -0x1.0ce396db7f853p-70,
    0x1.f2cf01972f578p-80};
__device__ __forceinline__ void sincos_turns_d(double u, double& dc, double& ds) {
    const double q = __dmul_rn(u, 4.0);
    const double k = floor(q);
    const double r = __dsub_rn(q, k);
    const double phi = __dmul_rn(r, 0x1.921fb54442d18p+0);
    const double p2 = __dmul_rn(phi, phi);
    double s = SIN_TAYLOR[12], c = COS_TAYLOR[12];
    for (int j = 11; j >= 0; j--) s = __dadd_rn(__dmul_rn(s, p2), SIN_TAYLOR[j]);
    for (int j = 11; j >= 0; j--) c = __dadd_rn(__dmul_rn(c, p2), COS_TAYLOR[j]);
    s = __dmul_rn(s, phi);
    switch ((int)k & 3) {
        case 0: dc = c; ds = s; break;
        case 1: dc = -s; ds = c; break;
        case 2: dc = -c; ds = -s; break;
        default: dc = s; ds = -c; break;
    }
}
__device__ __forceinline__ void sincos_turns(double u, float& co, float& si) {
    double dc, ds;
    sincos_turns_d(u, dc, ds);
    co = __double2float_rn(dc);
    si = __double2float_rn(ds);
}

// Natural logarithm of a positive normal double with IEEE additions, multiplications and divisions
// only, in the host generator's order (workload.ln_f64): x = m 2^e, m in [sqrt(1/2), sqrt(2)),
// ln m = 2 atanh(z), z = (m-1)/(m+1), 13 terms of the atanh series.
__constant__ double ATANH_C[13] = {
    0x1.0000000000000p+0, 0x1.5555555555555p-2, 0x1.999999999999ap-3, 0x1.2492492492492p-3,
    0x1.c71c71c71c71cp-4, 0x1.745d1745d1746p-4, 0x1.3b13b13b13b14p-4, 0x1.1111111111111p-4,
    0x1.e1e1e1e1e1e1ep-5, 0x1.af286bca1af28p-5, 0x1.8618618618618p-5, 0x1.642c8590b2164p-5,
    0x1.47ae147ae147bp-5};
__device__ __forceinline__ double ln_f64(double x) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    double e = (double)((long long)((bits >> 52) & 0x7FFull) - 1022);
    double m = __longlong_as_double((long long)((bits & ((1ull << 52) - 1)) | (1022ull << 52)));
    if (m < 0x1.6a09e667f3bcdp-1) {
        m = __dmul_rn(m, 2.0);
        e = __dsub_rn(e, 1.0);
    }
    const double z = __ddiv_rn(__dsub_rn(m, 1.0), __dadd_rn(m, 1.0));
    const double z2 = __dmul_rn(z, z);
    double sum = ATANH_C[12];
    for (int j = 11; j >= 0; j--) sum = __dadd_rn(__dmul_rn(sum, z2), ATANH_C[j]);
    const double t = __dmul_rn(__dmul_rn(2.0, z), sum);
    return __dadd_rn(__dmul_rn(e, 0x1.62e42fefa39efp-1), __dadd_rn(__dmul_rn(e, 0x1.abc9e3b39803fp-56), t));
}
// Box-Muller pair (workload.normal_pair): u1 in (0, 1], u2 in [0, 1)
__device__ __forceinline__ void normal_pair(double u1, double u2, double& z0, double& z1) {
    const double r = __dsqrt_rn(__dmul_rn(-2.0, ln_f64(u1)));
    double c, s;
    sincos_turns_d(u2, c, s);
    z0 = __dmul_rn(r, c);
    z1 = __dmul_rn(r, s);
}
__device__ __forceinline__ double draw_f64(unsigned long long key, unsigned long long i) {
    return (double)(draw(key, i) >> 11) * 0x1p-53;
}
__device__ __forceinline__ float draw_f32(unsigned long long key, unsigned long long i) {
    return __fmul_rn((float)(uint32_t)(draw(key, i) >> 40), 0x1p-24f);
}
__device__ __forceinline__ float draw_uniform(unsigned long long key, unsigned long long i, float lo, float hi,
                                              float hi_below) {
    return fminf(__fadd_rn(lo, __fmul_rn(draw_f32(key, i), __fsub_rn(hi, lo))), hi_below);
}

struct GenBox {
    float x0, x1, x1_below, y0, y1, y1_below;
};

// Candidate i of n of item t from the stream `key` — make_queries' draws in the workload generator:
// draw n+i: rotation (turns through sincos_turns, or one of the ocnt allowed (cos, sin) pairs by
// the draw modulo their count), 2n+i: x, 3n+i: y, uniform over the box.  qu[i] keeps the turns.
__device__ __forceinline__ void gen_uniform(unsigned long long key, unsigned long long n, uint32_t i, uint32_t t,
                                            const GenBox& b, const float2* orient, uint32_t ocnt, uint32_t* q,
                                            double* qu) {
    float c, s;
    double u = 0.0;
    const unsigned long long d = draw(key, n + i);
    if (ocnt) {
        const float2 cs = orient[(uint32_t)(d % ocnt)];
        c = cs.x;
        s = cs.y;
    } else {
        u = (double)(d >> 11) * 0x1p-53;
        sincos_turns(u, c, s);
    }
    uint32_t* r = q + (size_t)i * 5;
    r[0] = t;
    r[1] = __float_as_uint(c);
    r[2] = __float_as_uint(s);
    r[3] = __float_as_uint(draw_uniform(key, 2 * n + i, b.x0, b.x1, b.x1_below));
    r[4] = __float_as_uint(draw_uniform(key, 3 * n + i, b.y0, b.y1, b.y1_below));
    if (qu) qu[i] = u;
}

struct GenSegs {   // per segment (blockIdx.y): stream key and box, passed by value
    unsigned long long key[RES_GEN_SEGMENTS];
    GenBox box[RES_GEN_SEGMENTS];
};

__global__ void k_gen_candidates(GenSegs g, uint32_t n, uint32_t t, const float2* orient, uint32_t ocnt, uint32_t* q,
                                 double* qu) {
    const uint32_t k = blockIdx.y;
    uint32_t* qk = q + (size_t)k * n * 5;
    double* uk = qu ? qu + (size_t)k * n : nullptr;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        gen_uniform(g.key[k], n, i, t, g.box[k], orient, ocnt, qk, uk);
}

// Float value of an order-preserving cost key (the inverse of `orderable`).
__device__ __forceinline__ float cost_of_key(uint32_t v) {
    return __uint_as_float((v & 0x80000000u) ? (v & 0x7FFFFFFFu) : ~v);
}

// Candidates of round `round` of the current step.  The item type t ~ U{0..T-1} comes from the type
// stream (one draw per step).  Rounds 0 .. uni_rounds-1 are the uniform phase: round u draws
// rotation ~ U[0, 2pi) and translation ~ U(box) (make_queries' draws: n+i rotation, 2n+i x, 3n+i y)
// from the step's stream (seed, sid_base + s) for u = 0, else from (seed, uni_sid_base + 64 s + u)
// over the box whose x1 is the step's best cost so far / 10 (LBFLoss::tighten_sample_bbox,
// loss.rs:34-44) when there is a best.  Later rounds are local search: round r = round - uni_rounds + 1
// draws around the step's best so far from stream (seed, ls_sid_base + 64 s + r): x and y offsets
// float32(sigma * z) with the Box-Muller pair of draws i, m+i, the rotation sigma_turns * z' turns
// with the pair of draws 2m+i, 3m+i; with no best yet the round's candidates are marked invalid.
// `qu` keeps each candidate's turns.
__global__ void k_lbf_gen(LbfParams p, LbfDev* __restrict__ st, uint32_t* __restrict__ q, double* __restrict__ qu,
                          uint32_t round, bool ahead, uint32_t slot) {
    pdl_wait();
    // `ahead`: the first round of the next step, drawn while this step commits (the step state is
    // the commit's to clear); its step is gen_step[slot]
    const uint32_t step = ahead ? *(volatile uint32_t*)&st->gen_step[slot] : *(volatile uint32_t*)&st->step;
    if (round == 0 && blockIdx.x == 0 && threadIdx.x == 0) st->gen_step[slot ^ 1u] = step + 1;
    if (step >= p.max_steps) return;
    if (blockIdx.x == 0 && threadIdx.x == 0 && !ahead) {
        if (round == 0) {
            st->n_free = 0;
            st->rec_cost = ~0u;
            st->best = ~0ull;
        } else {
            // The round's choice starts from the step's best so far (key: its cost, index ~0), as
            // lbf's search tests a sample only if it beats the best so far (search.rs:52-56, :88): a
            // candidate that cannot is left unjudged by the polygon pass, and when none beats it the
            // merge keeps the best (its cost is not strictly lower).
            const uint32_t rc = st->rec_cost;
            st->best = rc == ~0u ? ~0ull : (((unsigned long long)rc << 32) | 0xFFFFFFFFull);
        }
    }
    const uint32_t t = p.seq ? p.seq[step] : (uint32_t)(draw(p.key_types, step) % p.n_types);
    uint32_t ooff = 0, ocnt = 0;   // allowed orientations of the item (none listed: continuous)
    if (p.orient_of) {
        const uint2 oo = p.orient_of[t];
        ooff = oo.x;
        ocnt = oo.y;
    }
    const volatile LbfDev* vs = st;
    if (round < p.uni_rounds) {
        const unsigned long long key = round == 0 ? stream_key(p.seed, (unsigned long long)p.sid_base + step)
                                                  : stream_key(p.seed, p.uni_sid_base + 64ull * step + round);
        GenBox b{p.x0, p.x1, p.x1_below, p.y0, p.y1, p.y1_below};
        const uint32_t rc = round == 0 ? ~0u : vs->rec_cost;
        if (rc != ~0u) {
            b.x1 = fminf(p.x1, __fdiv_rn(cost_of_key(rc), 10.0f));
            b.x1_below = nextafterf(b.x1, p.x0);
        }
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < p.n_uni; i += gridDim.x * blockDim.x)
            gen_uniform(key, p.n_uni, i, t, b, p.orient + ooff, ocnt, q, qu);
        return;
    }
    const uint32_t r = round - p.uni_rounds + 1;
    const bool have = vs->rec_cost != ~0u;
    const double ub = vs->rec_u;
    const float txb = __uint_as_float(vs->rec_q[3]), tyb = __uint_as_float(vs->rec_q[4]);
    const unsigned long long key = stream_key(p.seed, p.ls_sid_base + 64ull * step + r);
    const unsigned long long m = p.ls_cand;
    const double sg = (double)p.ls_sig[r], sth = p.ls_sth[r];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < p.ls_cand; i += gridDim.x * blockDim.x) {
        uint32_t* o = q + (size_t)i * 5;
        if (!have) {
            o[0] = 0xFFFFFFFFu;   // no best to search around: an invalid item, never free
            continue;
        }
        double zx, zy, zr, zu;
        normal_pair(__dsub_rn(1.0, draw_f64(key, i)), draw_f64(key, m + i), zx, zy);
        normal_pair(__dsub_rn(1.0, draw_f64(key, 2 * m + i)), draw_f64(key, 3 * m + i), zr, zu);
        float c, s;
        double u = ub;
        if (ocnt) {   // discrete orientations: the best's rotation is kept
            c = __uint_as_float(vs->rec_q[1]);
            s = __uint_as_float(vs->rec_q[2]);
        } else {
            const double x = __dadd_rn(ub, __dmul_rn(sth, zr));
            u = __dsub_rn(x, floor(x));
            sincos_turns(u, c, s);
        }
        o[0] = t;
        o[1] = __float_as_uint(c);
        o[2] = __float_as_uint(s);
        o[3] = __float_as_uint(__fadd_rn(txb, __double2float_rn(__dmul_rn(sg, zx))));
        o[4] = __float_as_uint(__fadd_rn(tyb, __double2float_rn(__dmul_rn(sg, zy))));
        qu[i] = u;
    }
}

// The step's best so far takes the round's choice when it costs strictly less (the first best
// is kept on ties, as search.rs:52 keeps it).
__device__ __forceinline__ void lbf_merge(LbfDev* st, const uint32_t* q, const double* qu, uint32_t round) {
    const unsigned long long b = st->best;
    if (b == ~0ull) return;
    const uint32_t cost = (uint32_t)(b >> 32), idx = (uint32_t)b;
    if (cost >= st->rec_cost) return;
    st->rec_cost = cost;
    st->rec_u = qu[idx];
    for (int k = 0; k < 5; k++) st->rec_q[k] = q[(size_t)idx * 5 + k];
    st->rec_cand = (round << 24) | idx;
}
__global__ void k_lbf_merge(LbfDev* __restrict__ st, const uint32_t* __restrict__ q, const double* __restrict__ qu,
                            uint32_t round) {
    pdl_wait();
    if (threadIdx.x == 0) lbf_merge(st, q, qu, round);
}

// End of a step: log it, register the chosen candidate, and every `remove_every` steps remove the
// placed item at a random position of the placement list (Layout::remove_item, layout.rs:88-100).
__global__ void __launch_bounds__(32) k_lbf_commit(RTree tg, const DItem* __restrict__ items,
                                                   const float2* __restrict__ iverts, uint32_t n_items, LbfParams p,
                                                   LbfDev* __restrict__ st, const uint32_t* __restrict__ q,
                                                   const double* __restrict__ qu, uint32_t round,
                                                   const uint8_t* __restrict__ verdicts, LbfLogs logs, bool ahead) {
    __shared__ RTask stasks[RT_SMEM_TASKS];
    pdl_wait();
    RTree t = tg;
    t.stasks = stasks;
    const int lane = threadIdx.x;
    volatile LbfDev* vs = st;
    const uint32_t step = vs->step;
    if (step >= p.max_steps) return;
    RState s = r_load(t.ctl);
    if (s.error) return;
    if (lane == 0) lbf_merge(st, q, qu, round);   // the last round's choice
    __syncwarp();
    uint32_t n_live = vs->n_live, n_removed = vs->n_removed, n_placed = vs->n_placed;
    if (lane == 0) logs.free_counts[step] = vs->n_free;
    if (logs.vlog && step < p.vlog_steps)   // (the verdicts of the last round)
        for (uint32_t i = lane; i < p.n_cand; i += 32) logs.vlog[(size_t)step * p.n_cand + i] = verdicts[i];
    if (vs->rec_cost != ~0u) {
        const uint32_t ci = vs->rec_cand;
        const RQuery rq{vs->rec_q[0], __uint_as_float(vs->rec_q[1]), __uint_as_float(vs->rec_q[2]),
                        __uint_as_float(vs->rec_q[3]), __uint_as_float(vs->rec_q[4])};
        const uint32_t key = rq.item < n_items ? r_insert_item(t, s, items, iverts, rq, lane) : ~0u;
        if (key != ~0u && !s.error) {
            if (lane == 0) {
                logs.live[n_live] = key;
                uint32_t* pl = logs.placements + (size_t)n_placed * 8;
                pl[0] = step;
                pl[1] = key;
                pl[2] = ci;
                pl[3] = rq.item;
                pl[4] = __float_as_uint(rq.c);
                pl[5] = __float_as_uint(rq.s);
                pl[6] = __float_as_uint(rq.tx);
                pl[7] = __float_as_uint(rq.ty);
            }
            n_live++;
            n_placed++;
        }
    }
    if (p.remove_every && (step + 1) % p.remove_every == 0 && n_live > 0 && !s.error) {
        __syncwarp();
        const uint32_t j = (uint32_t)(draw(p.key_remove, n_removed) % n_live);
        const uint32_t key = logs.live[j];
        for (uint32_t b = j; b + 1 < n_live; b += 32) {   // order-preserving removal from the list
            const uint32_t src = b + 1 + lane;
            const uint32_t v = src < n_live ? logs.live[src] : 0u;
            __syncwarp();
            if (src < n_live) logs.live[src - 1] = v;
            __syncwarp();
        }
        n_live--;
        if (lane == 0) {
            logs.removals[2 * n_removed] = step;
            logs.removals[2 * n_removed + 1] = key;
        }
        n_removed++;
        r_remove(t, s, key, lane);
    }
    r_store(t.ctl, s, lane);
    if (lane == 0) {
        vs->n_live = n_live;
        vs->n_removed = n_removed;
        vs->n_placed = n_placed;
        vs->step = step + 1;
        if (ahead) {   // the next step's state (its first round was generated alongside this commit)
            vs->n_free = 0;
            vs->rec_cost = ~0u;
            vs->best = ~0ull;
        }
    }
}

// ---------------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------------
void res_launch_init(const RTree& t, const float2* verts, const uint4* recs, const float2* pois, uint32_t n,
                     uint32_t n_slots, const uint32_t* kfree, uint32_t n_kfree, cudaStream_t s) {
    k_res_init<<<1, 32, 0, s>>>(t, verts, recs, pois, n, n_slots, kfree, n_kfree);
}
void res_launch_insert_placed(const RTree& t, const DItem* items, const float2* iverts, uint32_t n_items,
                              const uint32_t* q, uint32_t* out_key, cudaStream_t s) {
    k_res_insert_placed<<<1, 32, 0, s>>>(t, items, iverts, n_items, q, out_key);
}
void res_launch_remove(const RTree& t, const uint32_t* key, cudaStream_t s) { k_res_remove<<<1, 32, 0, s>>>(t, key); }
void res_launch_lbf_gen(const LbfParams& p, LbfDev* st, uint32_t* q, double* qu, uint32_t round, int n_sms,
                        cudaStream_t s, bool ahead, uint32_t slot) {
    const uint32_t n = round < p.uni_rounds ? p.n_uni : p.ls_cand;
    const uint32_t grid = std::min<uint32_t>((n + 255) / 256, (uint32_t)std::max(1, n_sms) * 4);
    // chained on the step's own stream; the next step's first round, drawn on a side stream while the
    // commit runs, is not (scheduled early it took SMs from the commit: build +0.9%)
    launch_chained(k_lbf_gen, dim3(grid), dim3(256), 0, s, !ahead, p, st, q, qu, round, ahead, slot);
}
void res_launch_gen_candidates(const unsigned long long* keys, const float (*bx)[4], uint32_t m, uint32_t n,
                               uint32_t item, const float2* orient, uint32_t n_orient, uint32_t* q, double* qu,
                               int n_sms, cudaStream_t s) {
    GenSegs g;
    for (uint32_t k = 0; k < m; k++) {
        g.key[k] = keys[k];
        g.box[k] = GenBox{bx[k][0], bx[k][2], std::nextafter(bx[k][2], bx[k][0]),
                          bx[k][1], bx[k][3], std::nextafter(bx[k][3], bx[k][1])};
    }
    const uint32_t per_seg = std::max<uint32_t>(1u, (uint32_t)std::max(1, n_sms) * 4 / m);
    const uint32_t gx = std::max<uint32_t>(1u, std::min<uint32_t>((n + 255) / 256, per_seg));
    k_gen_candidates<<<dim3(gx, m), 256, 0, s>>>(g, n, item, orient, n_orient, q, qu);
}
void res_launch_lbf_merge(LbfDev* st, const uint32_t* q, const double* qu, uint32_t round, cudaStream_t s) {
    launch_chained(k_lbf_merge, dim3(1), dim3(32), 0, s, true, st, q, qu, round);
}
void res_launch_lbf_commit(const RTree& t, const DItem* items, const float2* iverts, uint32_t n_items,
                           const LbfParams& p, LbfDev* st, const uint32_t* q, const double* qu, uint32_t round,
                           const uint8_t* verdicts, const LbfLogs& logs, cudaStream_t s, bool ahead) {
    launch_chained(k_lbf_commit, dim3(1), dim3(32), 0, s, true, t, items, iverts, n_items, p, st, q, qu, round,
                   verdicts, logs, ahead);
}

}  // namespace jcde
