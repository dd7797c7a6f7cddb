// jcde engine: C ABI (include/jcde.h), device mirror of the quadtree, kernel launches.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <list>
#include <mutex>
#include <string>
#include <thread>
#include <atomic>
#include <vector>

#include "../../include/jcde.h"
#include "kernels.cuh"
#include "resident.cuh"
#include "prep.hpp"
#include "qtree.hpp"

using namespace jcde;

namespace {

// Launch-shape defaults (jcde_tuning changes them per engine).
#ifndef JCDE_SURR_WARP_MAX
#define JCDE_SURR_WARP_MAX (1u << 17)
#endif
#ifndef JCDE_POLY_CHUNK
#define JCDE_POLY_CHUNK 2   // 0: large batches in grid-stride order
#endif
#ifndef JCDE_SURR_DYNAMIC
#define JCDE_SURR_DYNAMIC 1
#endif
#ifndef JCDE_COLLECT_DYNAMIC
#define JCDE_COLLECT_DYNAMIC 1
#endif
#ifndef JCDE_HOST_CHUNKS
#define JCDE_HOST_CHUNKS 1   // pipelined chunks of a large host batch (jcde_detect_batch_host)
#endif
#ifndef JCDE_ORDER_MIN_BATCH
#define JCDE_ORDER_MIN_BATCH 4096u
#endif

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    bool ensure(size_t bytes) {
        if (bytes <= cap) return true;
        if (p) cudaFree(p);
        p = nullptr;
        size_t want = std::max<size_t>(bytes, cap + cap / 2);
        want = (want + 255) & ~size_t(255);
        if (cudaMalloc(&p, want) != cudaSuccess) {
            cap = 0;
            p = nullptr;
            return false;
        }
        cap = want;
        return true;
    }
    template <class T>
    T* as() const { return reinterpret_cast<T*>(p); }
};

// One distinct filter: its ignored-key bitmask and per-node strongest presence on the device.
struct FilterSlot {
    std::vector<uint32_t> words;
    uint64_t version = ~0ull;   // tree version the strength array was computed for
    DevBuf d_mask, d_strength;
};

}  // namespace

struct jcde_snapshot {
    std::vector<HazardRec> dynamic_hazards;
};

struct jcde_engine {
    jcde_config cfg{};
    QuadTree tree;
    // items (shape_cd + surrogate) on the host
    std::vector<DItem> items;
    std::vector<float2> iverts;
    std::vector<float4> poles, piers;
    bool items_dirty = true;
    // device mirror
    uint64_t tree_version = ~0ull;
    FlatTree flat;
    std::vector<DHaz> haz;
    std::vector<float2> hverts;
    DevBuf d_nodes, d_nedges, d_strength0, d_entries, d_edges, d_cbox[EDGE_TILES], d_haz, d_hverts;
    DevBuf d_items, d_iverts, d_poles, d_piers;
    uint32_t n_nodes = 0;
    uint32_t level_end[MAX_STAGING_DEPTH + 1] = {};   // nodes of the top d + 1 levels, breadth-first
    // filters
    std::list<FilterSlot> filters;
    // staging for host entry points and single queries
    DevBuf d_q, d_out, d_raw, d_coll;
    DevBuf d_hist, d_order;   // spatial ordering of a query batch
    DevBuf d_next;            // work counters of the two passes (a pair per pipeline slot)
    DevBuf d_pend, d_pendc;   // undecided queries of the surrogate pass and their count (per pipeline slot)
    // hazard poles binned in a uniform grid (overlap proxy)
    uint64_t pole_version = ~0ull;
    DevBuf d_hpoles, d_hpstart, d_hpoles_c, d_hpstart_c;
    float hp_x0 = 0, hp_y0 = 0, hp_inv_cs = 0, hp_rmax = 0;
    int32_t hp_g = 1;
    float hp_inv_cs_c = 0;   // the coarse grid (cells 8x the pole-sized ones)
    int32_t hp_g_c = 1;
    uint32_t n_hpoles = 0;
    cudaStream_t last_stream = nullptr;
    bool have_last_stream = false;
    cudaStream_t own[2] = {nullptr, nullptr};
    cudaEvent_t ev_ready = nullptr;   // the host entry point's filter is ready (orders the second stream)
    int n_sms = 0;
    int detect_blocks_per_sm = 0, collect_blocks_per_sm = 0, tab_blocks_per_sm = 0, surr_blocks_per_sm = 0;
    // launch choices of the detect passes (jcde_set_tuning / jcde_autotune)
    jcde_tuning tune{JCDE_SURR_WARP_MAX, JCDE_SURR_WARP_MAX, (uint32_t)JCDE_POLY_CHUNK, JCDE_ORDER_MIN_BATCH,
                     (uint32_t)JCDE_SURR_GROUP, EDGE_TILE_DEFAULT, 0u};
    uint64_t launches = 0;
    // optional per-kernel timing (jcde_profile_enable): CUDA events around each launch
    bool prof = false;
    struct ProfMark { cudaEvent_t a, b; int kind; };
    std::vector<ProfMark> prof_open;
    std::vector<cudaEvent_t> prof_pool;
    double prof_ms[JCDE_PROF_KINDS] = {};
    uint64_t prof_n[JCDE_PROF_KINDS] = {};

    jcde_engine(const jcde_config& c, Box bbox) : cfg(c), tree(c.quadtree_depth, c.cd_threshold, bbox) {}
    ~jcde_engine() {
        for (auto& s : own)
            if (s) cudaStreamDestroy(s);
        if (ev_ready) cudaEventDestroy(ev_ready);
        for (auto& m : prof_open) {
            cudaEventDestroy(m.a);
            cudaEventDestroy(m.b);
        }
        for (auto ev : prof_pool) cudaEventDestroy(ev);
    }
};

#define CUDA_TRY(x)                                   \
    do {                                              \
        if ((x) != cudaSuccess) return JCDE_ERR_CUDA; \
    } while (0)

// Kernel timing: prof_begin/prof_end bracket one launch (or a group of launches of one kind) with a
// pair of events on the launch stream; jcde_profile_read folds finished pairs into totals.
static cudaEvent_t prof_event(jcde_engine* e) {
    if (!e->prof_pool.empty()) {
        cudaEvent_t ev = e->prof_pool.back();
        e->prof_pool.pop_back();
        return ev;
    }
    cudaEvent_t ev = nullptr;
    if (cudaEventCreate(&ev) != cudaSuccess) return nullptr;
    return ev;
}
static cudaEvent_t prof_begin(jcde_engine* e, cudaStream_t s) {
    if (!e->prof) return nullptr;
    cudaEvent_t a = prof_event(e);
    if (a) cudaEventRecord(a, s);
    return a;
}
static void prof_end(jcde_engine* e, cudaStream_t s, cudaEvent_t a, int kind) {
    if (!e->prof || !a) return;
    cudaEvent_t b = prof_event(e);
    if (!b) return;
    cudaEventRecord(b, s);
    e->prof_open.push_back({a, b, kind});
}

static jcde_status upload(DevBuf& b, const void* src, size_t bytes) {
    if (!b.ensure(std::max<size_t>(bytes, 16))) return JCDE_ERR_CUDA;
    if (bytes) CUDA_TRY(cudaMemcpy(b.p, src, bytes, cudaMemcpyHostToDevice));
    return JCDE_OK;
}

// Bring the device mirror up to date with the host quadtree and item table.  (The hazard-pole
// grids of the proxy kernels are refreshed separately, by sync_poles, only where they are used.)
static jcde_status noalloc_setup(void** out);

static jcde_status sync_device(jcde_engine* e) {
    if (e->tree_version == e->tree.version() && !e->items_dirty) return JCDE_OK;
    // the no-allocation entry point's set-up for this device, while allocating is still allowed
    // (its own status is reported by that entry point, which repeats the set-up if it failed here)
    (void)noalloc_setup(nullptr);
    // queries already queued on the caller's stream may still read the old image
    if (e->have_last_stream) CUDA_TRY(cudaStreamSynchronize(e->last_stream));
    if (e->tree_version != e->tree.version()) {
        e->tree.flatten(e->flat);
        e->haz.assign(e->tree.n_slots(), DHaz{});
        e->hverts.clear();
        const auto& hs = e->tree.hazards();
        for (uint32_t k = 0; k < hs.size(); k++) {
            if (!hs[k].alive) continue;
            const Polygon& s = hs[k].shape;
            DHaz& d = e->haz[k];
            d.box = s.bbox;
            d.poi_x = s.poi.c.x;
            d.poi_y = s.poi.c.y;
            d.v_off = (uint32_t)e->hverts.size();
            d.v_cnt_scope = (uint32_t)s.v.size() | (kind_is_exterior(hs[k].kind) ? 0x80000000u : 0u);
            for (const Pt& p : s.v) e->hverts.push_back(make_float2(p.x, p.y));
        }
        jcde_status st;
        if ((st = upload(e->d_nodes, e->flat.nodes.data(), e->flat.nodes.size() * sizeof(DNode)))) return st;
        if ((st = upload(e->d_nedges, e->flat.nedges.data(), e->flat.nedges.size() * 4))) return st;
        if ((st = upload(e->d_strength0, e->flat.strength.data(), e->flat.strength.size()))) return st;
        if ((st = upload(e->d_entries, e->flat.entries.data(), e->flat.entries.size() * sizeof(DEntry)))) return st;
        if ((st = upload(e->d_edges, e->flat.edges.data(), e->flat.edges.size() * 4))) return st;
        for (int t = 0; t < EDGE_TILES; t++)
            if ((st = upload(e->d_cbox[t], e->flat.cbox[t].data(), e->flat.cbox[t].size() * sizeof(Box)))) return st;
        if ((st = upload(e->d_haz, e->haz.data(), e->haz.size() * sizeof(DHaz)))) return st;
        if ((st = upload(e->d_hverts, e->hverts.data(), e->hverts.size() * sizeof(float2)))) return st;
        e->n_nodes = (uint32_t)e->flat.nodes.size();
        {   // breadth-first level boundaries: a level's children quartets follow it in order
            uint32_t a = 0, b = std::min<uint32_t>(1, e->n_nodes);
            for (uint32_t d = 0; d <= MAX_STAGING_DEPTH; d++) {
                e->level_end[d] = b;
                uint32_t internal = 0;
                for (uint32_t k = a; k < b; k++) internal += e->flat.nodes[k].child >= 0 ? 1u : 0u;
                a = b;
                b = std::min<uint32_t>(e->n_nodes, b + 4 * internal);
            }
        }
        e->tree_version = e->tree.version();
    }
    if (e->items_dirty) {
        jcde_status st;
        if ((st = upload(e->d_items, e->items.data(), e->items.size() * sizeof(DItem)))) return st;
        if ((st = upload(e->d_iverts, e->iverts.data(), e->iverts.size() * sizeof(float2)))) return st;
        if ((st = upload(e->d_poles, e->poles.data(), e->poles.size() * sizeof(float4)))) return st;
        if ((st = upload(e->d_piers, e->piers.data(), e->piers.size() * sizeof(float4)))) return st;
        e->items_dirty = false;
    }
    return JCDE_OK;
}

// The hazard-pole grids of the pole-overlap proxy (k_proxy, k_separate), rebuilt when the hazards
// or their poles changed since the last build.
static jcde_status sync_poles(jcde_engine* e) {
    if (e->pole_version == e->tree.pole_version()) return JCDE_OK;
    // proxy launches already queued on the caller's stream may still read the old grids
    if (e->have_last_stream) CUDA_TRY(cudaStreamSynchronize(e->last_stream));
    {
        // bin every live hazard pole into each grid cell its bounding box overlaps; a pair of poles
        // is then examined in one cell only, the one holding the low corner of their boxes' overlap
        const auto& hs = e->tree.hazards();
        const Box b = e->tree.bbox();
        std::vector<float> diam;
        float rmax = 0.0f;
        for (const HazardRec& h : hs)
            if (h.alive)
                for (const Disk& d : h.poles) {
                    diam.push_back(2.0f * d.r);
                    rmax = fmaxf(rmax, d.r);
                }
        const uint32_t np = (uint32_t)diam.size();
        const float ext = fmaxf(b.x1 - b.x0, b.y1 - b.y0);
        float typical = 0.0f;
        if (np) {   // cells about the size of a typical pole
            std::nth_element(diam.begin(), diam.begin() + diam.size() * 3 / 4, diam.end());
            typical = diam[diam.size() * 3 / 4];
        }
        const float cs = fmaxf(fmaxf(typical, ext / 1024.0f), 1e-6f);
        // a grid of cells of size `csz`: cell ranges and the poles binned into every cell they overlap
        auto build = [&](float csz, std::vector<uint32_t>& start, std::vector<float4>& hp, int32_t& g, float& inv) {
            g = std::max<int32_t>(1, std::min<int32_t>(1024, (int32_t)ceilf(ext / csz)));
            inv = (float)g / fmaxf(ext, 1e-6f);
            const int32_t gg = g;
            const float iv = inv;
            auto cix = [&](float x, float o) { return std::max(0, std::min(gg - 1, (int)floorf((x - o) * iv))); };
            start.assign((size_t)g * g + 1, 0u);
            auto for_cells = [&](const Disk& d, auto&& fn) {
                const int x0 = cix(d.c.x - d.r, b.x0), x1 = cix(d.c.x + d.r, b.x0);
                const int y0 = cix(d.c.y - d.r, b.y0), y1 = cix(d.c.y + d.r, b.y0);
                for (int iy = y0; iy <= y1; iy++)
                    for (int ix = x0; ix <= x1; ix++) fn((uint32_t)iy * (uint32_t)gg + (uint32_t)ix);
            };
            for (const HazardRec& h : hs)
                if (h.alive)
                    for (const Disk& d : h.poles) for_cells(d, [&](uint32_t c) { start[c + 1]++; });
            for (size_t c = 1; c < start.size(); c++) start[c] += start[c - 1];
            hp.assign(std::max<uint32_t>(start.back(), 1), make_float4(0.f, 0.f, 0.f, 0.f));
            std::vector<uint32_t> fill(start.begin(), start.end() - 1);
            for (uint32_t k = 0; k < hs.size(); k++)
                if (hs[k].alive)
                    for (const Disk& d : hs[k].poles) {
                        float kf;
                        std::memcpy(&kf, &k, 4);
                        for_cells(d, [&](uint32_t c) { hp[fill[c]++] = make_float4(d.c.x, d.c.y, d.r, kf); });
                    }
        };
        std::vector<uint32_t> start, start_c;
        std::vector<float4> hp, hp_c;
        int32_t g = 1, g_c = 1;
        float inv = 0.f, inv_c = 0.f;
        build(cs, start, hp, g, inv);          // pole-sized cells: pair lookups (k_proxy)
        build(8.0f * cs, start_c, hp_c, g_c, inv_c);   // coarse cells: a candidate's neighbourhood (k_separate)
        jcde_status st;
        if ((st = upload(e->d_hpoles, hp.data(), hp.size() * sizeof(float4)))) return st;
        if ((st = upload(e->d_hpstart, start.data(), start.size() * 4))) return st;
        if ((st = upload(e->d_hpoles_c, hp_c.data(), hp_c.size() * sizeof(float4)))) return st;
        if ((st = upload(e->d_hpstart_c, start_c.data(), start_c.size() * 4))) return st;
        e->hp_inv_cs_c = inv_c;
        e->hp_g_c = g_c;
        e->hp_x0 = b.x0;
        e->hp_y0 = b.y0;
        e->hp_inv_cs = inv;
        e->hp_rmax = rmax;
        e->hp_g = g;
        e->n_hpoles = np;
        e->pole_version = e->tree.pole_version();
    }
    return JCDE_OK;
}

static View base_view(const jcde_engine* e) {
    View v;
    v.nodes = e->d_nodes.as<DNode>();
    v.entries = e->d_entries.as<DEntry>();
    v.edges = e->d_edges.as<float4>();
    v.haz = e->d_haz.as<DHaz>();
    v.hverts = e->d_hverts.as<float2>();
    v.items = e->d_items.as<DItem>();
    v.iverts = e->d_iverts.as<float2>();
    v.poles = e->d_poles.as<float4>();
    v.piers = e->d_piers.as<float4>();
    v.strength = e->d_strength0.as<uint8_t>();
    v.mask = nullptr;
    v.nedges = e->d_nedges.as<uint32_t>();
    {   // the edge tile of the engine's launch choices: 4, 8 or 16 edges
        const int t = e->tune.edge_tile == 4 ? 0 : e->tune.edge_tile == 16 ? 2 : 1;
        v.cbox = e->d_cbox[t].as<float4>();
        v.eg_shift = (uint32_t)(2 + t);
    }
    v.cde = e->tree.bbox();
    v.coord_max = std::max(std::max(std::fabs(v.cde.x0), std::fabs(v.cde.x1)), std::max(std::fabs(v.cde.y0), std::fabs(v.cde.y1)));
    v.n_items = (uint32_t)e->items.size();
    v.n_slots = e->tree.n_slots();
    v.cd_threshold = e->cfg.cd_threshold;
    v.exterior = e->tree.exterior_key();
    v.hpoles = e->d_hpoles.as<float4>();
    v.hp_start = e->d_hpstart.as<uint32_t>();
    v.hp_x0 = e->hp_x0;
    v.hp_y0 = e->hp_y0;
    v.hp_inv_cs = e->hp_inv_cs;
    v.hp_rmax = e->hp_rmax;
    v.hp_g = e->hp_g;
    v.hpoles_c = e->d_hpoles_c.as<float4>();
    v.hp_start_c = e->d_hpstart_c.as<uint32_t>();
    v.hp_inv_cs_c = e->hp_inv_cs_c;
    v.hp_g_c = e->hp_g_c;
    return v;
}

static uint32_t mask_words(const jcde_engine* e) { return std::max<uint32_t>(1, (e->tree.n_slots() + 31) / 32); }

// Resolve a filter into the view: NoFilter uses the strength array built with the tree; any other
// filter gets a cached device bitmask and a strength array recomputed by k_strength when needed.
static jcde_status apply_filter(jcde_engine* e, const jcde_filter* f, cudaStream_t s, View& v) {
    if (!f || f->n_ignored == 0) return JCDE_OK;
    if (!f->ignored) return JCDE_ERR_ARG;
    const uint32_t W = mask_words(e);
    std::vector<uint32_t> words(W, 0u);
    for (uint32_t i = 0; i < f->n_ignored; i++) {
        uint32_t k = f->ignored[i];
        if (k < e->tree.n_slots()) words[k >> 5] |= 1u << (k & 31);   // unknown keys ignore nothing
    }
    FilterSlot* slot = nullptr;
    for (auto it = e->filters.begin(); it != e->filters.end(); ++it)
        if (it->words == words) {
            e->filters.splice(e->filters.begin(), e->filters, it);
            slot = &e->filters.front();
            break;
        }
    if (!slot) {
        if (e->filters.size() >= 8) {
            // the evicted slot may still be read by queued queries
            if (e->have_last_stream) CUDA_TRY(cudaStreamSynchronize(e->last_stream));
            e->filters.pop_back();
        }
        e->filters.emplace_front();
        slot = &e->filters.front();
        slot->words = words;
        if (!slot->d_mask.ensure(W * 4)) return JCDE_ERR_CUDA;
        CUDA_TRY(cudaMemcpy(slot->d_mask.p, words.data(), W * 4, cudaMemcpyHostToDevice));
    }
    v.mask = slot->d_mask.as<uint32_t>();
    if (slot->version != e->tree.version()) {
        if (!slot->d_strength.ensure(std::max<uint32_t>(e->n_nodes, 16))) return JCDE_ERR_CUDA;
        cudaEvent_t pa = prof_begin(e, s);
        k_strength<<<(e->n_nodes + 255) / 256, 256, 0, s>>>(v, e->n_nodes, slot->d_strength.as<uint8_t>());
        prof_end(e, s, pa, JCDE_PROF_FILTER);
        CUDA_TRY(cudaGetLastError());
        e->launches++;
        slot->version = e->tree.version();
    }
    v.strength = slot->d_strength.as<uint8_t>();
    return JCDE_OK;
}

static void init_launch_shape(jcde_engine* e) {
    if (e->n_sms) return;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&e->n_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e->cfg.quadtree_depth <= 8)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&e->detect_blocks_per_sm, k_poly<uint32_t, false>, POLY_WARPS * 32, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&e->detect_blocks_per_sm, k_poly<uint64_t, false>, POLY_WARPS * 32, 0);
    if (e->detect_blocks_per_sm < 1) e->detect_blocks_per_sm = 1;
    if (e->cfg.quadtree_depth <= 8)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&e->surr_blocks_per_sm, k_surrogate<uint32_t, false>, SURR_THREADS, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&e->surr_blocks_per_sm, k_surrogate<uint64_t, false>, SURR_THREADS, 0);
    if (e->surr_blocks_per_sm < 1) e->surr_blocks_per_sm = 1;
    // the small-batch polygon pass's leaf tables (dynamic shared memory) take its total above 48 KB
    const int tab_smem = (int)(POLY_WARPS * sizeof(LeafTab));
    cudaFuncSetAttribute(k_poly_tab<uint32_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, tab_smem);
    cudaFuncSetAttribute(k_poly_tab<uint64_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, tab_smem);
    if (e->cfg.quadtree_depth <= 8)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&e->tab_blocks_per_sm, k_poly_tab<uint32_t>, POLY_WARPS * 32, tab_smem);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&e->tab_blocks_per_sm, k_poly_tab<uint64_t>, POLY_WARPS * 32, tab_smem);
    if (e->tab_blocks_per_sm < 1) e->tab_blocks_per_sm = 1;
    if (e->n_sms < 1) e->n_sms = 1;
}

#ifndef JCDE_SPATIAL_ORDER
#define JCDE_SPATIAL_ORDER 1
#endif
static constexpr size_t STAGE_MAX_BYTES = 8192;   // shared memory the polygon pass may use for staged nodes


// Visit order of a batch: cell-by-cell over the CDE box (k_bucket_*), or nullptr for index order.
// `slot` selects one of two histogram/order buffer pairs, so that the two streams of the host
// entry point's pipeline never share one; `slot_cap` is the largest batch a slot must hold.
static const uint32_t* spatial_order_into(jcde_engine* e, const uint32_t* q, uint32_t n, cudaStream_t s,
                                          uint32_t* hist, uint32_t* order);
static const uint32_t* spatial_order(jcde_engine* e, const uint32_t* q, uint32_t n, cudaStream_t s, int slot,
                                     uint32_t slot_cap) {
    if (!JCDE_SPATIAL_ORDER || n < e->tune.order_min_batch) return nullptr;
    const size_t per_slot = std::max<size_t>(n, slot_cap);
    if (!e->d_hist.ensure(2 * ORDER_HIST_WORDS * 4)) return nullptr;
    if (e->d_order.cap < 2 * per_slot * 4) {
        // growing the buffer frees the old one, which queued batches may still read
        if (e->have_last_stream && cudaStreamSynchronize(e->last_stream) != cudaSuccess) return nullptr;
        if (!e->d_order.ensure(2 * per_slot * 4)) return nullptr;
    }
    uint32_t* hist = e->d_hist.as<uint32_t>() + (size_t)slot * ORDER_HIST_WORDS;
    uint32_t* order = e->d_order.as<uint32_t>() + (size_t)slot * (e->d_order.cap / 8);
    return spatial_order_into(e, q, n, s, hist, order);
}

// The ordering kernels over caller-owned buffers: hist of ORDER_HIST_WORDS words, order of n words.
static const uint32_t* spatial_order_into(jcde_engine* e, const uint32_t* q, uint32_t n, cudaStream_t s,
                                          uint32_t* hist, uint32_t* order) {
    if (cudaMemsetAsync(hist, 0, ORDER_HIST_WORDS * 4, s) != cudaSuccess) return nullptr;
    const Box b = e->tree.bbox();
    const uint32_t tiles = (uint32_t)((n + (size_t)ORDER_TILE - 1) / ORDER_TILE);
    const uint32_t grid = std::min<uint32_t>(tiles, (uint32_t)e->n_sms * 2);
    if (ORDER_SMEM > 48 * 1024) {
        static bool attr_set = false;
        if (!attr_set) {
            if (cudaFuncSetAttribute(k_order_count, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ORDER_SMEM) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_order_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ORDER_SMEM) !=
                    cudaSuccess)
                return nullptr;
            attr_set = true;
        }
    }
    cudaEvent_t pa = prof_begin(e, s);
    k_order_count<<<grid, ORDER_THREADS, ORDER_SMEM, s>>>(q, n, b, hist);
    k_order_scatter<<<grid, ORDER_THREADS, ORDER_SMEM, s>>>(q, n, b, hist, order);
    prof_end(e, s, pa, JCDE_PROF_ORDER);
    e->launches += 2;
    return order;
}

// The surrogate pass and/or the polygon pass; the walk's pending masks are 32-bit for trees of
// depth <= 8 and 64-bit above.  Batches of at most JCDE_SURR_WARP_MAX queries take the
// warp-per-query surrogate pass.

// With `n_pending`, the surrogate pass counts the queries it leaves to the polygon pass; with `best`
// the small-batch polygon pass makes the LBF choice, and with `skip` it leaves unjudged the queries
// that can no longer win it.
template <typename PendT>
static bool launch_passes_t(jcde_engine* e, const View& v, const uint32_t* q, uint32_t n, uint8_t* dout,
                            cudaStream_t s, RawShape raw, int mode, const uint32_t* order, uint32_t* next,
                            unsigned long long* best, uint32_t* n_pending, bool skip, PendList pend) {
    bool chose = false;
    // the compacted list of undecided queries serves the large-batch passes of a full detect only
    const bool large = n > e->tune.surrogate_warp_max && n > e->tune.leaf_table_max;
    if (!(mode == 3 && large && next && JCDE_SURR_DYNAMIC && e->tune.poly_chunk && !raw.verts && !n_pending) ||
        (pend.rec && cudaMemsetAsync(pend.count, 0, 4, s) != cudaSuccess))
        pend = PendList{nullptr, nullptr};
    // the small-batch polygon pass's counter, cleared by the warp surrogate pass when both run here
    bool poly_counter_zeroed = false;
    if (mode & 1) {
        const uint8_t miss = mode == 1 ? (uint8_t)0 : PENDING;
        cudaEvent_t pa = prof_begin(e, s);
        if (n <= e->tune.surrogate_warp_max) {   // too few queries to fill the GPU one thread each
            const uint32_t lanes = e->tune.surrogate_lanes;
            const uint32_t gpb = SURR_THREADS / lanes;   // query groups per block
            const uint32_t grid = std::min<uint32_t>((n + gpb - 1) / gpb, (uint32_t)e->n_sms * 8);
            uint32_t* zero = (mode & 2) && next && n <= e->tune.leaf_table_max ? next + 1 : nullptr;
            poly_counter_zeroed = zero != nullptr;
            // a chained launch: scheduled while the kernel before it (the LBF commit, in a build) ends
            auto kern = lanes == 8 ? k_surrogate_warp<PendT, 8>
                        : lanes == 16 ? k_surrogate_warp<PendT, 16> : k_surrogate_warp<PendT, 32>;
            launch_chained(kern, dim3(grid), dim3(SURR_THREADS), 0, s, true, v, q, n, dout, miss, order, n_pending,
                           zero);
        } else if (JCDE_SURR_DYNAMIC && next && cudaMemsetAsync(next, 0, 4, s) == cudaSuccess) {
            // persistent blocks; each warp takes the next 32 queries from a counter as it finishes
            const uint32_t grid = std::min<uint32_t>((n + SURR_THREADS - 1) / SURR_THREADS,
                                                     (uint32_t)e->n_sms * (uint32_t)e->surr_blocks_per_sm);
            k_surrogate<PendT, false><<<grid, SURR_THREADS, 0, s>>>(v, MultiSrc{}, q, n, dout, miss, order, next,
                                                                    n_pending, pend);
        } else {
            const uint32_t grid = (n + SURR_THREADS - 1) / SURR_THREADS;
            k_surrogate<PendT, false><<<grid, SURR_THREADS, 0, s>>>(v, MultiSrc{}, q, n, dout, miss, order, nullptr,
                                                                    n_pending);
            pend = PendList{nullptr, nullptr};   // this branch writes no list: the polygon pass reads the slots
        }
        prof_end(e, s, pa, JCDE_PROF_SURROGATE);
        e->launches++;
    }
    if (mode & 2) {
        const uint32_t want = (n + POLY_WARPS - 1) / POLY_WARPS;
        uint32_t grid = std::min<uint32_t>(want, (uint32_t)(e->n_sms * e->detect_blocks_per_sm));
        cudaEvent_t pa = prof_begin(e, s);
        // Queries are handed to warps from a counter (`next`), so that no warp queues behind slow
        // queries: one at a time in small batches, JCDE_POLY_CHUNK at a time in large ones.  Small
        // batches are latency-bound and also build per-query leaf tables.
        const bool tab = n <= e->tune.leaf_table_max;
        if (next) next += 1;   // the polygon pass's own counter
        if (!next || (!tab && !e->tune.poly_chunk) ||
            (!(tab && poly_counter_zeroed) && cudaMemsetAsync(next, 0, 4, s) != cudaSuccess))
            next = nullptr;
        if (tab) {
            grid = std::min<uint32_t>(want, (uint32_t)(e->n_sms * e->tab_blocks_per_sm));
            launch_chained(k_poly_tab<PendT>, dim3(grid), dim3(POLY_WARPS * 32), POLY_WARPS * sizeof(LeafTab), s, true,
                           v, q, n, dout, raw, mode == 3, order, next, best, skip);
            chose = best != nullptr;
        } else {
            // the top staging_depth levels of the tree in shared memory (at most STAGE_MAX_BYTES)
            uint32_t staged = e->tune.staging_depth ? e->level_end[e->tune.staging_depth - 1] : 0u;
            while (staged && (size_t)staged * (sizeof(DNode) + 1) > STAGE_MAX_BYTES) staged /= 4;
            if (staged) {
                View vs = v;
                vs.n_staged = staged;
                const size_t smem = ((size_t)staged * (sizeof(DNode) + 1) + 15) & ~size_t(15);
                k_poly<PendT, false, true><<<grid, POLY_WARPS * 32, smem, s>>>(
                    vs, MultiSrc{}, q, n, dout, raw, mode == 3, order, next, std::max(e->tune.poly_chunk, 1u), pend.rec,
                    pend.count);
            } else {
                k_poly<PendT, false><<<grid, POLY_WARPS * 32, 0, s>>>(v, MultiSrc{}, q, n, dout, raw, mode == 3, order,
                                                                      next, std::max(e->tune.poly_chunk, 1u), pend.rec,
                                                                      pend.count);
            }
        }
        prof_end(e, s, pa, JCDE_PROF_POLY);
        e->launches++;
    }
    return chose;
}
// Returns true when the polygon pass also made the LBF choice into `best` (which it does for
// batches that take the small-batch kernel; callers launch k_lbf_select otherwise).
static bool launch_passes(jcde_engine* e, const View& v, const uint32_t* q, uint32_t n, uint8_t* dout,
                          cudaStream_t s, RawShape raw, int mode, const uint32_t* order = nullptr,
                          uint32_t* next = nullptr, unsigned long long* best = nullptr, uint32_t* n_pending = nullptr,
                          bool skip = false, PendList pend = PendList{nullptr, nullptr}) {
    if (e->cfg.quadtree_depth <= 8)
        return launch_passes_t<uint32_t>(e, v, q, n, dout, s, raw, mode, order, next, best, n_pending, skip, pend);
    return launch_passes_t<uint64_t>(e, v, q, n, dout, s, raw, mode, order, next, best, n_pending, skip, pend);
}

// The pending-list buffers of pipeline slot `slot` for a batch of n (records of PEND_WORDS words),
// or an empty list when they cannot be had (the passes then run without it).
static PendList pend_list(jcde_engine* e, uint32_t n, int slot, uint32_t slot_cap) {
    const size_t per_slot = std::max<size_t>(n, slot_cap) * PEND_WORDS * 4;
    if (!e->d_pendc.ensure(2 * 4)) return PendList{nullptr, nullptr};
    if (e->d_pend.cap < 2 * per_slot) {
        // growing the buffer frees the old one, which queued batches may still read
        if (e->have_last_stream && cudaStreamSynchronize(e->last_stream) != cudaSuccess) return PendList{nullptr, nullptr};
        if (!e->d_pend.ensure(2 * per_slot)) return PendList{nullptr, nullptr};
    }
    return PendList{e->d_pend.as<uint32_t>() + (size_t)slot * (e->d_pend.cap / 8), e->d_pendc.as<uint32_t>() + slot};
}

// mode 1: surrogate only; 2: polygon only; 3: surrogate pass, then the polygon pass on the
// queries it left undecided (the order of lbf/benches/ci_bench.rs:111-119).
static jcde_status launch_detect(jcde_engine* e, int mode, const jcde_query* dq, uint32_t n, const jcde_filter* f,
                                 uint8_t* dout, cudaStream_t s, RawShape raw, int slot = 0, uint32_t slot_cap = 0) {
    jcde_status st = sync_device(e);
    if (st) return st;
    init_launch_shape(e);
    View v = base_view(e);
    if ((st = apply_filter(e, f, s, v))) return st;
    if (n == 0) return JCDE_OK;
    const uint32_t* q = reinterpret_cast<const uint32_t*>(dq);
    const uint32_t* order = raw.verts ? nullptr : spatial_order(e, q, n, s, slot, slot_cap);
    uint32_t* next = e->d_next.ensure(2 * 2 * 4) ? e->d_next.as<uint32_t>() + 2 * slot : nullptr;
    const PendList pend = (mode == 3 && !raw.verts && n > e->tune.surrogate_warp_max && n > e->tune.leaf_table_max)
                              ? pend_list(e, n, slot, slot_cap)
                              : PendList{nullptr, nullptr};
    launch_passes(e, v, q, n, dout, s, raw, mode, order, next, nullptr, nullptr, false, pend);
    CUDA_TRY(cudaGetLastError());
    e->last_stream = s;
    e->have_last_stream = true;
    return JCDE_OK;
}

static jcde_status launch_collect(jcde_engine* e, int mode, const jcde_query* dq, uint32_t n, const jcde_filter* f,
                                  uint32_t* d_off, uint32_t* d_cnt, uint32_t* d_ids, uint32_t cap, uint32_t* d_total,
                                  cudaStream_t s, RawShape raw) {
    jcde_status st = sync_device(e);
    if (st) return st;
    init_launch_shape(e);
    View v = base_view(e);
    if ((st = apply_filter(e, f, s, v))) return st;
    CUDA_TRY(cudaMemsetAsync(d_total, 0, 4, s));
    if (n == 0) return JCDE_OK;
    const uint32_t words = mask_words(e);
    // per warp: the key bitset and the item's transformed vertices
    const size_t smem = (size_t)COLLECT_WARPS * (words * 4 + POLY_MAXV * sizeof(float2));
    if (smem > 200 * 1024) return JCDE_ERR_CAPACITY;   // > ~1.5M hazard slots
    const bool wide = e->cfg.quadtree_depth > 8;   // 64-bit walk masks above depth 8
    static bool attr_set[2][4] = {};
    const void* fn = wide ? (mode == 1 ? (const void*)k_collect<1, uint64_t> : mode == 2 ? (const void*)k_collect<2, uint64_t>
                                                                                     : (const void*)k_collect<3, uint64_t>)
                          : (mode == 1 ? (const void*)k_collect<1, uint32_t> : mode == 2 ? (const void*)k_collect<2, uint32_t>
                                                                                     : (const void*)k_collect<3, uint32_t>);
    if (smem > 48 * 1024 && !attr_set[wide][mode]) {
        CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        attr_set[wide][mode] = true;
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, COLLECT_WARPS * 32, smem);
    if (per_sm < 1) per_sm = 1;
    uint32_t want = (n + COLLECT_WARPS - 1) / COLLECT_WARPS;
    uint32_t grid = std::min<uint32_t>(want, (uint32_t)(e->n_sms * per_sm));
    const uint32_t* q = reinterpret_cast<const uint32_t*>(dq);
    // the detect passes' visit order and work counter (slot 0)
    const uint32_t* order = raw.verts ? nullptr : spatial_order(e, q, n, s, 0, 0);
    uint32_t* next = nullptr;
    if (JCDE_COLLECT_DYNAMIC && e->d_next.ensure(2 * 2 * 4) && cudaMemsetAsync(e->d_next.p, 0, 4, s) == cudaSuccess)
        next = e->d_next.as<uint32_t>();
    cudaEvent_t pa = prof_begin(e, s);
    using K = void (*)(View, const uint32_t*, uint32_t, uint32_t, uint32_t*, uint32_t*, uint32_t*, uint32_t, uint32_t*,
                       RawShape, const uint32_t*, uint32_t*);
    const K k = reinterpret_cast<K>(const_cast<void*>(fn));
    k<<<grid, COLLECT_WARPS * 32, smem, s>>>(v, q, n, words, d_off, d_cnt, d_ids, cap, d_total, raw, order, next);
    CUDA_TRY(cudaGetLastError());
    prof_end(e, s, pa, JCDE_PROF_COLLECT);
    e->launches++;
    e->last_stream = s;
    e->have_last_stream = true;
    return JCDE_OK;
}

static bool valid_config(const jcde_config* c) {
    return c && c->quadtree_depth <= MAX_DEPTH && c->n_pole_limits <= 3;
}

static jcde_status make_hazard(const jcde_hazard* h, HazardRec& r) {
    if (!h || !h->xy || h->n_vertices < 3) return JCDE_ERR_ARG;
    if (h->kind < 0 || h->kind > 3) return JCDE_ERR_ARG;
    r.kind = h->kind;
    r.dynamic = h->dynamic != 0;
    r.tag = h->tag;
    r.shape.v.resize(h->n_vertices);
    for (uint32_t i = 0; i < h->n_vertices; i++) r.shape.v[i] = Pt{h->xy[2 * i], h->xy[2 * i + 1]};
    r.shape.poi = Disk{Pt{h->poi[0], h->poi[1]}, h->poi[2]};
    return JCDE_OK;
}

extern "C" {

const char* jcde_status_string(jcde_status s) {
    switch (s) {
        case JCDE_OK: return "ok";
        case JCDE_ERR_ARG: return "invalid argument";
        case JCDE_ERR_CUDA: return "CUDA runtime error";
        case JCDE_ERR_CAPACITY: return "output capacity exceeded";
        case JCDE_ERR_NOT_FOUND: return "not found";
        case JCDE_ERR_TIMEOUT: return "device wait timed out";
        case JCDE_ERR_STATE: return "invalid engine state";
        default: return "unknown status";
    }
}

void jcde_default_config(jcde_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->quadtree_depth = 5;
    c->cd_threshold = 16;
    c->n_pole_limits = 3;
    c->pole_limit_n[0] = 100; c->pole_limit_coverage[0] = 0.0f;
    c->pole_limit_n[1] = 20;  c->pole_limit_coverage[1] = 0.75f;
    c->pole_limit_n[2] = 10;  c->pole_limit_coverage[2] = 0.90f;
    c->n_ff_poles = 2;
    c->n_ff_piers = 0;
}

jcde_status jcde_create(const jcde_config* cfg, jcde_rect bbox, const jcde_hazard* hs, uint32_t n, jcde_engine** out) {
    if (!out || !valid_config(cfg) || (n && !hs)) return JCDE_ERR_ARG;
    if (!(bbox.x_min < bbox.x_max && bbox.y_min < bbox.y_max)) return JCDE_ERR_ARG;
    *out = nullptr;
    jcde_engine* e = new (std::nothrow) jcde_engine(*cfg, Box{bbox.x_min, bbox.y_min, bbox.x_max, bbox.y_max});
    if (!e) return JCDE_ERR_CUDA;
    for (uint32_t i = 0; i < n; i++) {
        HazardRec r;
        if (make_hazard(&hs[i], r)) {
            delete e;
            return JCDE_ERR_ARG;
        }
        e->tree.insert(std::move(r));
    }
    *out = e;
    return JCDE_OK;
}

void jcde_destroy(jcde_engine* e) {
    if (!e) return;
    if (e->have_last_stream) cudaStreamSynchronize(e->last_stream);
    delete e;
}

jcde_status jcde_bbox(const jcde_engine* e, jcde_rect* out) {
    if (!e || !out) return JCDE_ERR_ARG;
    Box b = e->tree.bbox();
    *out = jcde_rect{b.x0, b.y0, b.x1, b.y1};
    return JCDE_OK;
}

jcde_status jcde_register_hazard(jcde_engine* e, const jcde_hazard* h, uint32_t* out_key) {
    if (!e) return JCDE_ERR_ARG;
    HazardRec r;
    jcde_status st = make_hazard(h, r);
    if (st) return st;
    uint32_t k = e->tree.insert(std::move(r));
    if (out_key) *out_key = k;
    return JCDE_OK;
}

jcde_status jcde_deregister_hazard(jcde_engine* e, uint32_t key) {
    if (!e) return JCDE_ERR_ARG;
    return e->tree.remove(key) ? JCDE_OK : JCDE_ERR_NOT_FOUND;
}

jcde_status jcde_deregister_hazard_by_entity(jcde_engine* e, int32_t kind, uint64_t tag, uint32_t* out_key) {
    if (!e) return JCDE_ERR_ARG;
    const auto& hs = e->tree.hazards();
    for (uint32_t k = 0; k < hs.size(); k++)
        if (hs[k].alive && hs[k].kind == kind && hs[k].tag == tag) {
            e->tree.remove(k);
            if (out_key) *out_key = k;
            return JCDE_OK;
        }
    return JCDE_ERR_NOT_FOUND;
}

jcde_status jcde_n_hazard_slots(const jcde_engine* e, uint32_t* out) {
    if (!e || !out) return JCDE_ERR_ARG;
    *out = e->tree.n_slots();
    return JCDE_OK;
}

jcde_status jcde_register_item(jcde_engine* e, const float* xy, uint32_t nv, const float poi[3], const float* poles,
                               uint32_t n_poles, const float* piers, uint32_t n_piers, uint32_t* out_item) {
    if (!e || !xy || nv < 3 || !poi || (n_poles && !poles) || (n_piers && !piers)) return JCDE_ERR_ARG;
    DItem it{};
    it.v_off = (uint32_t)e->iverts.size();
    it.v_cnt = nv;
    it.pole_off = (uint32_t)e->poles.size();
    it.n_ff_poles = std::min<uint32_t>(e->cfg.n_ff_poles, n_poles);   // SPSurrogate::ff_poles (sp_surrogate.rs:55-57)
    it.pier_off = (uint32_t)e->piers.size();
    it.n_piers = n_piers;
    it.poi_x = poi[0];
    it.poi_y = poi[1];
    it.n_poles = n_poles;
    it.pole_r2max = 0.0f;
    it.pole_bound = 0.0f;
    for (uint32_t i = 0; i < n_poles; i++) {
        const float d2 = poles[3 * i] * poles[3 * i] + poles[3 * i + 1] * poles[3 * i + 1];
        it.pole_r2max = std::max(it.pole_r2max, d2);
        it.pole_bound = std::max(it.pole_bound, sqrtf(d2) + poles[3 * i + 2]);
    }
    for (uint32_t i = 0; i < nv; i++) e->iverts.push_back(make_float2(xy[2 * i], xy[2 * i + 1]));
    for (uint32_t i = 0; i < n_poles; i++) e->poles.push_back(make_float4(poles[3 * i], poles[3 * i + 1], poles[3 * i + 2], 0.0f));
    for (uint32_t i = 0; i < n_piers; i++)
        e->piers.push_back(make_float4(piers[4 * i], piers[4 * i + 1], piers[4 * i + 2], piers[4 * i + 3]));
    e->items.push_back(it);
    e->items_dirty = true;
    if (out_item) *out_item = (uint32_t)e->items.size() - 1;
    return JCDE_OK;
}

jcde_status jcde_detect_batch(jcde_engine* e, const jcde_query* dq, uint32_t n, const jcde_filter* f, uint8_t* dout,
                              void* stream) {
    if (!e || (n && (!dq || !dout))) return JCDE_ERR_ARG;
    return launch_detect(e, 3, dq, n, f, dout, (cudaStream_t)stream, RawShape{nullptr, 0, 0, 0, 0});
}
jcde_status jcde_detect_surrogate_batch(jcde_engine* e, const jcde_query* dq, uint32_t n, const jcde_filter* f,
                                        uint8_t* dout, void* stream) {
    if (!e || (n && (!dq || !dout))) return JCDE_ERR_ARG;
    return launch_detect(e, 1, dq, n, f, dout, (cudaStream_t)stream, RawShape{nullptr, 0, 0, 0, 0});
}
jcde_status jcde_detect_poly_batch(jcde_engine* e, const jcde_query* dq, uint32_t n, const jcde_filter* f,
                                   uint8_t* dout, void* stream) {
    if (!e || (n && (!dq || !dout))) return JCDE_ERR_ARG;
    return launch_detect(e, 2, dq, n, f, dout, (cudaStream_t)stream, RawShape{nullptr, 0, 0, 0, 0});
}

jcde_status jcde_detect_batch_host(jcde_engine* e, const jcde_query* hq, uint32_t n, const jcde_filter* f,
                                   uint8_t* hout) {
    if (!e || (n && (!hq || !hout))) return JCDE_ERR_ARG;
    if (n == 0) return JCDE_OK;
    for (auto& s : e->own)
        if (!s) CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    if (!e->d_q.ensure((size_t)n * sizeof(jcde_query)) || !e->d_out.ensure(n)) return JCDE_ERR_CUDA;
    const uint32_t n_chunks = n >= (1u << 18) ? (uint32_t)JCDE_HOST_CHUNKS : 1u;
    if (n_chunks == 1) {
        // The whole batch in one stream.  The copy is queued first, so that the engine's device image
        // and the filter are resolved on the host while it runs.  (On GB300 the copy of a 1M batch
        // takes ~8% of its kernels' time; splitting the batch into chunks whose copies overlap the
        // other chunk's kernels costs more in per-batch kernel overhead than it hides.)
        cudaStream_t s = e->own[0];
        CUDA_TRY(cudaMemcpyAsync(e->d_q.p, hq, (size_t)n * sizeof(jcde_query), cudaMemcpyHostToDevice, s));
        jcde_status st = launch_detect(e, 3, e->d_q.as<jcde_query>(), n, f, e->d_out.as<uint8_t>(), s,
                                       RawShape{nullptr, 0, 0, 0, 0});
        if (!st) st = cudaMemcpyAsync(hout, e->d_out.p, n, cudaMemcpyDeviceToHost, s) == cudaSuccess ? JCDE_OK
                                                                                                 : JCDE_ERR_CUDA;
        const bool synced = cudaStreamSynchronize(s) == cudaSuccess;
        e->have_last_stream = false;
        return st ? st : (synced ? JCDE_OK : JCDE_ERR_CUDA);
    }
    jcde_status st = sync_device(e);
    if (st) return st;
    // resolve the filter once, on the first stream, before the pipelined chunks (the second stream
    // waits for it on the device)
    View probe = base_view(e);
    if ((st = apply_filter(e, f, e->own[0], probe))) return st;
    if (!e->ev_ready) CUDA_TRY(cudaEventCreateWithFlags(&e->ev_ready, cudaEventDisableTiming));
    CUDA_TRY(cudaEventRecord(e->ev_ready, e->own[0]));
    CUDA_TRY(cudaStreamWaitEvent(e->own[1], e->ev_ready, 0));
    // chunks alternate between two streams so that copies overlap the other chunk's kernels
    const uint32_t chunk = (n + n_chunks - 1) / n_chunks;
    jcde_query* dq = e->d_q.as<jcde_query>();
    uint8_t* dout = e->d_out.as<uint8_t>();
    for (uint32_t c = 0; c < n_chunks; c++) {
        uint32_t a = c * chunk, b = std::min<uint32_t>(n, a + chunk);
        if (a >= b) break;
        cudaStream_t s = e->own[c & 1];
        CUDA_TRY(cudaMemcpyAsync(dq + a, hq + a, (size_t)(b - a) * sizeof(jcde_query), cudaMemcpyHostToDevice, s));
        if ((st = launch_detect(e, 3, dq + a, b - a, f, dout + a, s, RawShape{nullptr, 0, 0, 0, 0}, (int)(c & 1), chunk)))
            return st;
        CUDA_TRY(cudaMemcpyAsync(hout + a, dout + a, b - a, cudaMemcpyDeviceToHost, s));
    }
    CUDA_TRY(cudaStreamSynchronize(e->own[0]));
    CUDA_TRY(cudaStreamSynchronize(e->own[1]));
    e->have_last_stream = false;
    return JCDE_OK;
}

jcde_status jcde_collect_batch(jcde_engine* e, const jcde_query* dq, uint32_t n, const jcde_filter* f, uint32_t* d_off,
                               uint32_t* d_cnt, uint32_t* d_ids, uint32_t cap, uint32_t* d_total, void* stream) {
    if (!e || !d_total || (n && (!dq || !d_off || !d_cnt)) || (cap && !d_ids)) return JCDE_ERR_ARG;
    return launch_collect(e, 3, dq, n, f, d_off, d_cnt, d_ids, cap, d_total, (cudaStream_t)stream,
                          RawShape{nullptr, 0, 0, 0, 0});
}

static jcde_status single_detect(jcde_engine* e, int mode, const jcde_query* hq, const float* xy, uint32_t nv,
                                 const float* poi, const jcde_filter* f, uint8_t* out) {
    if (!e->d_q.ensure(sizeof(jcde_query)) || !e->d_out.ensure(16)) return JCDE_ERR_CUDA;
    RawShape raw{nullptr, 0, 0, 0, 0};
    if (xy) {
        if (!e->d_raw.ensure((size_t)nv * 8)) return JCDE_ERR_CUDA;
        CUDA_TRY(cudaMemcpy(e->d_raw.p, xy, (size_t)nv * 8, cudaMemcpyHostToDevice));
        raw = RawShape{e->d_raw.as<float2>(), nv, poi[0], poi[1], poi[2]};
    } else {
        CUDA_TRY(cudaMemcpy(e->d_q.p, hq, sizeof(jcde_query), cudaMemcpyHostToDevice));
    }
    jcde_status st = launch_detect(e, mode, e->d_q.as<jcde_query>(), 1, f, e->d_out.as<uint8_t>(), 0, raw);
    if (st) return st;
    uint8_t v = 0;
    CUDA_TRY(cudaMemcpy(&v, e->d_out.p, 1, cudaMemcpyDeviceToHost));
    *out = v;
    return JCDE_OK;
}

jcde_status jcde_detect_poly(jcde_engine* e, const float* xy, uint32_t nv, const float poi[3], const jcde_filter* f,
                             uint8_t* out) {
    if (!e || !xy || nv < 3 || !poi || !out) return JCDE_ERR_ARG;
    return single_detect(e, 2, nullptr, xy, nv, poi, f, out);
}

jcde_status jcde_detect_surrogate(jcde_engine* e, uint32_t item, const float t[4], const jcde_filter* f, uint8_t* out) {
    if (!e || !t || !out) return JCDE_ERR_ARG;
    if (item >= e->items.size()) return JCDE_ERR_NOT_FOUND;
    jcde_query q{item, t[0], t[1], t[2], t[3]};
    return single_detect(e, 1, &q, nullptr, 0, nullptr, f, out);
}

static jcde_status single_collect(jcde_engine* e, int mode, const jcde_query* hq, const float* xy, uint32_t nv,
                                  const float* poi, const jcde_filter* f, uint32_t* keys, uint32_t cap, uint32_t* n_out) {
    const uint32_t slots = std::max<uint32_t>(1, e->tree.n_slots());
    if (!e->d_q.ensure(sizeof(jcde_query)) || !e->d_coll.ensure((size_t)(3 + slots) * 4)) return JCDE_ERR_CUDA;
    RawShape raw{nullptr, 0, 0, 0, 0};
    if (xy) {
        if (!e->d_raw.ensure((size_t)nv * 8)) return JCDE_ERR_CUDA;
        CUDA_TRY(cudaMemcpy(e->d_raw.p, xy, (size_t)nv * 8, cudaMemcpyHostToDevice));
        raw = RawShape{e->d_raw.as<float2>(), nv, poi[0], poi[1], poi[2]};
    } else {
        CUDA_TRY(cudaMemcpy(e->d_q.p, hq, sizeof(jcde_query), cudaMemcpyHostToDevice));
    }
    uint32_t* c = e->d_coll.as<uint32_t>();
    jcde_status st = launch_collect(e, mode, e->d_q.as<jcde_query>(), 1, f, c, c + 1, c + 3, slots, c + 2, 0, raw);
    if (st) return st;
    std::vector<uint32_t> h(3 + slots);
    CUDA_TRY(cudaMemcpy(h.data(), c, h.size() * 4, cudaMemcpyDeviceToHost));
    const uint32_t cnt = h[1];
    *n_out = cnt;
    if (cnt > cap) return JCDE_ERR_CAPACITY;
    for (uint32_t i = 0; i < cnt; i++) keys[i] = h[3 + h[0] + i];
    return JCDE_OK;
}

jcde_status jcde_collect_poly(jcde_engine* e, const float* xy, uint32_t nv, const float poi[3], const jcde_filter* f,
                              uint32_t* keys, uint32_t cap, uint32_t* n_out) {
    if (!e || !xy || nv < 3 || !poi || !n_out || (cap && !keys)) return JCDE_ERR_ARG;
    return single_collect(e, 2, nullptr, xy, nv, poi, f, keys, cap, n_out);
}

jcde_status jcde_collect_surrogate(jcde_engine* e, uint32_t item, const float t[4], const jcde_filter* f, uint32_t* keys,
                                   uint32_t cap, uint32_t* n_out) {
    if (!e || !t || !n_out || (cap && !keys)) return JCDE_ERR_ARG;
    if (item >= e->items.size()) return JCDE_ERR_NOT_FOUND;
    jcde_query q{item, t[0], t[1], t[2], t[3]};
    return single_collect(e, 1, &q, nullptr, 0, nullptr, f, keys, cap, n_out);
}

jcde_status jcde_save(const jcde_engine* e, jcde_snapshot** out) {
    if (!e || !out) return JCDE_ERR_ARG;
    jcde_snapshot* s = new (std::nothrow) jcde_snapshot();
    if (!s) return JCDE_ERR_CUDA;
    for (const HazardRec& h : e->tree.hazards())
        if (h.alive && h.dynamic) s->dynamic_hazards.push_back(h);
    *out = s;
    return JCDE_OK;
}

// CDEngine::restore (cd_engine.rs:109-149): diff by entity, deregister the surplus, register the rest.
jcde_status jcde_restore(jcde_engine* e, const jcde_snapshot* s) {
    if (!e || !s) return JCDE_ERR_ARG;
    std::vector<std::pair<uint32_t, std::pair<int32_t, uint64_t>>> to_remove;
    const auto& hs = e->tree.hazards();
    for (uint32_t k = 0; k < hs.size(); k++)
        if (hs[k].alive && hs[k].dynamic) to_remove.push_back({k, {hs[k].kind, hs[k].tag}});
    std::vector<const HazardRec*> to_add;
    for (const HazardRec& h : s->dynamic_hazards) {
        auto it = std::find_if(to_remove.begin(), to_remove.end(),
                               [&](const auto& r) { return r.second.first == h.kind && r.second.second == h.tag; });
        if (it != to_remove.end()) {
            *it = to_remove.back();   // Vec::swap_remove
            to_remove.pop_back();
        } else {
            to_add.push_back(&h);
        }
    }
    for (const auto& r : to_remove) e->tree.remove(r.first);
    for (const HazardRec* h : to_add) {
        HazardRec c = *h;
        e->tree.insert(std::move(c));
    }
    return JCDE_OK;
}

void jcde_snapshot_free(jcde_snapshot* s) { delete s; }

jcde_status jcde_spolygon_new(const float* xy, uint32_t nv, float* xy_out, float* bbox_out, float* area_diam, float* poi) {
    if (!xy || !xy_out || !bbox_out || !area_diam || nv < 3) return JCDE_ERR_ARG;
    std::vector<Pt> pts(nv);
    for (uint32_t i = 0; i < nv; i++) pts[i] = Pt{xy[2 * i], xy[2 * i + 1]};
    PreparedPolygon p;
    if (spolygon_new(std::move(pts), &p, poi != nullptr)) return JCDE_ERR_ARG;
    for (uint32_t i = 0; i < nv; i++) {
        xy_out[2 * i] = p.v[i].x;
        xy_out[2 * i + 1] = p.v[i].y;
    }
    bbox_out[0] = p.bbox.x0; bbox_out[1] = p.bbox.y0; bbox_out[2] = p.bbox.x1; bbox_out[3] = p.bbox.y1;
    area_diam[0] = p.area;
    area_diam[1] = p.diameter;
    if (poi) {
        poi[0] = p.poi.c.x; poi[1] = p.poi.c.y; poi[2] = p.poi.r;
    }
    return JCDE_OK;
}

// SPolygon::centroid (simple_polygon.rs:173-192): sequential float32 sums over the edges
static void polygon_centroid(const float* xy, uint32_t nv, float area, float* out2) {
    float cx = 0.0f, cy = 0.0f;
    for (uint32_t i = 0; i < nv; i++) {
        const uint32_t j = i + 1 == nv ? 0 : i + 1;
        const float xi = xy[2 * i], yi = xy[2 * i + 1], xj = xy[2 * j], yj = xy[2 * j + 1];
        const float cr = xi * yj - xj * yi;
        cx = cx + (xi + xj) * cr;
        cy = cy + (yi + yj) * cr;
    }
    const float six_a = 6.0f * area;
    out2[0] = cx / six_a;
    out2[1] = cy / six_a;
}

jcde_status jcde_spolygon_batch(const float* xy, const uint32_t* voff, uint32_t n, float* xy_out, float* bbox_out,
                                float* area_diam, float* centroid_out, int32_t* status, uint32_t n_threads) {
    if (n && (!xy || !voff || !xy_out || !bbox_out || !area_diam || !status)) return JCDE_ERR_ARG;
    if (n_threads == 0) n_threads = std::max(1u, std::thread::hardware_concurrency());
    n_threads = std::min<uint32_t>(n_threads, std::max<uint32_t>(1u, n / 8));
    std::atomic<uint32_t> next{0};
    auto work = [&]() {
        for (uint32_t i; (i = next.fetch_add(1)) < n;) {
            const uint32_t v0 = voff[i], nv = voff[i + 1] - voff[i];
            status[i] = nv < 3 ? JCDE_ERR_ARG
                               : jcde_spolygon_new(xy + 2 * (size_t)v0, nv, xy_out + 2 * (size_t)v0, bbox_out + 4 * (size_t)i,
                                                   area_diam + 2 * (size_t)i, nullptr);
            if (centroid_out && status[i] == JCDE_OK)
                polygon_centroid(xy_out + 2 * (size_t)v0, nv, area_diam[2 * (size_t)i], centroid_out + 2 * (size_t)i);
        }
    };
    std::vector<std::thread> pool;
    for (uint32_t t = 1; t < n_threads; t++) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
    return JCDE_OK;
}

jcde_status jcde_close_concavities(const float* xy, uint32_t nv, int deflate, float ratio, float* xy_out,
                                   uint32_t* n_out) {
    if (!xy || !xy_out || !n_out || nv < 3) return JCDE_ERR_ARG;
    std::vector<Pt> pts(nv), out;
    for (uint32_t i = 0; i < nv; i++) pts[i] = Pt{xy[2 * i], xy[2 * i + 1]};
    if (close_concavities(std::move(pts), deflate != 0, ratio, &out)) return JCDE_ERR_ARG;
    *n_out = (uint32_t)out.size();
    for (size_t i = 0; i < out.size(); i++) {
        xy_out[2 * i] = out[i].x;
        xy_out[2 * i + 1] = out[i].y;
    }
    return JCDE_OK;
}

jcde_status jcde_surrogate_poles(const float* xy, uint32_t nv, float area, const float poi[3], const jcde_config* cfg,
                                 float* poles_xyr, uint32_t cap, uint32_t* n_out) {
    if (!xy || nv < 3 || !poi || !valid_config(cfg) || !n_out || (cap && !poles_xyr)) return JCDE_ERR_ARG;
    std::vector<Pt> pts(nv);
    for (uint32_t i = 0; i < nv; i++) pts[i] = Pt{xy[2 * i], xy[2 * i + 1]};
    PoleLimit lim[3];
    for (uint32_t i = 0; i < cfg->n_pole_limits; i++) lim[i] = PoleLimit{cfg->pole_limit_n[i], cfg->pole_limit_coverage[i]};
    std::vector<Disk> poles;
    if (surrogate_poles(pts, area, Disk{Pt{poi[0], poi[1]}, poi[2]}, lim, (int)cfg->n_pole_limits, &poles))
        return JCDE_ERR_ARG;
    *n_out = (uint32_t)poles.size();
    if (poles.size() > cap) return JCDE_ERR_CAPACITY;
    for (size_t i = 0; i < poles.size(); i++) {
        poles_xyr[3 * i] = poles[i].c.x;
        poles_xyr[3 * i + 1] = poles[i].c.y;
        poles_xyr[3 * i + 2] = poles[i].r;
    }
    return JCDE_OK;
}

jcde_status jcde_tree_dump(const jcde_engine* e, uint32_t* out, uint64_t cap, uint64_t* n_words) {
    if (!e || !n_words) return JCDE_ERR_ARG;
    std::vector<uint32_t> d;
    e->tree.dump(d);
    *n_words = d.size();
    if (d.size() > cap) return out ? JCDE_ERR_CAPACITY : JCDE_OK;
    if (out) std::memcpy(out, d.data(), d.size() * 4);
    return JCDE_OK;
}

jcde_status jcde_device_stats(jcde_engine* e, uint64_t* out5) {
    if (!e || !out5) return JCDE_ERR_ARG;
    jcde_status st = sync_device(e);
    if (st) return st;
    out5[0] = e->flat.nodes.size();
    out5[1] = e->flat.entries.size();
    out5[2] = e->flat.edges.size() / 4;
    out5[3] = e->hverts.size();
    out5[4] = e->iverts.size();
    return JCDE_OK;
}

uint64_t jcde_kernel_launches(const jcde_engine* e) { return e ? e->launches : 0; }

jcde_status jcde_profile_enable(jcde_engine* e, int enable) {
    if (!e) return JCDE_ERR_ARG;
    e->prof = enable != 0;
    return JCDE_OK;
}

jcde_status jcde_profile_read(jcde_engine* e, double* ms, uint64_t* count, int reset) {
    if (!e || !ms || !count) return JCDE_ERR_ARG;
    for (auto& m : e->prof_open) {
        float t = 0.0f;
        CUDA_TRY(cudaEventSynchronize(m.b));
        CUDA_TRY(cudaEventElapsedTime(&t, m.a, m.b));
        e->prof_ms[m.kind] += t;
        e->prof_n[m.kind] += 1;
        e->prof_pool.push_back(m.a);
        e->prof_pool.push_back(m.b);
    }
    e->prof_open.clear();
    for (int k = 0; k < JCDE_PROF_KINDS; k++) {
        ms[k] = e->prof_ms[k];
        count[k] = e->prof_n[k];
        if (reset) {
            e->prof_ms[k] = 0.0;
            e->prof_n[k] = 0;
        }
    }
    return JCDE_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Filtered detect that allocates nothing (jcde_detect_batch_noalloc).
//
// The regular filtered path keeps one device bitmask and one per-node strength array per distinct
// filter, allocated on first use.  This variant keeps those, and the two passes' work counters, in
// one static device array instead, so a call never allocates device memory.  Every GPU that loads
// the library holds the array until the process exits, every call shares it (it keeps the last
// call's contents), and calls that overlap on the GPU race on it.
//
// Layout of the array: [0, 256) the two work counters (cleared by each call), then the filter's
// key bitmask (n_slots bits, rounded up to 256 bytes), then the per-node strength table.
// ---------------------------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_noalloc_scratch[JCDE_NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mu;
static void* g_noalloc_addr[256] = {};   // device address of g_noalloc_scratch, per device ordinal

// Bitmask words handed over by value, in the launch parameters: nothing of the caller's key
// buffer is read after the call returns, and nothing is staged through host memory.
constexpr uint32_t NOALLOC_MASK_CHUNK = 960;
struct MaskChunk {
    uint32_t w[NOALLOC_MASK_CHUNK];
};
__global__ void k_mask_chunk(const MaskChunk c, uint32_t first, uint32_t count, uint32_t* __restrict__ mask) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) mask[first + i] = c.w[i];
}

// Set-up for the current device: the array's device address (the host name g_noalloc_scratch is
// only a stand-in, not a device address) and the code of k_mask_chunk, loaded now so that a later
// call loads nothing (CUDA loads kernels lazily by default).  Done once per device, with that
// device current: by the engine's first query of any kind (sync_device), or else by the first
// jcde_detect_batch_noalloc call on the device.  The address stays valid while the CUDA context
// lives; a cudaDeviceReset while the library is loaded is not supported.
static jcde_status noalloc_setup(void** out) {
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) return JCDE_ERR_STATE;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return JCDE_ERR_CUDA;
        // every kernel the call can launch
        cudaFuncAttributes fa;
        const void* fns[] = {(const void*)k_mask_chunk, (const void*)k_strength,
                             (const void*)k_surrogate_warp<uint32_t, 32>, (const void*)k_surrogate_warp<uint64_t, 32>,
                             (const void*)k_surrogate_warp<uint32_t, 16>, (const void*)k_surrogate_warp<uint64_t, 16>,
                             (const void*)k_surrogate_warp<uint32_t, 8>, (const void*)k_surrogate_warp<uint64_t, 8>,
                             (const void*)k_surrogate<uint32_t, false>, (const void*)k_surrogate<uint64_t, false>,
                             (const void*)k_poly_tab<uint32_t>, (const void*)k_poly_tab<uint64_t>,
                             (const void*)k_poly<uint32_t, false>, (const void*)k_poly<uint64_t, false>,
                             (const void*)k_poly<uint32_t, false, true>, (const void*)k_poly<uint64_t, false, true>};
        for (const void* fn : fns)
            if (cudaFuncGetAttributes(&fa, fn) != cudaSuccess) return JCDE_ERR_CUDA;
        g_noalloc_addr[dev] = p;
    }
    if (out) *out = g_noalloc_addr[dev];
    return JCDE_OK;
}

static inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

extern "C" jcde_status jcde_detect_batch_noalloc(jcde_engine* e, const jcde_query* dq, uint32_t n,
                                                  const jcde_filter* f, uint8_t* dout, void* stream) {
    if (!e || (n && (!dq || !dout))) return JCDE_ERR_ARG;
    const uint32_t n_keys = f ? f->n_ignored : 0u;
    if (n_keys && !f->ignored) return JCDE_ERR_ARG;
    // bringing the device mirror up to date may allocate: it must already be current
    if (e->tree_version != e->tree.version() || e->items_dirty) return JCDE_ERR_STATE;
    const uint32_t words = mask_words(e), n_slots = e->tree.n_slots();
    const size_t ctr_b = 256, mask_b = align256((size_t)words * 4);
    const size_t str_b = align256(e->n_nodes);
    if (ctr_b + mask_b + str_b > JCDE_NOALLOC_SCRATCH_BYTES) return JCDE_ERR_CAPACITY;
    void* base = nullptr;
    jcde_status st = noalloc_setup(&base);
    if (st) return st;
    init_launch_shape(e);
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char* b = static_cast<unsigned char*>(base);
    uint32_t* next = reinterpret_cast<uint32_t*>(b);
    uint32_t* mask = reinterpret_cast<uint32_t*>(b + ctr_b);
    uint8_t* strength = b + ctr_b + mask_b;
    // the bitmask, built here chunk by chunk and shipped by value (a chunk's words are all written,
    // so the previous call's mask needs no clearing)
    for (uint32_t w0 = 0; w0 < words; w0 += NOALLOC_MASK_CHUNK) {
        const uint32_t cnt = std::min(NOALLOC_MASK_CHUNK, words - w0);
        MaskChunk c;
        std::memset(c.w, 0, sizeof(c.w));
        for (uint32_t i = 0; i < n_keys; i++) {
            const uint32_t k = f->ignored[i];
            if (k < n_slots && (k >> 5) >= w0 && (k >> 5) < w0 + cnt) c.w[(k >> 5) - w0] |= 1u << (k & 31);
        }
        k_mask_chunk<<<(cnt + 255) / 256, 256, 0, s>>>(c, w0, cnt, mask);
        CUDA_TRY(cudaGetLastError());
        e->launches++;
    }
    View v = base_view(e);
    v.mask = mask;
    k_strength<<<(e->n_nodes + 255) / 256, 256, 0, s>>>(v, e->n_nodes, strength);
    CUDA_TRY(cudaGetLastError());
    v.strength = strength;
    e->launches++;
    if (n) {
        // counter-fed passes (the counters are cleared on the stream by the passes themselves); no
        // visit ordering, whose buffers grow with the batch
        launch_passes(e, v, reinterpret_cast<const uint32_t*>(dq), n, dout, s, RawShape{nullptr, 0, 0, 0, 0}, 3,
                      nullptr, next);
        CUDA_TRY(cudaGetLastError());
    }
    e->last_stream = s;
    e->have_last_stream = true;
    return JCDE_OK;
}

// ---------------------------------------------------------------------------------------------
// Several layouts queried together (jcde_multi_*): one ordering + surrogate + polygon launch
// sequence covers every engine's batch; each query reads the View of its own layout.
// ---------------------------------------------------------------------------------------------
struct jcde_multi {
    std::vector<jcde_engine*> engines;
    std::vector<View> views;          // views / offsets of the current call
    std::vector<uint32_t> offs;
    std::vector<View> up_views;       // what d_views / d_offs hold
    std::vector<uint32_t> up_offs;
    DevBuf d_views, d_offs, d_hist, d_order;
    DevBuf d_next;                    // work counters of the two passes
    DevBuf d_pend, d_pendc;           // the surrogate pass's list of undecided queries, its length
    bool wide = false;                // a tree deeper than 8 levels needs 64-bit walk masks
    int surr_blocks = 1;
    uint32_t poly_chunk = JCDE_POLY_CHUNK > 0 ? JCDE_POLY_CHUNK : 1;   // launch choices (jcde_multi_autotune)
    bool ordered = true;
    int n_sms = 1, poly_blocks = 1;
    // graph replay
    cudaGraphExec_t exec = nullptr;
    const void* g_q = nullptr;
    void* g_out = nullptr;
    cudaStream_t g_stream = nullptr;
    std::vector<View> g_views;
    std::vector<uint32_t> g_offs;
    uint64_t launches = 0;
    ~jcde_multi() {
        if (exec) cudaGraphExecDestroy(exec);
    }
};

// Bring every engine's device copy up to date, resolve its filter, and upload views + offsets.
static jcde_status multi_prepare(jcde_multi* m, const uint32_t* offsets, const jcde_filter* filters, cudaStream_t s) {
    const uint32_t L = (uint32_t)m->engines.size();
    m->views.resize(L);
    m->offs.assign(offsets, offsets + L + 1);
    for (uint32_t l = 0; l < L; l++) {
        if (m->offs[l + 1] < m->offs[l]) return JCDE_ERR_ARG;
        jcde_engine* e = m->engines[l];
        jcde_status st = sync_device(e);
        if (st) return st;
        init_launch_shape(e);
        View v = base_view(e);
        if ((st = apply_filter(e, filters ? &filters[l] : nullptr, s, v))) return st;
        m->views[l] = v;
    }
    const uint32_t total = m->offs[L];
    if (m->d_views.cap < L * sizeof(View) || m->d_offs.cap < (L + 1) * 4) {
        CUDA_TRY(cudaStreamSynchronize(s));
        if (!m->d_views.ensure(L * sizeof(View)) || !m->d_offs.ensure((L + 1) * 4)) return JCDE_ERR_CUDA;
        m->up_views.clear();
    }
    const size_t pend_bytes = std::max<size_t>(total, 1) * PEND_WORDS * 4;
    if (m->d_hist.cap < (size_t)L * N_BUCKETS * 4 || m->d_order.cap < std::max<size_t>(total, 1) * 4 ||
        m->d_pend.cap < pend_bytes || !m->d_pendc.p) {
        CUDA_TRY(cudaStreamSynchronize(s));   // growing frees buffers that queued launches may read
        if (!m->d_hist.ensure((size_t)L * N_BUCKETS * 4) || !m->d_order.ensure(std::max<size_t>(total, 1) * 4) ||
            !m->d_pend.ensure(pend_bytes) || !m->d_pendc.ensure(4))
            return JCDE_ERR_CUDA;
        m->up_views.clear();
    }
    // upload only what changed; the device copies are read by queued launches, so wait for them first
    const bool same = m->up_offs == m->offs && m->up_views.size() == L &&
                      std::memcmp(m->up_views.data(), m->views.data(), L * sizeof(View)) == 0;
    if (!same) {
        CUDA_TRY(cudaStreamSynchronize(s));
        CUDA_TRY(cudaMemcpy(m->d_views.p, m->views.data(), L * sizeof(View), cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(m->d_offs.p, m->offs.data(), (L + 1) * 4, cudaMemcpyHostToDevice));
        m->up_views = m->views;
        m->up_offs = m->offs;
    }
    return JCDE_OK;
}

#ifndef JCDE_MULTI_ORDER_MIN
#define JCDE_MULTI_ORDER_MIN (1u << 17)   // smaller multi-layout batches are visited in batch order
#endif
// Whether the current multi-layout batch is visited in Morton order: the tuned choice, for batches
// large enough that the ordering launches pay for themselves.
static bool multi_orders(const jcde_multi* m) { return m->ordered && !m->offs.empty() && m->offs.back() >= JCDE_MULTI_ORDER_MIN; }

template <typename PendT>
static void multi_launch_t(jcde_multi* m, const uint32_t* q, uint8_t* out, cudaStream_t s) {
    const uint32_t L = (uint32_t)m->engines.size(), n = m->offs[L];
    const MultiSrc ms{m->d_views.as<View>(), m->d_offs.as<uint32_t>(), L};
    uint32_t* hist = m->d_hist.as<uint32_t>();
    uint32_t* order = nullptr;
    const uint32_t grid = std::min<uint32_t>((n + 255) / 256, (uint32_t)m->n_sms * 8);
    if (multi_orders(m)) {
        order = m->d_order.as<uint32_t>();
        cudaMemsetAsync(hist, 0, (size_t)L * N_BUCKETS * 4, s);
        k_mbucket_count<<<grid, 256, 0, s>>>(q, n, ms, hist);
        k_scan_counts<<<1, 1024, 0, s>>>(hist, L * N_BUCKETS);
        k_mbucket_scatter<<<grid, 256, 0, s>>>(q, n, ms, hist, order);
        m->launches += 3;
    }
    // both passes take their queries from counters (see launch_passes_t); the polygon pass reads the
    // surrogate pass's list of undecided queries
    uint32_t* next = m->d_next.as<uint32_t>();
    const PendList pend{m->d_pend.as<uint32_t>(), m->d_pendc.as<uint32_t>()};
    cudaMemsetAsync(next, 0, 2 * 4, s);
    cudaMemsetAsync(pend.count, 0, 4, s);
    const uint32_t sgrid = std::min<uint32_t>((n + SURR_THREADS - 1) / SURR_THREADS, (uint32_t)(m->n_sms * m->surr_blocks));
    k_surrogate<PendT, true><<<sgrid, SURR_THREADS, 0, s>>>(View{}, ms, q, n, out, PENDING, order, next, nullptr, pend);
    const uint32_t pgrid = std::min<uint32_t>((n + POLY_WARPS - 1) / POLY_WARPS, (uint32_t)(m->n_sms * m->poly_blocks));
    k_poly<PendT, true><<<pgrid, POLY_WARPS * 32, 0, s>>>(View{}, ms, q, n, out, RawShape{nullptr, 0, 0, 0, 0}, true,
                                                          order, next + 1, m->poly_chunk, pend.rec, pend.count);
    m->launches += 2;
}
static void multi_launch(jcde_multi* m, const uint32_t* q, uint8_t* out, cudaStream_t s) {
    if (m->wide) multi_launch_t<uint64_t>(m, q, out, s);
    else multi_launch_t<uint32_t>(m, q, out, s);
}

extern "C" {

jcde_status jcde_multi_create(jcde_engine* const* engines, uint32_t n, jcde_multi** out) {
    if (!engines || !n || !out) return JCDE_ERR_ARG;
    jcde_multi* m = new (std::nothrow) jcde_multi();
    if (!m) return JCDE_ERR_CUDA;
    for (uint32_t l = 0; l < n; l++) {
        if (!engines[l]) {
            delete m;
            return JCDE_ERR_ARG;
        }
        m->engines.push_back(engines[l]);
        m->wide = m->wide || engines[l]->cfg.quadtree_depth > 8;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&m->n_sms, cudaDevAttrMultiProcessorCount, dev);
    if (m->wide) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m->poly_blocks, k_poly<uint64_t, true>, POLY_WARPS * 32, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m->surr_blocks, k_surrogate<uint64_t, true>, SURR_THREADS, 0);
    } else {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m->poly_blocks, k_poly<uint32_t, true>, POLY_WARPS * 32, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m->surr_blocks, k_surrogate<uint32_t, true>, SURR_THREADS, 0);
    }
    if (m->surr_blocks < 1) m->surr_blocks = 1;
    if (!m->d_next.ensure(2 * 4)) {
        delete m;
        return JCDE_ERR_CUDA;
    }
    if (m->n_sms < 1) m->n_sms = 1;
    if (m->poly_blocks < 1) m->poly_blocks = 1;
    *out = m;
    return JCDE_OK;
}

void jcde_multi_destroy(jcde_multi* m) { delete m; }

jcde_status jcde_multi_detect(jcde_multi* m, const jcde_query* dq, const uint32_t* offsets, const jcde_filter* filters,
                              uint8_t* dout, void* stream) {
    if (!m || !offsets) return JCDE_ERR_ARG;
    const uint32_t total = offsets[m->engines.size()];
    if (total && (!dq || !dout)) return JCDE_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    jcde_status st = multi_prepare(m, offsets, filters, s);
    if (st) return st;
    if (total == 0) return JCDE_OK;
    multi_launch(m, reinterpret_cast<const uint32_t*>(dq), dout, s);
    CUDA_TRY(cudaGetLastError());
    for (jcde_engine* e : m->engines) {
        e->last_stream = s;
        e->have_last_stream = true;
    }
    return JCDE_OK;
}

jcde_status jcde_multi_detect_graph(jcde_multi* m, const jcde_query* dq, const uint32_t* offsets,
                                    const jcde_filter* filters, uint8_t* dout, void* stream) {
    if (!m || !offsets || !stream) return JCDE_ERR_ARG;
    const uint32_t total = offsets[m->engines.size()];
    if (total == 0) return JCDE_OK;
    if (!dq || !dout) return JCDE_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    jcde_status st = multi_prepare(m, offsets, filters, s);
    if (st) return st;
    const bool same = m->exec && m->g_q == dq && m->g_out == dout && m->g_stream == s && m->g_offs == m->offs &&
                      m->g_views.size() == m->views.size() &&
                      std::memcmp(m->g_views.data(), m->views.data(), m->views.size() * sizeof(View)) == 0;
    if (!same) {
        if (m->exec) {
            cudaGraphExecDestroy(m->exec);
            m->exec = nullptr;
        }
        cudaGraph_t g = nullptr;
        CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        multi_launch(m, reinterpret_cast<const uint32_t*>(dq), dout, s);
        cudaError_t ce = cudaStreamEndCapture(s, &g);
        if (ce != cudaSuccess || !g) return JCDE_ERR_CUDA;
        ce = cudaGraphInstantiate(&m->exec, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            m->exec = nullptr;
            return JCDE_ERR_CUDA;
        }
        m->g_q = dq;
        m->g_out = dout;
        m->g_stream = s;
        m->g_views = m->views;
        m->g_offs = m->offs;
    }
    CUDA_TRY(cudaGraphLaunch(m->exec, s));
    m->launches += multi_orders(m) ? 5 : 2;
    for (jcde_engine* e : m->engines) {
        e->last_stream = s;
        e->have_last_stream = true;
    }
    return JCDE_OK;
}

uint64_t jcde_multi_kernel_launches(const jcde_multi* m) { return m ? m->launches : 0; }

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Pole-overlap proxy: hazard poles, forward/adjoint batch, gradient-descent separation, and the
// random-resampling baseline (no counterpart in the reference).
// ---------------------------------------------------------------------------------------------
extern "C" {

jcde_status jcde_set_hazard_poles(jcde_engine* e, uint32_t key, const float* xyr, uint32_t n) {
    if (!e || (n && !xyr)) return JCDE_ERR_ARG;
    std::vector<Disk> p(n);
    for (uint32_t i = 0; i < n; i++) p[i] = Disk{Pt{xyr[3 * i], xyr[3 * i + 1]}, xyr[3 * i + 2]};
    return e->tree.set_poles(key, std::move(p)) ? JCDE_OK : JCDE_ERR_NOT_FOUND;
}

static jcde_status proxy_prepare(jcde_engine* e, const jcde_filter* f, cudaStream_t s, View& v) {
    jcde_status st = sync_device(e);
    if (st) return st;
    if ((st = sync_poles(e))) return st;
    init_launch_shape(e);
    v = base_view(e);
    return apply_filter(e, f, s, v);
}

jcde_status jcde_proxy_batch(jcde_engine* e, const float* d_params, const uint32_t* d_items, uint32_t n,
                             const jcde_filter* f, float* d_value, float* d_grad, void* stream) {
    if (!e || (n && (!d_params || !d_items || !d_value || !d_grad))) return JCDE_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    View v;
    jcde_status st = proxy_prepare(e, f, s, v);
    if (st || n == 0) return st;
    const uint32_t grid = std::min<uint32_t>((n + PROXY_WARPS * 32 - 1) / (PROXY_WARPS * 32), (uint32_t)e->n_sms * 8);
    k_proxy<<<grid, PROXY_WARPS * 32, 0, s>>>(v, d_params, d_items, n, d_value, d_grad, nullptr);
    CUDA_TRY(cudaGetLastError());
    e->launches++;
    e->last_stream = s;
    e->have_last_stream = true;
    return JCDE_OK;
}

jcde_status jcde_proxy_forward(jcde_engine* e, const float* d_params, const uint32_t* d_items, uint32_t n,
                               const jcde_filter* f, float* d_value, void* stream) {
    if (!e || (n && (!d_params || !d_items || !d_value))) return JCDE_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    View v;
    jcde_status st = proxy_prepare(e, f, s, v);
    if (st || n == 0) return st;
    const uint32_t grid = std::min<uint32_t>((n + PROXY_WARPS * 32 - 1) / (PROXY_WARPS * 32), (uint32_t)e->n_sms * 8);
    k_proxy<<<grid, PROXY_WARPS * 32, 0, s>>>(v, d_params, d_items, n, d_value, nullptr, nullptr);
    CUDA_TRY(cudaGetLastError());
    e->launches++;
    e->last_stream = s;
    e->have_last_stream = true;
    return JCDE_OK;
}

jcde_status jcde_proxy_backward(jcde_engine* e, const float* d_params, const uint32_t* d_items, uint32_t n,
                                const jcde_filter* f, const float* d_grad_value, float* d_grad_params, void* stream) {
    if (!e || (n && (!d_params || !d_items || !d_grad_params))) return JCDE_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    View v;
    jcde_status st = proxy_prepare(e, f, s, v);
    if (st || n == 0) return st;
    const uint32_t grid = std::min<uint32_t>((n + PROXY_WARPS * 32 - 1) / (PROXY_WARPS * 32), (uint32_t)e->n_sms * 8);
    k_proxy<<<grid, PROXY_WARPS * 32, 0, s>>>(v, d_params, d_items, n, nullptr, d_grad_params, d_grad_value);
    CUDA_TRY(cudaGetLastError());
    e->launches++;
    e->last_stream = s;
    e->have_last_stream = true;
    return JCDE_OK;
}

jcde_status jcde_separate_batch(jcde_engine* e, float* d_params, const uint32_t* d_items, uint32_t n, uint32_t steps,
                                float step_t, float step_th, float clearance, const jcde_filter* f,
                                jcde_query* d_queries, float* d_value, void* stream) {
    if (!e || (n && (!d_params || !d_items || !d_queries || !d_value))) return JCDE_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    View v;
    jcde_status st = proxy_prepare(e, f, s, v);
    if (st || n == 0) return st;
    const uint32_t per_block = PROXY_WARPS * (32 / JCDE_SEP_LANES);
    const uint32_t grid = std::min<uint32_t>((n + per_block - 1) / per_block, (uint32_t)e->n_sms * 8);
    uint32_t* next = nullptr;
    if (e->d_next.ensure(2 * 2 * 4) && cudaMemsetAsync(e->d_next.p, 0, 4, s) == cudaSuccess) next = e->d_next.as<uint32_t>();
    cudaEvent_t pa = prof_begin(e, s);
    k_separate<<<grid, PROXY_WARPS * 32, 0, s>>>(v, d_params, d_items, n, steps, step_t, step_th, clearance,
                                                reinterpret_cast<uint32_t*>(d_queries), d_value, next);
    prof_end(e, s, pa, JCDE_PROF_PROXY);
    CUDA_TRY(cudaGetLastError());
    e->launches++;
    e->last_stream = s;
    e->have_last_stream = true;
    return JCDE_OK;
}

jcde_status jcde_resample_batch(jcde_engine* e, const float* d_params, const uint32_t* d_items, uint32_t n,
                                uint32_t k, float sigma_t, float sigma_th, uint32_t seed, jcde_query* d_queries,
                                void* stream) {
    if (!e || !k || (n && (!d_params || !d_items || !d_queries))) return JCDE_ERR_ARG;
    if (n == 0) return JCDE_OK;
    cudaStream_t s = (cudaStream_t)stream;
    init_launch_shape(e);
    const uint64_t total = (uint64_t)n * k;
    const uint32_t grid = (uint32_t)std::min<uint64_t>((total + 255) / 256, (uint64_t)e->n_sms * 16);
    k_resample<<<grid, 256, 0, s>>>(d_params, d_items, n, k, sigma_t, sigma_th, seed,
                                    reinterpret_cast<uint32_t*>(d_queries));
    CUDA_TRY(cudaGetLastError());
    e->launches++;
    return JCDE_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// LBF choice of a candidate batch (lbf/src/opt/search.rs:44-66): see k_lbf_select.
// ---------------------------------------------------------------------------------------------
extern "C" jcde_status jcde_lbf_select(jcde_engine* e, const jcde_query* d_queries, const uint8_t* d_verdicts,
                                        uint32_t n, uint64_t* d_best, void* stream) {
    return jcde_lbf_select_segments(e, d_queries, d_verdicts, n, 1, d_best, stream);
}

extern "C" jcde_status jcde_lbf_select_segments(jcde_engine* e, const jcde_query* d_queries, const uint8_t* d_verdicts,
                                                 uint32_t n, uint32_t n_segments, uint64_t* d_best, void* stream) {
    if (!e || !d_best || n_segments == 0 || n_segments > 65535 || (n && (!d_queries || !d_verdicts))) return JCDE_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    jcde_status st = sync_device(e);
    if (st) return st;
    init_launch_shape(e);
    CUDA_TRY(cudaMemsetAsync(d_best, 0xFF, 8 * (size_t)n_segments, s));
    if (n == 0) return JCDE_OK;
    const View v = base_view(e);
    const uint32_t gx = std::max<uint32_t>(1u, std::min<uint32_t>((n + 7) / 8, (uint32_t)e->n_sms * 8 / n_segments));
    k_lbf_select<<<dim3(gx, n_segments), 256, 0, s>>>(v, reinterpret_cast<const uint32_t*>(d_queries), d_verdicts, n,
                                                      reinterpret_cast<unsigned long long*>(d_best), nullptr);
    CUDA_TRY(cudaGetLastError());
    e->launches++;
    e->last_stream = s;
    e->have_last_stream = true;
    return JCDE_OK;
}

// ---------------------------------------------------------------------------------------------
// Device-resident engine (resident.cuh): the quadtree lives in device pools that register /
// deregister update on the GPU, and the LBF-style build that runs on it step by step.
// ---------------------------------------------------------------------------------------------
struct jcde_resident {
    jcde_engine* e = nullptr;
    RTree t{};
    int32_t exterior = -1;
    DevBuf d_nodes, d_ncap, d_level, d_strength, d_nedges, d_entries, d_edges, d_haz, d_hverts, d_alive, d_qfree,
        d_kfree, d_tasks, d_ctl;
    // LBF-style build
    bool lbf_ready = false;
    LbfParams lp{};
    DevBuf d_lbf, d_cand, d_candu, d_verd, d_place, d_remv, d_free, d_live, d_vlog;
    DevBuf d_cand2, d_candu2;   // the other candidate buffer: step k of a launch uses buffer k % 2
    DevBuf d_seq, d_orient, d_orient_of;   // instance mode: item sequence, allowed orientations
    DevBuf d_hist, d_order;   // spatial ordering of the resident's own query batches
    DevBuf d_next;            // work counters of its two passes
    cudaGraphExec_t exec = nullptr;
    uint32_t exec_steps = 0;
    uint64_t exec_launches = 0;   // kernels one launch of `exec` runs
    cudaStream_t exec_stream = nullptr;
    cudaStream_t own = nullptr;
    cudaStream_t last = nullptr;
    // the next step's first candidates are drawn on `side` while a step commits (fork and join)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    uint64_t launches = 0;
    uint64_t load_bytes = 0;   // host-to-device bytes of the last load of the engine's hazards
    ~jcde_resident() {
        if (last) cudaStreamSynchronize(last);
        if (side) cudaStreamSynchronize(side);
        if (exec) cudaGraphExecDestroy(exec);
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        if (side) cudaStreamDestroy(side);
        if (own) {
            // the engine must not wait on a stream that no longer exists
            if (e && e->have_last_stream && e->last_stream == own) {
                e->have_last_stream = false;
                e->last_stream = nullptr;
            }
            cudaStreamDestroy(own);
        }
    }
};

static View resident_view(const jcde_resident* r) {
    View v = base_view(r->e);
    v.nodes = r->t.nodes;
    v.entries = r->t.entries;
    v.edges = r->t.edges;
    v.haz = r->t.haz;
    v.hverts = r->t.hverts;
    v.strength = r->t.strength;
    v.nedges = r->t.nedges;
    v.cbox = nullptr;   // the resident pools keep no edge-tile boxes
    v.eg_shift = 3;
    v.mask = nullptr;
    v.n_slots = r->t.key_cap;
    v.exterior = r->exterior;
    return v;
}

static inline uint64_t host_mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
static inline uint64_t host_stream_key(uint64_t seed, uint64_t sid) {
    return host_mix64(seed * 0x100000001B3ull + sid * 0x9E3779B97F4A7C15ull);
}

extern "C" jcde_status jcde_gen_candidates(uint64_t seed, uint64_t sid, uint32_t n, uint32_t item, jcde_rect box,
                                           const float* d_orient, uint32_t n_orient, jcde_query* d_queries,
                                           double* d_turns, void* stream) {
    return jcde_gen_candidates_segments(seed, &sid, &box, 1, n, item, d_orient, n_orient, d_queries, d_turns, stream);
}

extern "C" jcde_status jcde_gen_candidates_segments(uint64_t seed, const uint64_t* sids, const jcde_rect* boxes,
                                                    uint32_t n_segments, uint32_t n, uint32_t item, const float* d_orient,
                                                    uint32_t n_orient, jcde_query* d_queries, double* d_turns,
                                                    void* stream) {
    if (n == 0 || n_segments == 0) return JCDE_OK;
    if (!sids || !boxes || !d_queries || (n_orient && !d_orient)) return JCDE_ERR_ARG;
    for (uint32_t k = 0; k < n_segments; k++)
        if (!(boxes[k].x_min < boxes[k].x_max) || !(boxes[k].y_min < boxes[k].y_max)) return JCDE_ERR_ARG;
    int dev = 0, n_sms = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&n_sms, cudaDevAttrMultiProcessorCount, dev));
    for (uint32_t k0 = 0; k0 < n_segments; k0 += RES_GEN_SEGMENTS) {   // segments by kernel-parameter batches
        const uint32_t m = std::min<uint32_t>(RES_GEN_SEGMENTS, n_segments - k0);
        unsigned long long keys[RES_GEN_SEGMENTS];
        float bx[RES_GEN_SEGMENTS][4];
        for (uint32_t k = 0; k < m; k++) {
            keys[k] = host_stream_key(seed, sids[k0 + k]);
            bx[k][0] = boxes[k0 + k].x_min;
            bx[k][1] = boxes[k0 + k].y_min;
            bx[k][2] = boxes[k0 + k].x_max;
            bx[k][3] = boxes[k0 + k].y_max;
        }
        res_launch_gen_candidates(keys, bx, m, n, item, reinterpret_cast<const float2*>(d_orient), n_orient,
                                  reinterpret_cast<uint32_t*>(d_queries + (size_t)k0 * n),
                                  d_turns ? d_turns + (size_t)k0 * n : nullptr, n_sms, (cudaStream_t)stream);
        CUDA_TRY(cudaGetLastError());
    }
    return JCDE_OK;
}

// The resident's ordering buffers hold a batch of n queries (growing them waits for queued work).
static jcde_status ensure_order_buffers(jcde_resident* r, uint32_t n) {
    if (!r->d_hist.ensure(ORDER_HIST_WORDS * 4)) return JCDE_ERR_CUDA;
    if (r->d_order.cap < (size_t)n * 4) {
        if (r->last) CUDA_TRY(cudaStreamSynchronize(r->last));
        if (!r->d_order.ensure((size_t)n * 4)) return JCDE_ERR_CUDA;
    }
    return JCDE_OK;
}

static bool resident_detect(jcde_resident* r, const uint32_t* q, uint32_t n, uint8_t* dout, cudaStream_t s,
                            unsigned long long* best = nullptr, uint32_t* n_pending = nullptr, bool skip = false) {
    jcde_engine* e = r->e;
    const View v = resident_view(r);
    // small batches (one LBF step's candidates) gain nothing from the visit order
    const uint32_t* order = nullptr;
    if (JCDE_SPATIAL_ORDER && n >= e->tune.order_min_batch && n > e->tune.surrogate_warp_max)
        order = spatial_order_into(e, q, n, s, r->d_hist.as<uint32_t>(), r->d_order.as<uint32_t>());
    const bool chose =
        launch_passes(e, v, q, n, dout, s, RawShape{}, 3, order, r->d_next.as<uint32_t>(), best, n_pending, skip);
    r->launches += (order ? 2 : 0) + 2;
    return chose;
}

// One step of the LBF-style build: a uniform round and ls_rounds local-search rounds, each
// generate -> surrogate pass -> polygon pass + choice (-> merge into the step's best), then the
// commit.  With `drawn`, the first round's candidates were generated while the previous step
// committed; with `ahead`, the next step's are generated on the side stream while this step
// commits (the commit touches neither the candidates nor the generator's inputs, and the generation
// neither the tree nor the step state).
static void lbf_step(jcde_resident* r, cudaStream_t s, uint32_t k, bool ahead) {
    jcde_engine* e = r->e;
    LbfDev* st = r->d_lbf.as<LbfDev>();
    const bool drawn = k > 0;   // the first round was generated while the previous step committed
    uint32_t* cand = (k & 1u) ? r->d_cand2.as<uint32_t>() : r->d_cand.as<uint32_t>();
    double* cu = (k & 1u) ? r->d_candu2.as<double>() : r->d_candu.as<double>();
    uint8_t* verd = r->d_verd.as<uint8_t>();
    const uint32_t last = r->lp.uni_rounds + r->lp.ls_rounds - 1;   // uniform rounds, then local search
    for (uint32_t round = 0; round <= last; round++) {
        const uint32_t n = round < r->lp.uni_rounds ? r->lp.n_uni : r->lp.ls_cand;
        cudaEvent_t pa = nullptr;
        if (round > 0 || !drawn) {
            pa = prof_begin(e, s);
            res_launch_lbf_gen(r->lp, st, cand, cu, round, e->n_sms, s, false, k & 1u);
            prof_end(e, s, pa, JCDE_PROF_LBF);
            r->launches++;
        }
        // the polygon pass makes the choice itself when it runs its small-batch kernel, skipping the
        // candidates that can no longer win unless every verdict is logged; n_free counts the
        // candidates the surrogate pass leaves to the polygon pass
        const bool skip = r->lp.vlog_steps == 0;
        if (!resident_detect(r, cand, n, verd, s, &st->best, &st->n_free, skip)) {
            const View v = resident_view(r);
            const uint32_t grid = std::min<uint32_t>((n + 7) / 8, (uint32_t)e->n_sms * 8);
            pa = prof_begin(e, s);
            k_lbf_select<<<grid, 256, 0, s>>>(v, cand, verd, n, &st->best, nullptr);
            prof_end(e, s, pa, JCDE_PROF_LBF);
            r->launches++;
        }
        if (round < last) {
            pa = prof_begin(e, s);
            res_launch_lbf_merge(st, cand, cu, round, s);
            prof_end(e, s, pa, JCDE_PROF_LBF);
            r->launches++;
        }
    }
    LbfLogs logs{r->d_place.as<uint32_t>(), r->d_remv.as<uint32_t>(), r->d_free.as<uint32_t>(),
                 r->d_live.as<uint32_t>(), r->lp.vlog_steps ? r->d_vlog.as<uint8_t>() : nullptr};
    cudaEvent_t pa = nullptr;
    if (ahead) {   // the next step's first round, into the other buffer, while this step commits
        uint32_t* cand_n = (k & 1u) ? r->d_cand.as<uint32_t>() : r->d_cand2.as<uint32_t>();
        double* cu_n = (k & 1u) ? r->d_candu.as<double>() : r->d_candu2.as<double>();
        cudaEventRecord(r->ev_fork, s);
        cudaStreamWaitEvent(r->side, r->ev_fork, 0);
        pa = prof_begin(e, r->side);
        res_launch_lbf_gen(r->lp, st, cand_n, cu_n, 0, e->n_sms, r->side, true, (k + 1) & 1u);
        prof_end(e, r->side, pa, JCDE_PROF_LBF);
        r->launches++;
        cudaEventRecord(r->ev_join, r->side);
    }
    pa = prof_begin(e, s);
    res_launch_lbf_commit(r->t, e->d_items.as<DItem>(), e->d_iverts.as<float2>(), (uint32_t)e->items.size(), r->lp,
                          st, cand, cu, last, verd, logs, s, ahead);
    prof_end(e, s, pa, JCDE_PROF_UPDATE);
    r->launches++;
    if (ahead) cudaStreamWaitEvent(s, r->ev_join, 0);
}

// Loads the engine's live hazards, each under its own key, into empty pools (jcde_resident_create
// and jcde_resident_reset).  Synchronises.
static jcde_status resident_load(jcde_resident* r) {
    jcde_engine* e = r->e;
    const RTree& t = r->t;
    const auto& hs = e->tree.hazards();
    std::vector<float2> verts;
    std::vector<uint4> recs;
    std::vector<float2> pois;
    for (uint32_t k = 0; k < hs.size(); k++) {
        if (!hs[k].alive) continue;
        const Polygon& p = hs[k].shape;
        recs.push_back(make_uint4(k, (uint32_t)hs[k].kind, (uint32_t)verts.size(), (uint32_t)p.v.size()));
        pois.push_back(make_float2(p.poi.c.x, p.poi.c.y));
        for (const Pt& v : p.v) verts.push_back(make_float2(v.x, v.y));
    }
    const std::vector<uint32_t>& fk = e->tree.free_keys();
    DevBuf d_v, d_r, d_p, d_k;
    cudaStream_t s = r->own;
    if (!d_v.ensure(std::max<size_t>(verts.size(), 1) * sizeof(float2)) ||
        !d_r.ensure(std::max<size_t>(recs.size(), 1) * sizeof(uint4)) ||
        !d_p.ensure(std::max<size_t>(pois.size(), 1) * sizeof(float2)) || !d_k.ensure(std::max<size_t>(fk.size(), 1) * 4))
        return JCDE_ERR_CUDA;
    CUDA_TRY(cudaMemsetAsync(t.alive, 0, t.key_cap, s));
    CUDA_TRY(cudaMemsetAsync(t.ctl, 0, sizeof(RCtl), s));
    if (verts.size()) CUDA_TRY(cudaMemcpyAsync(d_v.p, verts.data(), verts.size() * sizeof(float2), cudaMemcpyHostToDevice, s));
    if (recs.size()) CUDA_TRY(cudaMemcpyAsync(d_r.p, recs.data(), recs.size() * sizeof(uint4), cudaMemcpyHostToDevice, s));
    if (pois.size()) CUDA_TRY(cudaMemcpyAsync(d_p.p, pois.data(), pois.size() * sizeof(float2), cudaMemcpyHostToDevice, s));
    if (fk.size()) CUDA_TRY(cudaMemcpyAsync(d_k.p, fk.data(), fk.size() * 4, cudaMemcpyHostToDevice, s));
    r->load_bytes = verts.size() * sizeof(float2) + recs.size() * sizeof(uint4) + pois.size() * sizeof(float2) + fk.size() * 4;
    res_launch_init(t, d_v.as<float2>(), d_r.as<uint4>(), d_p.as<float2>(), (uint32_t)recs.size(), e->tree.n_slots(),
                    d_k.as<uint32_t>(), (uint32_t)fk.size(), s);
    CUDA_TRY(cudaGetLastError());
    RCtl ctl{};
    CUDA_TRY(cudaMemcpyAsync(&ctl, t.ctl, sizeof(RCtl), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    r->launches++;
    r->last = nullptr;
    return ctl.error ? JCDE_ERR_CAPACITY : JCDE_OK;
}

extern "C" {

void jcde_resident_default_config(jcde_resident_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->max_entries = 1u << 21;
    c->max_edges = 1u << 23;
    c->max_hazard_vertices = 1u << 22;
    c->max_keys = 1u << 20;
    c->max_tasks = 1u << 16;
}

jcde_status jcde_resident_create(jcde_engine* e, const jcde_resident_config* cfg, jcde_resident** out) {
    if (!e || !out) return JCDE_ERR_ARG;
    *out = nullptr;
    jcde_resident_config c;
    jcde_resident_default_config(&c);
    if (cfg) {
        if (cfg->max_nodes) c.max_nodes = cfg->max_nodes;
        if (cfg->max_entries) c.max_entries = cfg->max_entries;
        if (cfg->max_edges) c.max_edges = cfg->max_edges;
        if (cfg->max_hazard_vertices) c.max_hazard_vertices = cfg->max_hazard_vertices;
        if (cfg->max_keys) c.max_keys = cfg->max_keys;
        if (cfg->max_tasks) c.max_tasks = cfg->max_tasks;
    }
    if (!c.max_nodes) {   // every node of a full tree of the engine's depth, at most 2^22
        uint64_t full = 0, lv = 1;
        for (int d = 0; d <= e->cfg.quadtree_depth && full < (1u << 22); d++, lv *= 4) full += lv;
        c.max_nodes = (uint32_t)std::min<uint64_t>(full, 1u << 22);
    }
    if (c.max_keys < e->tree.n_slots() || c.max_nodes < 1) return JCDE_ERR_CAPACITY;
    jcde_status st = sync_device(e);
    if (st) return st;
    init_launch_shape(e);
    jcde_resident* r = new (std::nothrow) jcde_resident();
    if (!r) return JCDE_ERR_CUDA;
    r->e = e;
    r->exterior = e->tree.exterior_key();
    RTree& t = r->t;
    const uint32_t nq = c.max_nodes / 4 + 1;
    bool ok = r->d_nodes.ensure((size_t)c.max_nodes * sizeof(DNode)) && r->d_ncap.ensure((size_t)c.max_nodes * 4) &&
              r->d_level.ensure(c.max_nodes) && r->d_strength.ensure(c.max_nodes) &&
              r->d_nedges.ensure((size_t)c.max_nodes * 4) &&
              r->d_entries.ensure((size_t)c.max_entries * sizeof(DEntry)) &&
              r->d_edges.ensure((size_t)c.max_edges * sizeof(float4)) &&
              r->d_haz.ensure((size_t)c.max_keys * sizeof(DHaz)) &&
              r->d_hverts.ensure((size_t)c.max_hazard_vertices * sizeof(float2)) && r->d_alive.ensure(c.max_keys) &&
              r->d_qfree.ensure((size_t)nq * 4) && r->d_kfree.ensure((size_t)c.max_keys * 4) &&
              r->d_tasks.ensure((size_t)c.max_tasks * sizeof(RTask)) && r->d_ctl.ensure(sizeof(RCtl)) &&
              r->d_next.ensure(2 * 4);
    if (!ok || cudaStreamCreateWithFlags(&r->own, cudaStreamNonBlocking) != cudaSuccess) {
        delete r;
        return JCDE_ERR_CUDA;
    }
    t.nodes = r->d_nodes.as<DNode>();
    t.ncap = r->d_ncap.as<uint32_t>();
    t.level = r->d_level.as<uint8_t>();
    t.strength = r->d_strength.as<uint8_t>();
    t.nedges = r->d_nedges.as<uint32_t>();
    t.entries = r->d_entries.as<DEntry>();
    t.edges = r->d_edges.as<float4>();
    t.haz = r->d_haz.as<DHaz>();
    t.hverts = r->d_hverts.as<float2>();
    t.alive = r->d_alive.as<uint8_t>();
    t.qfree = r->d_qfree.as<int32_t>();
    t.kfree = r->d_kfree.as<uint32_t>();
    t.tasks = r->d_tasks.as<RTask>();
    t.ctl = r->d_ctl.as<RCtl>();
    t.node_cap = c.max_nodes;
    t.entry_cap = c.max_entries;
    t.edge_cap = c.max_edges;
    t.hvert_cap = c.max_hazard_vertices;
    t.key_cap = c.max_keys;
    t.task_cap = c.max_tasks;
    t.cde = e->tree.bbox();
    t.depth = e->cfg.quadtree_depth;
    if ((st = resident_load(r))) {
        delete r;
        return st;
    }
    *out = r;
    return JCDE_OK;
}

void jcde_resident_destroy(jcde_resident* r) { delete r; }

jcde_status jcde_resident_reset(jcde_resident* r, uint64_t* h2d_bytes) {
    if (!r) return JCDE_ERR_ARG;
    if (r->last) CUDA_TRY(cudaStreamSynchronize(r->last));
    jcde_status st = sync_device(r->e);
    if (st) return st;
    r->exterior = r->e->tree.exterior_key();
    st = resident_load(r);
    if (h2d_bytes) *h2d_bytes = r->load_bytes;
    return st;
}

jcde_status jcde_resident_register_placed(jcde_resident* r, const jcde_query* d_query, uint32_t* d_key, void* stream) {
    if (!r || !d_query) return JCDE_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    jcde_engine* e = r->e;
    res_launch_insert_placed(r->t, e->d_items.as<DItem>(), e->d_iverts.as<float2>(), (uint32_t)e->items.size(),
                             reinterpret_cast<const uint32_t*>(d_query), d_key, s);
    CUDA_TRY(cudaGetLastError());
    r->launches++;
    r->last = s;
    return JCDE_OK;
}

jcde_status jcde_resident_deregister(jcde_resident* r, const uint32_t* d_key, void* stream) {
    if (!r || !d_key) return JCDE_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    res_launch_remove(r->t, d_key, s);
    CUDA_TRY(cudaGetLastError());
    r->launches++;
    r->last = s;
    return JCDE_OK;
}

jcde_status jcde_resident_detect_batch(jcde_resident* r, const jcde_query* d_queries, uint32_t n, uint8_t* d_out,
                                       void* stream) {
    if (!r || (n && (!d_queries || !d_out))) return JCDE_ERR_ARG;
    if (n == 0) return JCDE_OK;
    cudaStream_t s = (cudaStream_t)stream;
    jcde_status st = ensure_order_buffers(r, n);
    if (st) return st;
    resident_detect(r, reinterpret_cast<const uint32_t*>(d_queries), n, d_out, s);
    CUDA_TRY(cudaGetLastError());
    r->e->last_stream = s;
    r->e->have_last_stream = true;
    r->last = s;
    return JCDE_OK;
}

jcde_status jcde_resident_status(jcde_resident* r, uint32_t* out8) {
    if (!r || !out8) return JCDE_ERR_ARG;
    if (r->last) CUDA_TRY(cudaStreamSynchronize(r->last));
    RCtl c{};
    CUDA_TRY(cudaMemcpy(&c, r->t.ctl, sizeof(RCtl), cudaMemcpyDeviceToHost));
    const uint32_t v[8] = {c.error, c.not_found, c.n_live, c.n_slots, c.n_nodes, c.entry_top, c.edge_top, c.hvert_top};
    std::memcpy(out8, v, sizeof(v));
    return c.error ? JCDE_ERR_CAPACITY : JCDE_OK;
}

jcde_status jcde_resident_tree_dump(jcde_resident* r, uint32_t* out, uint64_t cap, uint64_t* n_words) {
    if (!r || !n_words) return JCDE_ERR_ARG;
    if (r->last) CUDA_TRY(cudaStreamSynchronize(r->last));
    RCtl c{};
    CUDA_TRY(cudaMemcpy(&c, r->t.ctl, sizeof(RCtl), cudaMemcpyDeviceToHost));
    std::vector<DNode> nodes(c.n_nodes);
    std::vector<uint8_t> level(c.n_nodes);
    std::vector<uint32_t> nedges(c.n_nodes);
    std::vector<DEntry> ents(c.entry_top);
    std::vector<float4> edges(c.edge_top);
    CUDA_TRY(cudaMemcpy(nodes.data(), r->t.nodes, nodes.size() * sizeof(DNode), cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(level.data(), r->t.level, level.size(), cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(nedges.data(), r->t.nedges, nedges.size() * 4, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(ents.data(), r->t.entries, ents.size() * sizeof(DEntry), cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(edges.data(), r->t.edges, edges.size() * sizeof(float4), cudaMemcpyDeviceToHost));
    // the canonical form of QuadTree::dump: depth-first, entries by key, edges sorted
    std::vector<uint32_t> o;
    auto fb = [](float f) {
        uint32_t u;
        std::memcpy(&u, &f, 4);
        return u;
    };
    auto box = [&](const Box& b) {
        o.push_back(fb(b.x0));
        o.push_back(fb(b.y0));
        o.push_back(fb(b.x1));
        o.push_back(fb(b.y1));
    };
    std::vector<int32_t> stack{0};
    while (!stack.empty()) {
        const int32_t ni = stack.back();
        stack.pop_back();
        if (ni < 0 || (uint32_t)ni >= c.n_nodes) return JCDE_ERR_STATE;
        const DNode& n = nodes[ni];
        o.push_back(level[ni]);
        o.push_back(n.child >= 0 ? 1u : 0u);
        o.push_back(n.hz_cnt);
        o.push_back(nedges[ni]);
        box(n.box);
        if (n.hz_off + (uint64_t)n.hz_cnt > ents.size()) return JCDE_ERR_STATE;
        std::vector<const DEntry*> hs;
        for (uint32_t k = 0; k < n.hz_cnt; k++) hs.push_back(&ents[n.hz_off + k]);
        std::sort(hs.begin(), hs.end(), [](const DEntry* a, const DEntry* b) { return a->hkey < b->hkey; });
        for (const DEntry* h : hs) {
            o.push_back(h->hkey);
            o.push_back(h->presence);
            if (h->presence == PRES_PARTIAL) {
                box(h->ff);
                if (h->edge_off + (uint64_t)h->edge_cnt > edges.size()) return JCDE_ERR_STATE;
                std::vector<std::array<uint32_t, 4>> es;
                for (uint32_t j = 0; j < h->edge_cnt; j++) {
                    const float4 f = edges[h->edge_off + j];
                    es.push_back({fb(f.x), fb(f.y), fb(f.z), fb(f.w)});
                }
                std::sort(es.begin(), es.end());
                o.push_back((uint32_t)es.size());
                for (auto& e4 : es) o.insert(o.end(), e4.begin(), e4.end());
            }
        }
        if (n.child >= 0)
            for (int i = 3; i >= 0; i--) stack.push_back(n.child + i);
    }
    *n_words = o.size();
    if (!out || cap < o.size()) return out ? JCDE_ERR_CAPACITY : JCDE_OK;
    std::memcpy(out, o.data(), o.size() * 4);
    return JCDE_OK;
}

uint64_t jcde_resident_kernel_launches(const jcde_resident* r) { return r ? r->launches : 0; }

jcde_status jcde_lbf_begin(jcde_resident* r, const jcde_lbf_params* p) {
    if (!r || !p || !p->n_candidates || !p->max_steps) return JCDE_ERR_ARG;
    if ((!p->item_sequence && !p->n_types) || p->n_types > r->e->items.size()) return JCDE_ERR_ARG;
    const jcde_rect b = p->sample_box;
    if (!(b.x_min < b.x_max && b.y_min < b.y_max)) return JCDE_ERR_ARG;
    if (r->last) CUDA_TRY(cudaStreamSynchronize(r->last));
    LbfParams& lp = r->lp;
    lp = LbfParams{};
    lp.seed = p->seed;
    lp.key_types = host_stream_key(p->seed, 2);
    lp.key_remove = host_stream_key(p->seed, 4);
    lp.sid_base = 10000;
    lp.n_cand = p->n_candidates;
    lp.n_types = p->n_types;
    lp.remove_every = p->remove_every;
    lp.max_steps = p->max_steps;
    lp.vlog_steps = std::min(p->verdict_log_steps, p->max_steps);
    lp.x0 = b.x_min;
    lp.y0 = b.y_min;
    lp.x1 = b.x_max;
    lp.y1 = b.y_max;
    lp.x1_below = std::nextafter(b.x_max, b.x_min);
    lp.y1_below = std::nextafter(b.y_max, b.y_min);
    if (p->ls_rounds > LBF_MAX_LS || (p->ls_rounds && (!p->ls_candidates || p->ls_candidates > p->n_candidates)))
        return JCDE_ERR_ARG;
    const uint32_t uni = std::max(1u, p->uniform_rounds);
    if (uni > LBF_MAX_UNIFORM || p->n_candidates % uni) return JCDE_ERR_ARG;
    lp.uni_rounds = uni;
    lp.n_uni = p->n_candidates / uni;
    lp.uni_sid_base = 2000000ull;
    lp.ls_rounds = p->ls_rounds;
    lp.ls_cand = p->ls_rounds ? p->ls_candidates : 0;
    lp.ls_sid_base = 1000000ull;
    for (uint32_t k = 1; k <= p->ls_rounds; k++) {   // round r's deviations, as given
        if (!(p->ls_sigma_t[k - 1] >= 0.0f) || !(p->ls_sigma_turns[k - 1] >= 0.0)) return JCDE_ERR_ARG;
        lp.ls_sig[k] = p->ls_sigma_t[k - 1];
        lp.ls_sth[k] = p->ls_sigma_turns[k - 1];
    }
    // the verdict log keeps one round per step
    if ((lp.ls_rounds || lp.uni_rounds > 1) && lp.vlog_steps) return JCDE_ERR_ARG;
    // instance mode: the item sequence and the allowed orientations
    const uint32_t n_items = (uint32_t)r->e->items.size();
    if (p->item_sequence) {
        if (p->n_sequence < p->max_steps) return JCDE_ERR_ARG;
        for (uint32_t k = 0; k < p->n_sequence; k++)
            if (p->item_sequence[k] >= n_items) return JCDE_ERR_ARG;
        if (!r->d_seq.ensure((size_t)p->n_sequence * 4)) return JCDE_ERR_CUDA;
        CUDA_TRY(cudaMemcpy(r->d_seq.p, p->item_sequence, (size_t)p->n_sequence * 4, cudaMemcpyHostToDevice));
        lp.seq = r->d_seq.as<uint32_t>();
    }
    if (p->orientation_offsets) {
        if (p->n_orientation_items != n_items || !p->orientation_cs) return JCDE_ERR_ARG;
        std::vector<uint2> of(n_items);
        for (uint32_t k = 0; k < n_items; k++) {
            const uint32_t a = p->orientation_offsets[k], b = p->orientation_offsets[k + 1];
            if (b < a) return JCDE_ERR_ARG;
            of[k] = make_uint2(a, b - a);
        }
        const uint32_t n_or = p->orientation_offsets[n_items];
        if (!r->d_orient_of.ensure(of.size() * sizeof(uint2)) || !r->d_orient.ensure(std::max<size_t>(n_or, 1) * 8))
            return JCDE_ERR_CUDA;
        CUDA_TRY(cudaMemcpy(r->d_orient_of.p, of.data(), of.size() * sizeof(uint2), cudaMemcpyHostToDevice));
        if (n_or) CUDA_TRY(cudaMemcpy(r->d_orient.p, p->orientation_cs, (size_t)n_or * 8, cudaMemcpyHostToDevice));
        lp.orient = r->d_orient.as<float2>();
        lp.orient_of = r->d_orient_of.as<uint2>();
    }
    const size_t n = p->n_candidates, ms = p->max_steps;
    const bool ok = r->d_lbf.ensure(sizeof(LbfDev)) && r->d_cand.ensure(n * 20) && r->d_candu.ensure(n * 8) &&
                    r->d_cand2.ensure(n * 20) && r->d_candu2.ensure(n * 8) &&
                    r->d_verd.ensure(n) &&
                    r->d_place.ensure(ms * 32) && r->d_remv.ensure(ms * 8) && r->d_free.ensure(ms * 4) &&
                    r->d_live.ensure(ms * 4) && (!lp.vlog_steps || r->d_vlog.ensure((size_t)lp.vlog_steps * n));
    if (!ok) return JCDE_ERR_CUDA;
    CUDA_TRY(cudaMemset(r->d_lbf.p, 0, sizeof(LbfDev)));
    if (r->exec) {
        cudaGraphExecDestroy(r->exec);
        r->exec = nullptr;
    }
    jcde_status st = ensure_order_buffers(r, p->n_candidates);
    if (st) return st;
    if (!r->side) CUDA_TRY(cudaStreamCreateWithFlags(&r->side, cudaStreamNonBlocking));
    if (!r->ev_fork) CUDA_TRY(cudaEventCreateWithFlags(&r->ev_fork, cudaEventDisableTiming));
    if (!r->ev_join) CUDA_TRY(cudaEventCreateWithFlags(&r->ev_join, cudaEventDisableTiming));
    r->lbf_ready = true;
    return JCDE_OK;
}

jcde_status jcde_lbf_steps(jcde_resident* r, uint32_t n_steps, uint32_t steps_per_graph, void* stream) {
    if (!r || !r->lbf_ready) return JCDE_ERR_STATE;
    cudaStream_t s = stream ? (cudaStream_t)stream : r->own;
    jcde_engine* e = r->e;
    const bool prof = e->prof;
    uint32_t done = 0;
    if (steps_per_graph > 0 && n_steps >= steps_per_graph) {
        if (!r->exec || r->exec_steps != steps_per_graph || r->exec_stream != s) {
            if (r->exec) {
                cudaGraphExecDestroy(r->exec);
                r->exec = nullptr;
            }
            cudaGraph_t g = nullptr;
            if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return JCDE_ERR_CUDA;
            const uint64_t before = r->launches;
            e->prof = false;   // per-kernel events are not recorded inside graphs
            // every graph launch is self-contained: its first step draws its own candidates and its
            // last step draws none ahead
            for (uint32_t i = 0; i < steps_per_graph; i++) lbf_step(r, s, i, i + 1 < steps_per_graph);
            e->prof = prof;
            r->exec_launches = r->launches - before;   // kernels per graph launch
            r->launches = before;
            cudaError_t ce = cudaStreamEndCapture(s, &g);
            if (ce == cudaSuccess && g) ce = cudaGraphInstantiate(&r->exec, g, 0);
            if (g) cudaGraphDestroy(g);
            if (ce != cudaSuccess) {
                r->exec = nullptr;
                return JCDE_ERR_CUDA;
            }
            r->exec_steps = steps_per_graph;
            r->exec_stream = s;
        }
        for (; done + steps_per_graph <= n_steps; done += steps_per_graph) {
            if (cudaGraphLaunch(r->exec, s) != cudaSuccess) return JCDE_ERR_CUDA;
            r->launches += r->exec_launches;
        }
    }
    for (uint32_t i = 0; done < n_steps; done++, i++) lbf_step(r, s, i, done + 1 < n_steps);
    CUDA_TRY(cudaGetLastError());
    r->last = s;
    e->last_stream = s;
    e->have_last_stream = true;
    return JCDE_OK;
}

jcde_status jcde_lbf_read(jcde_resident* r, uint32_t* counts4, uint32_t* placements, uint32_t place_cap,
                          uint32_t* removals, uint32_t removal_cap, uint32_t* free_counts, uint32_t free_cap,
                          uint8_t* verdicts, uint64_t verdict_cap) {
    if (!r || !counts4) return JCDE_ERR_ARG;
    if (!r->lbf_ready) return JCDE_ERR_STATE;
    if (r->last) CUDA_TRY(cudaStreamSynchronize(r->last));
    LbfDev d{};
    CUDA_TRY(cudaMemcpy(&d, r->d_lbf.p, sizeof(LbfDev), cudaMemcpyDeviceToHost));
    counts4[0] = d.step;
    counts4[1] = d.n_placed;
    counts4[2] = d.n_removed;
    counts4[3] = d.n_live;
    if (placements && place_cap)
        CUDA_TRY(cudaMemcpy(placements, r->d_place.p, (size_t)std::min(place_cap, d.n_placed) * 32, cudaMemcpyDeviceToHost));
    if (removals && removal_cap)
        CUDA_TRY(cudaMemcpy(removals, r->d_remv.p, (size_t)std::min(removal_cap, d.n_removed) * 8, cudaMemcpyDeviceToHost));
    if (free_counts && free_cap)
        CUDA_TRY(cudaMemcpy(free_counts, r->d_free.p, (size_t)std::min(free_cap, d.step) * 4, cudaMemcpyDeviceToHost));
    if (verdicts && verdict_cap && r->lp.vlog_steps) {
        const uint64_t have = (uint64_t)std::min(d.step, r->lp.vlog_steps) * r->lp.n_cand;
        CUDA_TRY(cudaMemcpy(verdicts, r->d_vlog.p, std::min(verdict_cap, have), cudaMemcpyDeviceToHost));
    }
    RCtl c{};
    CUDA_TRY(cudaMemcpy(&c, r->t.ctl, sizeof(RCtl), cudaMemcpyDeviceToHost));
    return c.error ? JCDE_ERR_CAPACITY : JCDE_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Launch tuning (no counterpart in the reference).
// ---------------------------------------------------------------------------------------------
extern "C" {

jcde_status jcde_get_tuning(const jcde_engine* e, jcde_tuning* out) {
    if (!e || !out) return JCDE_ERR_ARG;
    *out = e->tune;
    return JCDE_OK;
}

jcde_status jcde_set_tuning(jcde_engine* e, const jcde_tuning* t) {
    if (!e || !t) return JCDE_ERR_ARG;
    const bool lanes = t->surrogate_lanes == 8 || t->surrogate_lanes == 16 || t->surrogate_lanes == 32;
    const bool tile = t->edge_tile == 4 || t->edge_tile == 8 || t->edge_tile == 16;
    if (!lanes || !tile || t->staging_depth > MAX_STAGING_DEPTH) return JCDE_ERR_ARG;
    e->tune = *t;
    return JCDE_OK;
}

// Times every combination of the launch choices on the caller's batch (one warm-up, then the median
// of three timed runs each, CUDA events on `stream`), checks that all of them give the same
// verdicts, keeps the fastest in the engine and returns it.
// The autotuners time every choice from a cold L2, as a fresh batch meets it: before each timed
// repetition a buffer larger than L2 is written on the stream (outside the timed events).
static constexpr size_t TUNE_FLUSH_BYTES = 256u << 20;
static jcde_status tune_flush(DevBuf& f, cudaStream_t s) {
    if (!f.p) return JCDE_OK;   // no buffer (allocation refused): timed warm
    return cudaMemsetAsync(f.p, 0, f.cap, s) == cudaSuccess ? JCDE_OK : JCDE_ERR_CUDA;
}

jcde_status jcde_autotune(jcde_engine* e, const jcde_query* d_queries, uint32_t n, const jcde_filter* f, void* stream,
                          jcde_tuning* out, double* best_ms) {
    if (!e || !d_queries || !n) return JCDE_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const jcde_tuning saved = e->tune;
    DevBuf d_ref, d_out, d_flush;
    if (!d_ref.ensure(n) || !d_out.ensure(n)) return JCDE_ERR_CUDA;
    d_flush.ensure(TUNE_FLUSH_BYTES);
    std::vector<uint8_t> ref(n), got(n);
    cudaEvent_t a = nullptr, b = nullptr;
    CUDA_TRY(cudaEventCreate(&a));
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        return JCDE_ERR_CUDA;
    }
    bool have_ref = false;
    // one choice: a warm-up, then the median of three runs from a cold L2; its verdicts must equal
    // the first choice's (launch choices never change a verdict)
    auto time_choice = [&](const jcde_tuning& t, double* ms_out) -> jcde_status {
        e->tune = t;
        float ms[3] = {0, 0, 0};
        jcde_status st = JCDE_OK;
        for (int r = -1; r < 3 && !st; r++) {
            if (r >= 0) st = tune_flush(d_flush, s);
            if (!st && r >= 0 && cudaEventRecord(a, s) != cudaSuccess) st = JCDE_ERR_CUDA;
            if (!st) st = launch_detect(e, 3, d_queries, n, f, d_out.as<uint8_t>(), s, RawShape{nullptr, 0, 0, 0, 0});
            if (!st && r >= 0 &&
                (cudaEventRecord(b, s) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess ||
                 cudaEventElapsedTime(&ms[r], a, b) != cudaSuccess))
                st = JCDE_ERR_CUDA;
        }
        if (st) return st;
        std::sort(ms, ms + 3);
        if (cudaMemcpy(have_ref ? got.data() : ref.data(), d_out.p, n, cudaMemcpyDeviceToHost) != cudaSuccess)
            return JCDE_ERR_CUDA;
        if (have_ref && std::memcmp(ref.data(), got.data(), n) != 0) return JCDE_ERR_STATE;
        have_ref = true;
        *ms_out = ms[1];
        return JCDE_OK;
    };
    jcde_status st = JCDE_OK;
    jcde_tuning best = saved;
    double best_t = 1e300;
    const uint32_t all = 0xFFFFFFFFu;
    // 1. launch shapes: surrogate pass warp/thread x polygon pass leaf tables / grabs of 1, 2, 4 x order
    for (int sm = 0; sm < 2 && !st; sm++)
        for (int pm = 0; pm < 4 && !st; pm++)
            for (int om = 0; om < 2 && !st; om++) {
                jcde_tuning t = saved;
                t.surrogate_warp_max = sm == 0 ? all : 0u;
                t.leaf_table_max = pm == 0 ? all : 0u;
                t.poly_chunk = pm == 0 ? 1u : (1u << (pm - 1));
                t.order_min_batch = om == 0 ? 0u : all;
                double ms = 0;
                if ((st = time_choice(t, &ms))) break;
                if (ms < best_t) {
                    best_t = ms;
                    best = t;
                }
            }
    // 2-4. with that shape: the edge tile, the staging depth (large-batch polygon kernel only) and the
    // lanes per query of the warp surrogate pass (when that pass is chosen), one knob at a time
    auto try_knob = [&](uint32_t jcde_tuning::*field, const uint32_t* values, int count) {
        for (int k = 0; k < count && !st; k++) {
            if (best.*field == values[k]) continue;
            jcde_tuning t = best;
            t.*field = values[k];
            double ms = 0;
            if ((st = time_choice(t, &ms))) return;
            if (ms < best_t) {
                best_t = ms;
                best = t;
            }
        }
    };
    const uint32_t tiles[3] = {4, 8, 16}, depths[5] = {0, 1, 2, 3, 4}, lanes[3] = {8, 16, 32};
    if (!st) try_knob(&jcde_tuning::edge_tile, tiles, 3);
    if (!st && best.leaf_table_max == 0u) try_knob(&jcde_tuning::staging_depth, depths, 5);
    if (!st && best.surrogate_warp_max == all) try_knob(&jcde_tuning::surrogate_lanes, lanes, 3);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    // thresholds of the winner, extended to every batch at least this large / at most this small
    if (!st) {
        if (best.surrogate_warp_max == all) best.surrogate_warp_max = std::max(n, saved.surrogate_warp_max);
        else best.surrogate_warp_max = std::min(n - 1, saved.surrogate_warp_max);
        if (best.leaf_table_max == all) best.leaf_table_max = std::max(n, saved.leaf_table_max);
        else best.leaf_table_max = std::min(n - 1, saved.leaf_table_max);
        if (best.order_min_batch == all) best.order_min_batch = std::max(n + 1, saved.order_min_batch);
        else best.order_min_batch = std::min(n, saved.order_min_batch);
    }
    e->tune = st ? saved : best;
    if (out) *out = e->tune;
    if (best_ms) *best_ms = st ? 0.0 : best_t;
    return st;
}

}  // extern "C"

extern "C" jcde_status jcde_multi_autotune(jcde_multi* m, const jcde_query* dq, const uint32_t* offsets,
                                           const jcde_filter* filters, uint8_t* d_out, void* stream, uint32_t* out3,
                                           double* best_ms) {
    if (!m || !offsets || !dq || !d_out) return JCDE_ERR_ARG;
    const uint32_t n = offsets[m->engines.size()];
    if (!n) return JCDE_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t saved_chunk = m->poly_chunk;
    const bool saved_ordered = m->ordered;
    std::vector<uint8_t> ref(n), got(n);
    DevBuf d_flush;
    d_flush.ensure(TUNE_FLUSH_BYTES);
    cudaEvent_t a = nullptr, b = nullptr;
    CUDA_TRY(cudaEventCreate(&a));
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        return JCDE_ERR_CUDA;
    }
    jcde_status st = JCDE_OK;
    double best_t = 1e300;
    uint32_t best_chunk = saved_chunk;
    bool best_ordered = saved_ordered, have_ref = false;
    std::vector<uint32_t> saved_tiles;
    for (jcde_engine* e : m->engines) saved_tiles.push_back(e->tune.edge_tile);
    uint32_t best_tile = saved_tiles.empty() ? EDGE_TILE_DEFAULT : saved_tiles[0];
    // grab sizes 1-8 x order on/off with the engines' edge tile; then, with the fastest, edge tiles of
    // 4, 8 and 16 for every engine
    for (int om = 0; om < 3 && !st; om++)
        for (uint32_t chunk = 1; chunk <= (om < 2 ? 8u : 16u) && !st; chunk *= (om < 2 ? 2u : 2u)) {
            uint32_t tile = 0;
            if (om < 2) {
                m->ordered = om == 0;
                m->poly_chunk = chunk;
            } else {   // chunk walks 1, 2, 4, 8, 16: the tiles 4, 8 and 16 (1 and 2 are skipped)
                if (chunk < 4) continue;
                tile = chunk;
                m->ordered = best_ordered;
                m->poly_chunk = best_chunk;
                for (jcde_engine* e : m->engines) e->tune.edge_tile = tile;
            }
            float ms[3] = {0, 0, 0};
            for (int r = -1; r < 3 && !st; r++) {
                if (r >= 0) st = tune_flush(d_flush, s);
                if (!st && r >= 0 && cudaEventRecord(a, s) != cudaSuccess) st = JCDE_ERR_CUDA;
                if (!st) st = jcde_multi_detect(m, dq, offsets, filters, d_out, s);
                if (!st && r >= 0 &&
                    (cudaEventRecord(b, s) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess ||
                     cudaEventElapsedTime(&ms[r], a, b) != cudaSuccess))
                    st = JCDE_ERR_CUDA;
            }
            if (st) break;
            std::sort(ms, ms + 3);
            if (cudaMemcpy(have_ref ? got.data() : ref.data(), d_out, n, cudaMemcpyDeviceToHost) != cudaSuccess) {
                st = JCDE_ERR_CUDA;
                break;
            }
            if (have_ref && std::memcmp(ref.data(), got.data(), n) != 0) {
                st = JCDE_ERR_STATE;   // launch choices must never change a verdict
                break;
            }
            have_ref = true;
            if (ms[1] < best_t) {
                best_t = ms[1];
                if (om < 2) {
                    best_chunk = chunk;
                    best_ordered = om == 0;
                } else {
                    best_tile = tile;
                }
            }
        }
    for (size_t k = 0; k < m->engines.size(); k++) m->engines[k]->tune.edge_tile = st ? saved_tiles[k] : best_tile;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    m->poly_chunk = st ? saved_chunk : best_chunk;
    m->ordered = st ? saved_ordered : best_ordered;
    if (m->exec && (m->poly_chunk != saved_chunk || m->ordered != saved_ordered)) {   // recapture next time
        cudaGraphExecDestroy(m->exec);
        m->exec = nullptr;
    }
    if (m->exec && !st) {   // a changed edge tile changes the views: recapture next time
        cudaGraphExecDestroy(m->exec);
        m->exec = nullptr;
    }
    if (out3) {
        out3[0] = m->poly_chunk;
        out3[1] = m->ordered ? 1u : 0u;
        out3[2] = st ? (saved_tiles.empty() ? EDGE_TILE_DEFAULT : saved_tiles[0]) : best_tile;
    }
    if (best_ms) *best_ms = st ? 0.0 : best_t;
    return st;
}

#ifdef JCDE_POLY_STATS
// The polygon pass's work counters (measurement builds only; see kernels.cuh).
extern "C" jcde_status jcde_poly_stats(unsigned long long* out16, int reset) {
    if (!out16) return JCDE_ERR_ARG;
    CUDA_TRY(cudaDeviceSynchronize());
    CUDA_TRY(cudaMemcpyFromSymbol(out16, g_poly_stats, 16 * sizeof(unsigned long long)));
    if (reset) {
        static const unsigned long long zero[16] = {};
        CUDA_TRY(cudaMemcpyToSymbol(g_poly_stats, zero, sizeof(zero)));
    }
    return JCDE_OK;
}
#endif
