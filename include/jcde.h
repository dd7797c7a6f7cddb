/*
 * jcde — C ABI of the GB300 collision detection engine for 2D irregular nesting.
 *
 * One jcde_engine replaces one jagua-rs `CDEngine` (jagua-rs/src/collision_detection/cd_engine.rs:22-31):
 * it owns the hazard registry, the quadtree (kept on the host and mirrored into device memory as a
 * flat structure of arrays) and the item shapes with their surrogates.  Queries run as sm_103a
 * kernels; every verdict and every collected hazard set equals the reference's f32 answer.
 *
 * Conventions
 *   - every entry point returns a jcde_status (0 = JCDE_OK) and never aborts the process;
 *   - hazard keys are dense uint32 slots (the reference's slotmap HazKey, hazards/hazard.rs:8-11);
 *     a freed key is reused last-in first-out;
 *   - a jcde_query carries the transformation as matrix entries (cos, sin, tx, ty) — the matrix
 *     [[cos, -sin, tx], [sin, cos, ty]] of rot_transl_m (geometry/transformation.rs:475-483), which
 *     is what the reference's CDE consumes (`&Transformation`); sin/cos are the caller's;
 *   - `stream` arguments are cudaStream_t values passed as void* (NULL = legacy default stream);
 *     "device" pointers must be CUDA device (or managed) memory, "host" pointers plain host memory;
 *   - mutations (register / deregister / restore) must not overlap queries on the same engine, and
 *     query batches of one engine must not overlap each other on the GPU (they share the engine's
 *     scratch buffers): issue them on one stream, or synchronise between streams.
 */
#ifndef JCDE_H
#define JCDE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t jcde_status;
#define JCDE_OK 0
#define JCDE_ERR_ARG (-1)        /* invalid argument (null pointer, bad size, bad polygon, ...) */
#define JCDE_ERR_CUDA (-2)       /* a CUDA runtime call failed */
#define JCDE_ERR_CAPACITY (-3)   /* an output buffer is too small; sizes are reported */
#define JCDE_ERR_NOT_FOUND (-4)  /* unknown hazard key / entity / item */
#define JCDE_ERR_TIMEOUT (-5)    /* a bounded device wait gave up */
#define JCDE_ERR_STATE (-6)      /* engine in a state that forbids the call */

/* query verdicts */
#define JCDE_FREE 0u       /* no collision */
#define JCDE_COLLIDES 1u   /* collision */
#define JCDE_INVALID 2u    /* the query names an unknown item */

/* HazardEntity kinds (collision_detection/hazards/hazard.rs:38-51); Exterior has exterior scope */
#define JCDE_PLACED_ITEM 0
#define JCDE_EXTERIOR 1
#define JCDE_HOLE 2
#define JCDE_QUALITY_ZONE 3

typedef struct jcde_engine jcde_engine;
typedef struct jcde_snapshot jcde_snapshot;

typedef struct { float x_min, y_min, x_max, y_max; } jcde_rect;   /* Rect (primitives/rect.rs:12-19) */

/* CDEConfig (cd_engine.rs:346-353) incl. SPSurrogateConfig (fail_fast/sp_surrogate.rs:120-131) */
typedef struct {
    uint8_t quadtree_depth;        /* <= 15 */
    uint8_t cd_threshold;
    uint8_t reserved[2];
    uint32_t n_pole_limits;        /* entries used in pole_limit_n / pole_limit_coverage (<= 3) */
    uint32_t pole_limit_n[3];
    float pole_limit_coverage[3];
    uint32_t n_ff_poles;
    uint32_t n_ff_piers;
} jcde_config;

/* Hazard (hazards/hazard.rs:16-23): entity kind + final shape.  `xy` holds n_vertices (x, y)
 * pairs, `poi` the shape's pole of inaccessibility (x, y, r) — SPolygon::poi — used by the
 * containment test (cd_engine.rs:231-255).  `tag` identifies the entity for deregistration by
 * entity (cd_engine.rs:72-85); `dynamic` marks hazards that snapshots track (cd_engine.rs:98-106). */
typedef struct {
    int32_t kind;
    int32_t dynamic;
    const float* xy;
    uint32_t n_vertices;
    float poi[3];
    uint64_t tag;
} jcde_hazard;

/* One candidate placement: item type + transformation matrix entries (20 bytes, packed). */
#pragma pack(push, 1)
typedef struct {
    uint32_t item;
    float cos_r, sin_r, tx, ty;
} jcde_query;
#pragma pack(pop)

/* HazKeyFilter (hazards/filter.rs:13-48); n_ignored == 0 is NoFilter (filter.rs:58-65). */
typedef struct {
    const uint32_t* ignored;
    uint32_t n_ignored;
} jcde_filter;

const char* jcde_status_string(jcde_status s);
/* default CDEConfig of lbf (lbf/src/config.rs:37-45): depth 5, threshold 16, poles (100,0),(20,.75),(10,.9), 2 ff poles, 0 piers */
void jcde_default_config(jcde_config* out);

/* --- engine lifetime: CDEngine::new (cd_engine.rs:34-56) ------------------------------------ */
jcde_status jcde_create(const jcde_config* cfg, jcde_rect bbox, const jcde_hazard* static_hazards,
                        uint32_t n_static, jcde_engine** out);
void jcde_destroy(jcde_engine* e);
jcde_status jcde_bbox(const jcde_engine* e, jcde_rect* out);                     /* cd_engine.rs:329-331 */

/* --- hazards --------------------------------------------------------------------------------- */
jcde_status jcde_register_hazard(jcde_engine* e, const jcde_hazard* h, uint32_t* out_key);  /* cd_engine.rs:59-70 */
jcde_status jcde_deregister_hazard(jcde_engine* e, uint32_t key);                            /* cd_engine.rs:87-96 */
jcde_status jcde_deregister_hazard_by_entity(jcde_engine* e, int32_t kind, uint64_t tag,
                                             uint32_t* out_key);                             /* cd_engine.rs:72-85 */
jcde_status jcde_n_hazard_slots(const jcde_engine* e, uint32_t* out);

/* --- items: shape_cd + surrogate of an Item (entities/item.rs:27-48) -------------------------- */
/* poles_xyr: all surrogate poles (x, y, r), poles[0] = poi; the first cfg.n_ff_poles are probed
 * (sp_surrogate.rs:55-57).  piers_xyxy: ff piers (sp_surrogate.rs:59-61), may be NULL. */
jcde_status jcde_register_item(jcde_engine* e, const float* xy, uint32_t n_vertices, const float poi[3],
                               const float* poles_xyr, uint32_t n_poles, const float* piers_xyxy,
                               uint32_t n_piers, uint32_t* out_item);

/* --- batched queries (device buffers, stream ordered) ----------------------------------------- */
/* verdict[i] = detect_surrogate_collision(item.surrogate, T_i) || detect_poly_collision(T_i(item.shape))
 * (cd_engine.rs:204-223 then :160-197, in the protocol of lbf/benches/ci_bench.rs:107-121). */
jcde_status jcde_detect_batch(jcde_engine* e, const jcde_query* d_queries, uint32_t n,
                              const jcde_filter* filter, uint8_t* d_verdicts, void* stream);
/* Surrogate-only and polygon-only halves of the verdict (cd_engine.rs:204-223 / :160-197). */
jcde_status jcde_detect_surrogate_batch(jcde_engine* e, const jcde_query* d_queries, uint32_t n,
                                        const jcde_filter* filter, uint8_t* d_verdicts, void* stream);
jcde_status jcde_detect_poly_batch(jcde_engine* e, const jcde_query* d_queries, uint32_t n,
                                   const jcde_filter* filter, uint8_t* d_verdicts, void* stream);
/* Same as jcde_detect_batch with host buffers: copies in, kernel, copies out, synchronises. */
jcde_status jcde_detect_batch_host(jcde_engine* e, const jcde_query* h_queries, uint32_t n,
                                   const jcde_filter* filter, uint8_t* h_verdicts);

/* All colliding hazards per query: collect_surrogate_collisions then collect_poly_collisions into
 * one collector (cd_engine.rs:296-310, :261-289; lbf/benches/ci_bench.rs:56-68).  A filter acts as
 * keys pre-seeded into the collector (hazards/filter.rs:69-76): they are skipped and not reported.
 * Keys of query i are d_ids[d_offsets[i] .. d_offsets[i] + d_counts[i]), ascending.  The order of
 * the per-query runs inside d_ids is unspecified.  *d_total receives the number of keys needed; if
 * it exceeds ids_cap, runs that did not fit are not written (d_counts still holds their sizes) and
 * the host entry point returns JCDE_ERR_CAPACITY. */
jcde_status jcde_collect_batch(jcde_engine* e, const jcde_query* d_queries, uint32_t n,
                               const jcde_filter* filter, uint32_t* d_offsets, uint32_t* d_counts,
                               uint32_t* d_ids, uint32_t ids_cap, uint32_t* d_total, void* stream);

/* --- filtered detect that allocates nothing -------------------------------------------------- */
/* No counterpart in the reference.  Same verdicts as jcde_detect_batch (device buffers, stream
 * ordered), for callers that may not allocate device memory during a query: jcde_detect_batch
 * allocates a device bitmask and a per-node table the first time it sees a filter, and cudaMalloc
 * synchronizes the whole device and needs free memory — which a caller whose GPU memory is all
 * owned by its own pool, or that runs queries on a latency-critical stream next to other work,
 * cannot accept.  This entry point keeps the two passes' work counters, the filter's bitmask and
 * the per-node table in one static device array of JCDE_NOALLOC_SCRATCH_BYTES that every GPU
 * loading the library holds until the process exits; it returns JCDE_ERR_CAPACITY when
 * 256 B + n_slots / 8 B + one byte per quadtree node (each part rounded up to 256 B) exceed it,
 * i.e. for engines of more than about 8 million hazard slots or 1 million nodes.  The ignored keys
 * are turned into the bitmask on the host during the call and handed to the GPU by value in launch
 * parameters, so the caller's key array may be reused as soon as the call returns, and its length
 * costs no device memory.  Every call shares the array and leaves its contents behind, so calls
 * that overlap on the GPU (another stream, another thread) race on it.  The engine's device copy
 * must be current: after a register / deregister / restore / register_item, run any other query
 * first (jcde_detect_batch with n = 0 suffices), else JCDE_ERR_STATE.  That first query of the
 * engine also looks up the array's device address and loads this entry point's kernels on the
 * current device (a call on a device where that has not happened does it itself; make such a call
 * before any stream capture).  A cudaDeviceReset while the library is loaded is not supported.
 * Visit ordering, whose buffers grow with the batch, is not used, so batches at or above the
 * engine's order_min_batch (jcde_tuning; 4,096 by default) run somewhat slower than through
 * jcde_detect_batch. */
#define JCDE_NOALLOC_SCRATCH_BYTES 1048576u
jcde_status jcde_detect_batch_noalloc(jcde_engine* e, const jcde_query* d_queries, uint32_t n,
                                      const jcde_filter* filter, uint8_t* d_verdicts, void* stream);

/* --- several layouts in one launch sequence (no counterpart in the reference) ------------------- */
/* A jcde_multi groups engines (one per layout, e.g. the bins of a bin-packing problem, each a
 * Layout with its own CDEngine, entities/layout.rs:14-21) so that one ordering + surrogate +
 * polygon launch sequence answers all their batches: d_queries holds layout l's queries at
 * [offsets[l], offsets[l+1]) (offsets: host array of n+1), filters is an array of n filters or
 * NULL, d_verdicts one slot per query.  Verdicts equal those of jcde_detect_batch per engine.  The
 * engines are borrowed; destroy the group before them.  The _graph variant captures the sequence
 * into a CUDA graph on first use and replays it while the engines' device images, offsets, filters,
 * buffers and stream stay the same (the stream must not be the legacy default stream). */
typedef struct jcde_multi jcde_multi;
jcde_status jcde_multi_create(jcde_engine* const* engines, uint32_t n, jcde_multi** out);
void jcde_multi_destroy(jcde_multi* m);
jcde_status jcde_multi_detect(jcde_multi* m, const jcde_query* d_queries, const uint32_t* offsets,
                              const jcde_filter* filters, uint8_t* d_verdicts, void* stream);
jcde_status jcde_multi_detect_graph(jcde_multi* m, const jcde_query* d_queries, const uint32_t* offsets,
                                    const jcde_filter* filters, uint8_t* d_verdicts, void* stream);
uint64_t jcde_multi_kernel_launches(const jcde_multi* m);

/* --- single queries with the reference's signatures (host buffers, synchronous) -------------- */
/* detect_poly_collision (cd_engine.rs:160-197) of an already transformed shape with its poi. */
jcde_status jcde_detect_poly(jcde_engine* e, const float* xy, uint32_t n_vertices, const float poi[3],
                             const jcde_filter* filter, uint8_t* out);
/* detect_surrogate_collision (cd_engine.rs:204-223) of an item's surrogate under a transformation. */
jcde_status jcde_detect_surrogate(jcde_engine* e, uint32_t item, const float transform[4],
                                  const jcde_filter* filter, uint8_t* out);
/* collect_poly_collisions (cd_engine.rs:261-289); *n_out receives the count (even when > cap). */
jcde_status jcde_collect_poly(jcde_engine* e, const float* xy, uint32_t n_vertices, const float poi[3],
                              const jcde_filter* filter, uint32_t* keys, uint32_t cap, uint32_t* n_out);
/* collect_surrogate_collisions (cd_engine.rs:296-310). */
jcde_status jcde_collect_surrogate(jcde_engine* e, uint32_t item, const float transform[4],
                                   const jcde_filter* filter, uint32_t* keys, uint32_t cap, uint32_t* n_out);

/* --- differentiable pole-overlap proxy (no counterpart in the reference) -------------------- */
/* For a candidate (theta, tx, ty) of an item with surrogate poles p_i (all of them, poles[0] = poi;
 * fail_fast/sp_surrogate.rs:19) placed at c_i = R(theta) p_i + t, and the poles (c_j, r_j) given to the
 * hazards with jcde_set_hazard_poles (a placed item's are its item's poles under its placement,
 * as SPolygon::transform moves the surrogate, simple_polygon.rs:214-216):
 *     P = sum_ij max(0, r_i + r_j - |c_i - c_j|)^2,   grad = dP/d(theta, tx, ty)
 * in float32.  Hazards ignored by the filter contribute nothing.  Params are 3 floats per candidate
 * (theta, tx, ty); grad is 3 floats per candidate in the same order. */
jcde_status jcde_set_hazard_poles(jcde_engine* e, uint32_t key, const float* poles_xyr, uint32_t n);
jcde_status jcde_proxy_batch(jcde_engine* e, const float* d_params, const uint32_t* d_items, uint32_t n,
                             const jcde_filter* filter, float* d_value, float* d_grad, void* stream);
/* The same as a forward / backward pair (the two halves of a torch.autograd.Function): forward
 * writes P; backward writes dL/d(theta, tx, ty) = d_grad_value[i] * dP_i/d(theta, tx, ty) (upstream
 * gradient per candidate; null = all ones). */
jcde_status jcde_proxy_forward(jcde_engine* e, const float* d_params, const uint32_t* d_items, uint32_t n,
                               const jcde_filter* filter, float* d_value, void* stream);
jcde_status jcde_proxy_backward(jcde_engine* e, const float* d_params, const uint32_t* d_items, uint32_t n,
                                const jcde_filter* filter, const float* d_grad_value, float* d_grad_params,
                                void* stream);
/* `steps` descent steps per candidate on P: a step tries t - eta*step_t*dP/dt and
 * theta - eta*step_th/max|p_i|^2*dP/dtheta, keeps it if P drops (eta x1.5, at most 4) and halves eta
 * otherwise (eta starts at 1), stopping once P = 0.  `clearance` grows every hazard pole's radius
 * during the descent (poles under-cover a shape, so separating them by a clearance frees more
 * placements; 0 descends on P itself).  Params are updated in place, d_queries receives
 * the final placements as query records (cos, sin of the final theta) ready for jcde_detect_batch,
 * d_value the final P. */
jcde_status jcde_separate_batch(jcde_engine* e, float* d_params, const uint32_t* d_items, uint32_t n,
                                uint32_t steps, float step_t, float step_th, float clearance,
                                const jcde_filter* filter, jcde_query* d_queries, float* d_value, void* stream);
/* Random-resampling baseline: k Gaussian perturbations (sigma_t in translation, sigma_th in
 * rotation) of each candidate, as query records d_queries[i * k + j]. */
jcde_status jcde_resample_batch(jcde_engine* e, const float* d_params, const uint32_t* d_items, uint32_t n,
                                uint32_t k, float sigma_t, float sigma_th, uint32_t seed, jcde_query* d_queries,
                                void* stream);

/* --- LBF choice of a candidate batch (lbf/src/opt/search.rs:44-66, LBFLoss lbf/src/opt/loss.rs) -- */
/* Among queries whose verdict is JCDE_FREE: the smallest cost x_max * 10 + y_max of the transformed
 * shape's bounding box, lowest index among equal costs.  *d_best (device) receives
 * (order-preserving cost bits << 32) | index, or all ones when no candidate is free. */
jcde_status jcde_lbf_select(jcde_engine* e, const jcde_query* d_queries, const uint8_t* d_verdicts, uint32_t n,
                            uint64_t* d_best, void* stream);
/* jcde_lbf_select for n_segments batches of n queries each, back to back (d_queries + k n,
 * d_verdicts + k n): d_best[k] is segment k's choice (index within the segment), in one launch.
 * The engine supplies the item shapes only. */
jcde_status jcde_lbf_select_segments(jcde_engine* e, const jcde_query* d_queries, const uint8_t* d_verdicts,
                                     uint32_t n, uint32_t n_segments, uint64_t* d_best, void* stream);
/* n candidate placements of one item drawn on the device from the counter-based stream (seed, sid)
 * — the generator of the LBF build's uniform round (no counterpart in the reference, whose samplers
 * draw from its own RNG, lbf/src/samplers/uniform_rect_sampler.rs): draw n+i gives the rotation (a
 * turn u in [0, 1), or one of the n_orient allowed (cos, sin) pairs of d_orient by the draw modulo
 * n_orient), draws 2n+i and 3n+i the translation, uniform over `box`.  d_turns (may be NULL) gets
 * each candidate's u (0 for allowed orientations).  Device buffers, stream ordered. */
jcde_status jcde_gen_candidates(uint64_t seed, uint64_t sid, uint32_t n, uint32_t item, jcde_rect box,
                                const float* d_orient, uint32_t n_orient, jcde_query* d_queries, double* d_turns,
                                void* stream);
/* The same for n_segments streams at once: segment k draws n candidates from stream (seed, sids[k])
 * over boxes[k] (host arrays) into d_queries + k n and d_turns + k n — one launch per 64 segments. */
jcde_status jcde_gen_candidates_segments(uint64_t seed, const uint64_t* sids, const jcde_rect* boxes,
                                         uint32_t n_segments, uint32_t n, uint32_t item, const float* d_orient,
                                         uint32_t n_orient, jcde_query* d_queries, double* d_turns, void* stream);

/* --- Device-resident engine: register / deregister on the GPU ---------------------------------
 * A copy of an engine's quadtree in device pools that single-warp kernels update in place,
 * restating QTNode::register_hazard / deregister_hazard (quadtree/qt_node.rs:38-94) and
 * QTHazard::constrict (quadtree/qt_hazard.rs:48-167) on the device.  Every call is stream-ordered
 * and asynchronous (no host round trip), so a whole query -> choose -> register loop can be
 * captured in one CUDA graph.  Keys follow the host engine's rule (a freed key is reused
 * last-in first-out).  The resident copy shares the engine's items and staging buffers: it is
 * created from the engine's current hazards, and while it is in use the engine's own query calls
 * must not overlap it on the GPU.  Capacities are fixed at creation; exceeding one sets a sticky
 * error (jcde_resident_status returns JCDE_ERR_CAPACITY) and further updates are skipped.  Destroy
 * the resident copy before its engine; the engine's items must not change while it exists. */
typedef struct jcde_resident jcde_resident;
typedef struct jcde_resident_config {
    uint32_t max_nodes;             /* 0: every node of a full tree of the engine's depth */
    uint32_t max_entries;           /* hazard entries over all nodes (slabs, grown by doubling) */
    uint32_t max_edges;             /* clipped edges over all Partial entries */
    uint32_t max_hazard_vertices;   /* vertices of all hazards ever registered */
    uint32_t max_keys;              /* hazard keys */
    uint32_t max_tasks;             /* work stack of one update */
} jcde_resident_config;
void jcde_resident_default_config(jcde_resident_config* c);
jcde_status jcde_resident_create(jcde_engine* e, const jcde_resident_config* cfg, jcde_resident** out);
void jcde_resident_destroy(jcde_resident* r);
/* Back to a copy of the engine's current hazards (pools emptied, keys as the engine's); synchronises.
 * *h2d_bytes (may be null) receives the bytes uploaded. */
jcde_status jcde_resident_reset(jcde_resident* r, uint64_t* h2d_bytes);
/* Layout::place_item (entities/layout.rs:73-85): PlacedItem::new of item d_query->item under the
 * query's transformation, then CDEngine::register_hazard (cd_engine.rs:59-70).  *d_key (device,
 * may be null) receives the key, ~0 on failure. */
jcde_status jcde_resident_register_placed(jcde_resident* r, const jcde_query* d_query, uint32_t* d_key, void* stream);
/* CDEngine::deregister_hazard_by_key (cd_engine.rs:87-96) of the key at d_key (device); unknown keys are
 * counted (status word 1) and ignored. */
jcde_status jcde_resident_deregister(jcde_resident* r, const uint32_t* d_key, void* stream);
/* jcde_detect_batch (surrogate pass, then polygon pass) against the resident tree, no filter. */
jcde_status jcde_resident_detect_batch(jcde_resident* r, const jcde_query* d_queries, uint32_t n, uint8_t* d_out,
                                       void* stream);
/* Synchronises; out8 = error, unknown-key count, live hazards, key slots, node pool high-water mark,
 * entry / edge / hazard-vertex pool use. */
jcde_status jcde_resident_status(jcde_resident* r, uint32_t* out8);
/* Synchronises; the canonical form of jcde_tree_dump for the resident tree. */
jcde_status jcde_resident_tree_dump(jcde_resident* r, uint32_t* out, uint64_t cap, uint64_t* n_words);
uint64_t jcde_resident_kernel_launches(const jcde_resident* r);

/* --- LBF-style build on the device (lbf/src/opt/search.rs:17-106, restated) ----------------------
 * Step s: item type t = draw s of stream (seed, 2) mod n_types; n_candidates placements of t with
 * rotation ~ U[0, 2pi) and translation ~ U(sample_box) from stream (seed, 10000 + s) (draw n+i, 2n+i,
 * 3n+i of candidate i); verdicts by the surrogate and polygon passes; the free candidate of least
 * LBFLoss cost (lbf/src/opt/loss.rs:29-31, lowest index on ties) is registered; after every
 * remove_every-th step the placed item at position (draw k of stream (seed, 4)) mod live of the
 * placement list is deregistered (k = removals so far).  Streams: SplitMix64 counter-based draws,
 * mix(key ^ mix(i)) with key = mix(seed * 0x100000001B3 + sid * 0x9E3779B97F4A7C15).
 * No host round trip per step; steps_per_graph > 0 replays that many steps per CUDA graph launch. */
typedef struct jcde_lbf_params {
    uint64_t seed;
    uint32_t n_candidates;         /* per step, over the uniform rounds */
    uint32_t n_types;              /* item types 0..n_types-1 of the engine */
    uint32_t remove_every;         /* 0: no removals */
    uint32_t max_steps;            /* log capacity; steps beyond it do nothing */
    uint32_t verdict_log_steps;    /* keep the verdicts of the first steps (0: none; needs one round per step) */
    /* the uniform phase of lbf's search (search.rs:41-66) in rounds of n_candidates / uniform_rounds
     * (0 counts as 1): round 0 from stream (seed, 10000 + s), round u >= 1 from stream
     * (seed, 2000000 + 64 s + u) over the sample box with x_max tightened to the step's best cost so
     * far / 10 (LBFLoss::tighten_sample_bbox, loss.rs:34-44, after every improvement in search.rs:62-63,
     * here after every round); draws i: item (unused), n+i: rotation, 2n+i: x, 3n+i: y */
    uint32_t uniform_rounds;
    jcde_rect sample_box;
    /* local search after the uniform rounds (search.rs:80-101): round r = 1..ls_rounds draws
     * ls_candidates placements of the step's item around the step's best so far from stream
     * (seed, 1000000 + 64 s + r) with Normal offsets (a Box-Muller pair of draws i, m+i for x and y,
     * another of draws 2m+i, 3m+i for the rotation, m = ls_candidates): translation deviation
     * ls_sigma_t[r-1], rotation deviation ls_sigma_turns[r-1] (in turns; LSSampler's decaying
     * deviations, ls_sampler.rs:84-90, one value per round); the round's least-cost free candidate
     * replaces the best when it costs strictly less. */
    uint32_t ls_rounds;            /* 0..8 */
    uint32_t ls_candidates;        /* per round, at most n_candidates */
    float ls_sigma_t[8];
    double ls_sigma_turns[8];
    /* instance mode (both optional, host arrays copied at jcde_lbf_begin): the item of step s is
     * item_sequence[s] instead of a type-stream draw; item t rotates to one of its allowed
     * orientations orientation_cs[2 * (offsets[t] + k)..] (cos, sin), k = (draw n+i) mod count, or
     * continuously when offsets[t + 1] == offsets[t]; local-search rounds keep a discrete
     * orientation.  (lbf/src/opt/lbf_spp.rs:37-123 places the instance's items in this order.) */
    const uint32_t* item_sequence;
    uint32_t n_sequence;           /* at least max_steps */
    uint32_t n_orientation_items;  /* the engine's item count when orientation_offsets is given */
    const uint32_t* orientation_offsets;   /* n_items + 1 */
    const float* orientation_cs;
} jcde_lbf_params;
jcde_status jcde_lbf_begin(jcde_resident* r, const jcde_lbf_params* p);
jcde_status jcde_lbf_steps(jcde_resident* r, uint32_t n_steps, uint32_t steps_per_graph, void* stream);
/* Synchronises.  counts4 = steps done, placements, removals, placed items still live.  placements:
 * 8 words each (step, key, round << 24 | candidate, item, cos, sin, tx, ty as float bits); removals: 2 words each
 * (step, key); free_counts: per step, the candidates the surrogate pass left to the polygon pass
 * (all rounds); verdicts: step-major verdict log.  Without a verdict log the polygon pass only
 * judges candidates that could still beat the step's best free one (search.rs:52-56), which
 * changes no placement. */
jcde_status jcde_lbf_read(jcde_resident* r, uint32_t* counts4, uint32_t* placements, uint32_t place_cap,
                          uint32_t* removals, uint32_t removal_cap, uint32_t* free_counts, uint32_t free_cap,
                          uint8_t* verdicts, uint64_t verdict_cap);

/* --- Launch tuning (no counterpart in the reference) ---------------------------------------------
 * How the detect passes are launched for a batch of n queries.  None of these choices changes a
 * verdict.  Defaults suit both a 1M-query batch and an LBF step of 16K candidates. */
typedef struct jcde_tuning {
    uint32_t surrogate_warp_max;   /* n <= this: one warp per query in the surrogate pass, else one thread */
    uint32_t leaf_table_max;       /* n <= this: polygon pass with per-query leaf tables, queries one by one */
    uint32_t poly_chunk;           /* otherwise: queries per counter grab in the polygon pass (0: grid stride) */
    uint32_t order_min_batch;      /* n >= this: queries visited in Morton order of their translation */
    uint32_t surrogate_lanes;      /* lanes per query in the warp surrogate pass: 8, 16 or 32 */
    uint32_t edge_tile;            /* edges per tile box a leaf test skips by (edge.rs:188-199): 4, 8 or 16 */
    uint32_t staging_depth;        /* top quadtree levels the large-batch polygon pass keeps in shared
                                      memory (0-4; levels whose nodes do not fit are left in global) */
} jcde_tuning;
jcde_status jcde_get_tuning(const jcde_engine* e, jcde_tuning* out);
jcde_status jcde_set_tuning(jcde_engine* e, const jcde_tuning* t);
/* Times, on the caller's batch, all 16 launch shapes (surrogate pass warp/thread x polygon pass leaf
 * tables/grabs of 1, 2, 4 x Morton order on/off), then with the fastest the edge tiles 4/8/16, the
 * staging depths 0-4 (when the large-batch polygon pass is chosen) and 8/16/32 lanes per query (when
 * the warp surrogate pass is chosen), one knob at a time; checks that every choice gives the same
 * verdicts (JCDE_ERR_STATE otherwise), keeps the fastest in the engine (its thresholds set so that
 * batches of this size take it) and returns it with its median time.  Each timing starts from a
 * cold L2 (a 256 MB buffer, allocated for the call, is written before it), as a fresh batch would.
 * Synchronises. */
jcde_status jcde_autotune(jcde_engine* e, const jcde_query* d_queries, uint32_t n, const jcde_filter* f, void* stream,
                          jcde_tuning* out, double* best_ms);
/* The same for a jcde_multi batch: polygon-pass grabs of 1, 2, 4, 8 x Morton order on/off, then edge
 * tiles of 4, 8, 16 for every engine, verdicts checked identical, timed from a cold L2; d_out
 * (device, total queries) receives verdicts; out3 = chosen grab size, order flag, edge tile.  The
 * choice applies to later jcde_multi_detect / _graph calls (the edge tile is set in the engines).
 * Synchronises. */
jcde_status jcde_multi_autotune(jcde_multi* m, const jcde_query* d_queries, const uint32_t* offsets,
                                const jcde_filter* filters, uint8_t* d_out, void* stream, uint32_t* out3,
                                double* best_ms);

/* --- snapshots: CDEngine::save / restore (cd_engine.rs:98-149) ------------------------------- */
jcde_status jcde_save(const jcde_engine* e, jcde_snapshot** out);
jcde_status jcde_restore(jcde_engine* e, const jcde_snapshot* s);
void jcde_snapshot_free(jcde_snapshot* s);

/* --- shape preparation (host): SPolygon::new (simple_polygon.rs:41-71) and surrogate poles
 *     (fail_fast/pole.rs:12-47) — what Item::new / Container::new compute once per shape ------ */
/* xy_out: n_vertices (x, y) in internal counter-clockwise order; bbox_out[4]; area_diam[2]; poi[3]
 * (poi NULL: the poi is not computed, e.g. when jcde_poi_batch computes it on the device) */
jcde_status jcde_spolygon_new(const float* xy, uint32_t n_vertices, float* xy_out, float* bbox_out,
                              float* area_diam, float* poi);
/* jcde_spolygon_new without the poi for n shapes at once (host buffers): xy holds the shapes' (x, y)
 * vertices back to back, voff[n + 1] the offsets; xy_out the same layout in internal order, bbox_out
 * 4 per shape, area_diam 2 per shape, centroid_out (may be NULL) 2 per shape — SPolygon::centroid
 * (simple_polygon.rs:173-192) of the internal vertices, the importer's centring point
 * (io/import.rs:214-217) — and status[i] 0 or JCDE_ERR_ARG for an invalid polygon.  Shapes are
 * spread over n_threads host threads (0: one per hardware thread). */
jcde_status jcde_spolygon_batch(const float* xy, const uint32_t* voff, uint32_t n, float* xy_out, float* bbox_out,
                                float* area_diam, float* centroid_out, int32_t* status, uint32_t n_threads);
/* close_narrow_concavities (geometry/shape_modification.rs:374-478) of a shape after SPolygon::new
 * (host): deflate 0 = ShapeModifyMode::Inflate, 1 = Deflate; ratio = the cutoff as a fraction of the
 * diameter (lbf's default config: 0.01, applied between a simplification and one at a tenth of its
 * tolerance, original_shape.rs:33-42).  xy_out holds up to n_vertices (x, y); *n_out the count. */
jcde_status jcde_close_concavities(const float* xy, uint32_t n_vertices, int deflate, float ratio, float* xy_out,
                                   uint32_t* n_out);
/* poles of an internal shape with the given area and poi; *n_out receives the count (even when > cap) */
jcde_status jcde_surrogate_poles(const float* xy, uint32_t n_vertices, float area, const float poi[3],
                                 const jcde_config* cfg, float* poles_xyr, uint32_t cap, uint32_t* n_out);

/* --- shape preparation on the device, many shapes per call (no counterpart in the reference: the
 *     reference runs compute_pole, fail_fast/pole.rs:52-77, once per shape on the host).  The same
 *     poles as jcde_spolygon_new / jcde_surrogate_poles, bit for bit.  Device buffers, stream
 *     ordered: d_xy holds every shape's (x, y) vertices back to back (the internal counter-clockwise
 *     order), d_voff[n_shapes + 1] the vertex offsets, max_vertices bounds every shape's count.
 *     d_status[i] is written per shape: 0 ok, 1 invalid shape (fewer than 3 or more than
 *     max_vertices vertices), 2 no pole found, 3 a thousand poles reached (pole.rs:42-45), 4 a level of
 *     the cell tree wider than the device lists hold, 5 more poles than `cap`.  d_order (may be NULL: batch
 *     order) is a permutation of the shapes giving the order CTAs take them in; larger shapes first
 *     (e.g. by descending vertex count) shortens the tail of a batch.  d_workspace may be NULL
 *     (allocated per call, stream ordered) or hold jcde_poles_workspace_bytes bytes, 256-byte aligned. */
uint64_t jcde_poles_workspace_bytes(uint32_t n_shapes, uint32_t max_vertices, int with_poles);
/* simplify_shape (geometry/shape_modification.rs:48-144) of each shape up to its final
 * SPolygon::new: d_area the shape's area, deflate 0 = ShapeModifyMode::Inflate (items), 1 = Deflate
 * (container outers), tolerance = max_area_change_ratio.  d_xy_out has the layout of d_xy (each
 * shape's simplified vertices from its own offset on), d_n_out the simplified counts, d_status 0 or
 * 1 (invalid shape).  Items of lbf's default config are simplified with tolerance 0.001
 * (lbf/src/config.rs:42) before their poi and poles are computed (original_shape.rs:23-50). */
jcde_status jcde_simplify_batch(const float* d_xy, const uint32_t* d_voff, uint32_t n_shapes, uint32_t max_vertices,
                                const float* d_area, int deflate, float tolerance, float* d_xy_out, uint32_t* d_n_out,
                                int32_t* d_status, void* stream);
/* the pole of inaccessibility of each shape (SPolygon::calculate_poi, simple_polygon.rs:152-171):
 * d_poi n_shapes x (x, y, r) */
jcde_status jcde_poi_batch(const float* d_xy, const uint32_t* d_voff, uint32_t n_shapes, uint32_t max_vertices,
                           float* d_poi, int32_t* d_status, const uint32_t* d_order, void* d_workspace,
                           uint64_t workspace_bytes, void* stream);
/* generate_surrogate_poles (pole.rs:12-47) of each shape with its area (d_area) and poi (d_poi, 3 per
 * shape) under cfg's pole limits: d_poles n_shapes x cap x (x, y, r), pole 0 = the poi; d_n_out the
 * count per shape */
jcde_status jcde_surrogate_poles_batch(const float* d_xy, const uint32_t* d_voff, uint32_t n_shapes,
                                       uint32_t max_vertices, const float* d_area, const float* d_poi,
                                       const jcde_config* cfg, float* d_poles, uint32_t cap, uint32_t* d_n_out,
                                       int32_t* d_status, const uint32_t* d_order, void* d_workspace,
                                       uint64_t workspace_bytes, void* stream);

/* --- introspection (tests, tooling) ----------------------------------------------------------- */
/* canonical dump of the quadtree (pre-order, hazards by key, edges sorted); *n_words always set */
jcde_status jcde_tree_dump(const jcde_engine* e, uint32_t* out, uint64_t cap, uint64_t* n_words);
/* node count and flattened sizes currently mirrored on the device */
jcde_status jcde_device_stats(jcde_engine* e, uint64_t* out5);
/* number of kernels this engine has launched since creation (bench accounting) */
uint64_t jcde_kernel_launches(const jcde_engine* e);
/* Measurement helper (no counterpart in the reference): the L2 read bandwidth of the current device
 * in GB/s for a buffer of `bytes` (>= 1 MiB) that stays L2-resident, read `reps` times by a
 * hand-written streaming kernel (16-byte loads cached in L2 only), timed with CUDA events.  The
 * query kernels read their layout from L2, so this is their bandwidth ceiling.  Allocates and frees
 * its buffer; synchronizes the device. */
jcde_status jcde_l2_read_peak(uint64_t bytes, uint32_t reps, double* out_gbs);
/* Kernel timing (no counterpart in the reference): when enabled, every launch is bracketed by CUDA
 * events on its stream; jcde_profile_read synchronises on them and returns, per kind, the summed
 * milliseconds and launch counts (arrays of JCDE_PROF_KINDS), optionally resetting the totals. */
#define JCDE_PROF_SURROGATE 0   /* surrogate pass (detect) */
#define JCDE_PROF_POLY 1        /* polygon pass (detect) */
#define JCDE_PROF_COLLECT 2     /* collect kernel */
#define JCDE_PROF_ORDER 3       /* spatial ordering of a batch (3 small kernels) */
#define JCDE_PROF_FILTER 4      /* per-node presence under a new filter */
#define JCDE_PROF_PROXY 5       /* gradient-descent separation on the pole-overlap proxy */
#define JCDE_PROF_UPDATE 6      /* device-resident register / deregister (LBF commit) */
#define JCDE_PROF_LBF 7         /* LBF candidate generation and choice */
#define JCDE_PROF_KINDS 8
jcde_status jcde_profile_enable(jcde_engine* e, int enable);
jcde_status jcde_profile_read(jcde_engine* e, double* ms, uint64_t* count, int reset);

#ifdef __cplusplus
}
#endif
#endif /* JCDE_H */
