// Device-resident quadtree: the CDE's register / deregister run on the GPU.
//
// The image the query kernels walk (kernels.cuh: nodes, per-node hazard entries, edge lists,
// hazard table) lives in fixed-capacity pools in device memory and is updated in place by
// single-warp kernels that restate QTNode::register_hazard / deregister_hazard
// (collision_detection/quadtree/qt_node.rs:38-94) and QTHazard::constrict (qt_hazard.rs:48-167):
//   * nodes form a pool in which every quartet of children is contiguous and starts at 1 + 4k,
//     like the host tree's node pool; freed quartets are reused last-in first-out;
//   * each node owns a slab of entries (an unordered set: a node's answer does not depend on the
//     order of its hazards), doubled when full; removal swaps in the slab's last entry;
//   * every Partial entry owns its clipped edge list in the edge pool (a quadrant that keeps all of
//     its parent's edges shares the parent's list); edge lists are never moved;
//   * the strongest presence and the active-edge count of every node are kept up to date.
// Hazard keys follow the host registry: a freed key is reused last-in first-out (slotmap order).
//
// The same headers hold the device state of the LBF-style build (lbf/src/opt/search.rs:17-106):
// candidate generation, the selection of the left-bottom-most free candidate, its registration and
// the periodic removal of a random placed item, all on the device so that one CUDA graph replays
// a whole step.
#pragma once
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdint>

#include "geom.cuh"
#include "qtree.hpp"

#ifndef JCDE_PDL
#define JCDE_PDL 1   // chained kernels of the small-batch passes and the LBF step: programmatic launch
#endif

namespace jcde {

// Launches `kern` on `s`, with the programmatic stream-serialization attribute when `pdl` (and
// JCDE_PDL): the grid may then be scheduled before the grid ahead of it has completed, so `kern`
// must call pdl_wait() before its first global access.  In the LBF build's graph (three chained
// kernels per step) this takes 150.7 -> 146.8 ms per 2000-step build.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_chained(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, bool pdl,
                                  Args... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = (JCDE_PDL && pdl) ? 1u : 0u;
    return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

enum : uint32_t {
    RES_OK = 0,
    RES_ERR_NODES = 1,
    RES_ERR_ENTRIES = 2,
    RES_ERR_EDGES = 3,
    RES_ERR_HVERTS = 4,
    RES_ERR_KEYS = 5,
    RES_ERR_TASKS = 6,
};

// Allocation state of the pools (device memory; loaded by the update kernels, written back at the end).
struct RCtl {
    uint32_t n_nodes;     // high-water mark of the node pool
    uint32_t n_qfree;     // depth of the free-quartet stack
    uint32_t entry_top;   // entry pool bump pointer
    uint32_t edge_top;    // edge pool bump pointer
    uint32_t hvert_top;   // hazard vertex pool bump pointer
    uint32_t n_slots;     // hazard key high-water mark
    uint32_t n_kfree;     // depth of the free-key stack
    uint32_t error;       // first capacity failure (RES_ERR_*), sticky
    uint32_t not_found;   // deregistrations of unknown keys, placements of unknown items
    uint32_t last_key;    // key of the last registration (~0 when it failed)
    uint32_t n_live;      // registered hazards
    uint32_t pad[5];
};

struct RTask {
    int32_t node;
    uint32_t kind;
    uint32_t pad[2];
    DEntry e;
};

// The task stack's bottom entries live in the update kernel's shared memory (a warp pops a task right
// after pushing it, so a global-memory stack put a round trip through L2 on every task).
constexpr uint32_t RT_SMEM_TASKS = 512;

struct RTree {
    DNode* nodes;
    uint32_t* ncap;      // entry slab capacity per node
    uint8_t* level;
    uint8_t* strength;   // strongest presence per node (the query kernels' unfiltered strength)
    uint32_t* nedges;    // active edges per node
    DEntry* entries;
    float4* edges;
    DHaz* haz;
    float2* hverts;
    uint8_t* alive;
    int32_t* qfree;
    uint32_t* kfree;
    RTask* tasks;
    RTask* stasks;   // in a kernel: the bottom RT_SMEM_TASKS entries of the stack, in shared memory
    RCtl* ctl;
    uint32_t node_cap, entry_cap, edge_cap, hvert_cap, key_cap, task_cap;
    Box cde;
    uint32_t depth;
};

// LBF-style build state (device memory).
struct LbfDev {
    uint32_t step;        // next step
    uint32_t n_live;      // placed items not removed
    uint32_t n_removed;   // removals so far (index of the next removal draw)
    uint32_t n_placed;
    unsigned long long best;   // choice of the current round: (order-preserving cost bits << 32) | candidate
    uint32_t n_free;           // candidates the surrogate pass left to the polygon pass (all rounds)
    uint32_t rec_cost;         // the step's best so far: order-preserving cost bits, ~0 = none
    double rec_u;              //   its rotation in turns
    uint32_t rec_q[5];         //   its query record
    uint32_t rec_cand;         //   round << 24 | candidate index
    // the step the next first-round generation draws for, in two slots: the generation of a graph
    // launch's k-th step reads slot k % 2 (when drawn ahead) and writes slot (k + 1) % 2, so that a
    // generation never writes the slot its own blocks read
    uint32_t gen_step[2];
};

constexpr int LBF_MAX_LS = 8;        // local-search rounds per step
constexpr int LBF_MAX_UNIFORM = 64;  // uniform rounds per step

struct LbfParams {
    unsigned long long seed;   // candidate stream of step s: (seed, sid_base + s)
    unsigned long long key_types, key_remove;   // stream keys of the type and removal draws
    uint32_t sid_base, n_cand, n_types, remove_every, max_steps, vlog_steps;
    float x0, y0, x1, y1;      // sampling box of the translations
    float x1_below, y1_below;  // the largest float32 below x1 / y1 (draws stay inside the box)
    // uniform phase: uni_rounds rounds of n_uni candidates; round u >= 1 draws from stream
    // (seed, uni_sid_base + 64 s + u) with the box's x1 tightened to the step's best cost / 10
    uint32_t uni_rounds, n_uni;
    unsigned long long uni_sid_base;
    // local search: round r of step s draws ls_cand candidates around the step's best from stream
    // (seed, ls_sid_base + 64 s + r): Normal offsets with deviations ls_sig[r] (translation) and
    // ls_sth[r] (rotation, in turns)
    uint32_t ls_rounds, ls_cand;
    unsigned long long ls_sid_base;
    float ls_sig[LBF_MAX_LS + 1];
    double ls_sth[LBF_MAX_LS + 1];
    // instance mode: the item of step s is seq[s] (else drawn from the type stream); item t rotates
    // to one of orient[orient_of[t].x ..][0 .. orient_of[t].y) (count 0: continuous rotation)
    const uint32_t* seq;
    const float2* orient;
    const uint2* orient_of;
};

struct LbfLogs {
    uint32_t* placements;   // 8 words per placement: step, key, candidate, item, cos, sin, tx, ty (bits)
    uint32_t* removals;     // 2 words per removal: step, key
    uint32_t* free_counts;  // free candidates per step
    uint32_t* live;         // keys of the placed items, in placement order
    uint8_t* vlog;          // verdicts of the first vlog_steps steps (optional)
};

// Host-side launchers (resident.cu).  All launch one warp unless stated.
void res_launch_init(const RTree& t, const float2* verts, const uint4* recs, const float2* pois, uint32_t n,
                     uint32_t n_slots, const uint32_t* kfree, uint32_t n_kfree, cudaStream_t s);
void res_launch_insert_placed(const RTree& t, const DItem* items, const float2* iverts, uint32_t n_items,
                              const uint32_t* q, uint32_t* out_key, cudaStream_t s);
void res_launch_remove(const RTree& t, const uint32_t* key, cudaStream_t s);
// n candidates of one item per segment k < m, from the stream with key keys[k] over box bx[k] (the
// LBF build's uniform round), written at q + k n (5 words each) and qu + k n
constexpr uint32_t RES_GEN_SEGMENTS = 64;
void res_launch_gen_candidates(const unsigned long long* keys, const float (*bx)[4], uint32_t m, uint32_t n,
                               uint32_t item, const float2* orient, uint32_t n_orient, uint32_t* q, double* qu,
                               int n_sms, cudaStream_t s);
void res_launch_lbf_gen(const LbfParams& p, LbfDev* st, uint32_t* q, double* qu, uint32_t round, int n_sms,
                        cudaStream_t s, bool ahead = false, uint32_t slot = 0);
// The next step's first round can be generated while a step commits (into the other candidate
// buffer): gen with `ahead` draws for st->gen_step[slot] and leaves the step's state alone, and the
// commit, with `ahead`, clears that state for the next step when it ends.  A first-round generation
// writes st->gen_step[slot ^ 1] (its step + 1).
void res_launch_lbf_merge(LbfDev* st, const uint32_t* q, const double* qu, uint32_t round, cudaStream_t s);
void res_launch_lbf_commit(const RTree& t, const DItem* items, const float2* iverts, uint32_t n_items,
                           const LbfParams& p, LbfDev* st, const uint32_t* q, const double* qu, uint32_t round,
                           const uint8_t* verdicts, const LbfLogs& logs, cudaStream_t s, bool ahead = false);

}  // namespace jcde
