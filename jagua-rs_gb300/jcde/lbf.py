"""LBF-style incremental build over the engine (the caller of the CDE in lbf/src/opt/search.rs).

Each step draws an item type and a batch of candidate placements, asks the engine for their
verdicts, commits the candidate with the lowest LBF cost among the free ones
(LBFLoss::cost = x_max * 10 + y_max of the placed shape's bounding box, lbf/src/opt/loss.rs:29-31;
ties keep the first, search.rs:52) by registering it as a hazard, and every `remove_every` steps
deregisters a random placed item (as Layout::remove_item does, entities/layout.rs:88-100).

Each step restates lbf's search (search.rs:17-106) in rounds, so that every engine sees the same
candidates and a whole round is one batch:
* the uniform phase is `uniform_rounds` rounds of n_cand / uniform_rounds candidates drawn from a
  seeded stream over the sampling box; after each round the box's x_max is tightened to the best
  cost so far / 10 (LBFLoss::tighten_sample_bbox, loss.rs:34-44, applied by search.rs:62-63 after
  every improvement; here after every round);
* the optional local-search phase (search.rs:80-101) is `ls_rounds` rounds of `ls_cand`
  candidates around the step's best so far, with Normal offsets whose standard deviations decay
  exponentially from 1% to 0.05% of the CDE box's largest side (translation) and from 2 to 0.5
  degrees (rotation), as LSSampler does (ls_sampler.rs:9-13, :84-90) per round instead of per
  sample; the normals come from a project-owned Box-Muller generator (workload.normal_pair) fed by
  the seeded streams, identical on the host and the device (lbf's own generator, rand_distr's
  Normal, is not reproducible outside Rust);
* a round's least-cost free candidate replaces the step's best when it costs strictly less.

Two drivers share the definition: `run_host` (one engine call per step from Python: the oracle,
or the GPU engine with host-side registration) and `run_device` (jcde_lbf_*: generation, verdicts,
choice, registration and removal all on the GPU, no host round trip per step).  Both return the
same log: placements (step, key, candidate, item, cos, sin, tx, ty as float32 bits), removals
(step, key) and, per step, the number of candidates the surrogate pass left to the polygon pass.
As in lbf's search (search.rs:52-56, "worth testing"), a candidate only needs its polygon test if
it could still beat the best free candidate: the device skips the others (unless it logs every
verdict), which changes no choice.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import workload as W

SEED = 0xC3
TYPE_SID, REMOVE_SID, CAND_SID_BASE = 2, 4, 10_000   # stream ids of the build's draws
LS_SID_BASE = 1_000_000    # local-search round r of step s: stream LS_SID_BASE + 64 s + r
UNI_SID_BASE = 2_000_000   # uniform round u >= 1 of step s: stream UNI_SID_BASE + 64 s + u (round 0: CAND_SID_BASE + s)
# LSSampler's default deviations (ls_sampler.rs:9-13): translation as fractions of the CDE box's
# largest side, rotation in radians, each (start, end)
SD_TRANSL = (0.01, 0.0005)
SD_ROT = (2.0 * math.pi / 180.0, 0.5 * math.pi / 180.0)


@dataclass
class LbfSpec:
    """The strip build: 60 star types of 8-120 vertices, a 20000 x 2000 strip, 16384 candidates per step."""

    seed: int = SEED
    n_types: int = 60
    v_range: tuple = (8, 120)
    r_range: tuple = (20.0, 60.0)
    width: float = 20000.0
    height: float = 2000.0
    steps: int = 2000
    n_cand: int = 16384
    remove_every: int = 50
    depth: int = W.DEFAULT_DEPTH
    cd_threshold: int = W.DEFAULT_CD_THRESHOLD
    # uniform phase in rounds (the sampling box tightened after each; 1: the benchmark's build, every
    # candidate of a step drawn over the whole strip); local search after it (0: off)
    uniform_rounds: int = 1
    ls_rounds: int = 0
    ls_cand: int = 0
    ls_max_dim: float = 0.0   # largest side of the CDE box the deviations scale with (0: the strip's)
    # instance mode: the item of each step (else drawn from the type stream) and, per item, a float32
    # (cos, sin) table of allowed orientations or None for continuous rotation
    item_seq: np.ndarray | None = None
    orient: list | None = None

    def ls_sigmas(self):
        """Per local round r = 1..ls_rounds: (translation deviation float32, rotation deviation in
        turns float64) at progress (r-1)/ls_rounds of LSSampler::decay_stddev's exponential curve
        (ls_sampler.rs:84-90)."""
        dim = float(self.ls_max_dim) or max(float(self.width), float(self.height))
        out = []
        for r in range(1, self.ls_rounds + 1):
            pct = (r - 1) / self.ls_rounds
            st = SD_TRANSL[0] * dim * (SD_TRANSL[1] / SD_TRANSL[0]) ** pct
            sr = SD_ROT[0] * (SD_ROT[1] / SD_ROT[0]) ** pct
            out.append((np.float32(st), sr / (2.0 * math.pi)))
        return out

    @property
    def n_uniform(self) -> int:
        """Candidates per uniform round."""
        assert self.n_cand % self.uniform_rounds == 0, "n_cand must be a multiple of uniform_rounds"
        return self.n_cand // self.uniform_rounds

    @property
    def box(self) -> np.ndarray:
        return np.array([0.0, 0.0, self.width, self.height], np.float32)


@dataclass
class LbfLog:
    placements: np.ndarray   # (n, 8) uint32
    removals: np.ndarray     # (m, 2) uint32
    free_counts: np.ndarray  # (steps,) uint32: candidates the surrogate pass left to the polygon pass
    verdicts: list = field(default_factory=list)   # per-step verdict arrays (host driver, if kept)

    def same_as(self, other: "LbfLog") -> bool:
        return (np.array_equal(self.placements, other.placements) and np.array_equal(self.removals, other.removals)
                and np.array_equal(self.free_counts, other.free_counts))


def lbf_cost(xy: np.ndarray) -> np.float32:
    """LBFLoss::cost of a placed shape (loss.rs:29-31) in float32."""
    return np.float32(np.float32(xy[:, 0].max()) * np.float32(10.0) + np.float32(xy[:, 1].max()))


def select_host(items, q: np.ndarray, verdicts: np.ndarray) -> int:
    """The LBF choice on the host: index of the free candidate of least cost, first on ties, or -1.

    The transformation is TRANSFORM_FORMULA in float32 (workload.transform_points), vectorised over
    the candidates; min/max and the argmin's first-occurrence rule are exact."""
    return select_host_cost(items, q, verdicts)[0]


def select_host_cost(items, q: np.ndarray, verdicts: np.ndarray):
    """(index, float32 cost) of the LBF choice, or (-1, None)."""
    free = np.flatnonzero(verdicts == 0)
    if len(free) == 0:
        return -1, None
    costs = np.empty(len(free), dtype=np.float32)
    item_ids = q["item"][free]
    for t in np.unique(item_ids):
        sel = np.flatnonzero(item_ids == t)
        rows = q[free[sel]]
        xy = np.asarray(items[int(t)].xy, dtype=np.float32)
        c, s = rows["cos"][:, None], rows["sin"][:, None]
        one = np.float32(1.0)
        ox = (c * xy[None, :, 0] + (-s) * xy[None, :, 1]) + rows["tx"][:, None] * one
        oy = (s * xy[None, :, 0] + c * xy[None, :, 1]) + rows["ty"][:, None] * one
        costs[sel] = ox.max(axis=1) * np.float32(10.0) + oy.max(axis=1)
    k = int(np.argmin(costs))
    return int(free[k]), costs[k]


NO_KEY = (1 << 64) - 1   # the key of a round with no free candidate


def cost_key(cost, index: int) -> int:
    """The 64-bit choice key of a free candidate: the order-preserving bits of its float32 cost
    above its index, so that the least key is the least cost, first on ties (the order the
    device's 64-bit atomicMin choice uses).  -0 is keyed as +0: the two compare equal."""
    u = int(np.asarray(np.float32(cost) + np.float32(0.0), dtype=np.float32).view(np.uint32))
    u = (~u & 0xFFFFFFFF) if u & 0x80000000 else (u | 0x80000000)
    return (u << 32) | int(index)


def _judge(lay, eng, q: np.ndarray, ranks):
    """One round's (choice index or -1, its float32 cost, candidates the surrogate pass left to the
    polygon pass, verdicts).  With ranks = (rank, world size) a rank judges its contiguous slice of
    the candidates; the choice is the least cost_key over the ranks and the count their sum, and
    every rank recomputes the winner's cost from its record (verdicts are then None)."""
    if ranks is None:
        verdicts, n_free = eng.detect_with_surrogate(q)
        b, cb = select_host_cost(lay.items, q, verdicts)
        return b, cb, n_free, verdicts
    from . import shards

    r, w = ranks
    lo, hi = len(q) * r // w, len(q) * (r + 1) // w
    v, n_free = eng.detect_with_surrogate(q[lo:hi]) if hi > lo else (np.zeros(0, np.uint8), 0)
    b, cb = select_host_cost(lay.items, q[lo:hi], v)
    key = shards.min_u64_over_ranks(NO_KEY if b < 0 else cost_key(cb, lo + b))
    n_free = shards.sum_over_ranks(n_free)
    if key == NO_KEY:
        return -1, None, n_free, None
    b = key & 0xFFFFFFFF
    return b, select_host_cost(lay.items, q[b : b + 1], np.zeros(1, np.uint8))[1], n_free, None


def _select_host_scalar(items, q: np.ndarray, verdicts: np.ndarray) -> int:
    best, best_cost = -1, None
    for i in np.flatnonzero(verdicts == 0):
        it = items[int(q["item"][i])]
        cost = lbf_cost(W.transform_points(it.xy, q["cos"][i], q["sin"][i], q["tx"][i], q["ty"][i]))
        if best_cost is None or cost < best_cost:
            best, best_cost = int(i), cost
    return best


def raw_shapes(spec: LbfSpec) -> list:
    """The item types' star shapes as drawn (before import): stream (seed, 1)."""
    st = W.Stream(spec.seed, 1)
    out = []
    for _ in range(spec.n_types):
        nv = int(st.randint(spec.v_range[0], spec.v_range[1], 1)[0])
        out.append(W.star_polygon(st, nv, *spec.r_range))
    return out


def setup(backend, spec: LbfSpec, item_pool=None):
    """Items, the strip container (an Exterior hazard) and a fresh engine: (layout, engine)."""
    items = item_pool
    if items is None:
        items = [W.import_item(backend, xy) for xy in raw_shapes(spec)]
    outer = W.import_static(backend, W.rect_polygon(0.0, 0.0, spec.width, spec.height), W.EXTERIOR)
    lay = W.Layout("lbf-strip", spec.depth, spec.cd_threshold, W.inflate_to_square(W.bbox_of(outer.xy)), items=items)
    lay.hazards.append(outer)
    return lay, W._new_layout_engine(backend, lay)


def step_queries(spec: LbfSpec, step: int) -> np.ndarray:
    t = int(W.Stream(spec.seed, TYPE_SID).u64(step + 1)[step] % np.uint64(spec.n_types))
    q = W.make_queries(W.Stream(spec.seed, CAND_SID_BASE + step), spec.n_cand, 1, spec.box)
    q["item"] = t
    return q


def _orient_of(spec: LbfSpec, t: int):
    return None if spec.orient is None else spec.orient[t]


def _uniform_round(spec: LbfSpec, step: int, u: int, t: int, x1):
    """Uniform round u of a step over the sampling box with x_max = x1: make_queries' candidates
    and their rotations in turns (with allowed orientations: orientation (draw n+i) mod count,
    turns unused)."""
    n = spec.n_uniform
    sid = CAND_SID_BASE + step if u == 0 else UNI_SID_BASE + 64 * step + u
    box = spec.box.copy()
    box[2] = np.float32(x1)
    q = W.make_queries(W.Stream(spec.seed, sid), n, 1, box)
    q["item"] = t
    st = W.Stream(spec.seed, sid)
    st.pos = n   # make_queries draws the items first, then the rotations
    o = _orient_of(spec, t)
    if o is None:
        return q, st.f64(n)
    k = (st.u64(n) % np.uint64(len(o))).astype(np.int64)
    q["cos"] = o[k, 0]
    q["sin"] = o[k, 1]
    return q, np.zeros(n)


def _local_round(spec: LbfSpec, step: int, r: int, t: int, best_u: float, best_q, sg, sth):
    """Local round r >= 1: candidates around the step's best.  Draws i and m+i give the normals of
    x and y (Box-Muller), 2m+i and 3m+i the rotation's; translation offsets are float32(sg * z), the
    rotation moves by sth * z turns."""
    m = spec.ls_cand
    d = W.Stream(spec.seed, LS_SID_BASE + 64 * step + r).f64(4 * m)
    zx, zy = W.normal_pair(1.0 - d[:m], d[m:2 * m])
    zr, _ = W.normal_pair(1.0 - d[2 * m:3 * m], d[3 * m:])
    q = np.zeros(m, dtype=W.QUERY_DTYPE)
    q["item"] = t
    if _orient_of(spec, t) is not None:   # discrete orientations: the best's rotation is kept
        u = np.full(m, best_u)
        q["cos"] = best_q["cos"]
        q["sin"] = best_q["sin"]
    else:
        x = best_u + float(sth) * zr
        u = x - np.floor(x)
        c, s = W.sincos_turns(u)
        q["cos"] = c.astype(np.float32)
        q["sin"] = s.astype(np.float32)
    sg64 = np.float64(np.float32(sg))
    q["tx"] = np.float32(best_q["tx"]) + (sg64 * zx).astype(np.float32)
    q["ty"] = np.float32(best_q["ty"]) + (sg64 * zy).astype(np.float32)
    return q, u


def run_host(lay, eng, spec: LbfSpec, steps: int | None = None, keep_verdicts: int = 0, on_step=None,
             ranks: tuple | None = None) -> LbfLog:
    """The build with one engine call per round (oracle or GPU engine).  With ranks = (rank, world
    size) under an initialised process group, each rank judges a slice of every round's candidates
    against its own replica and the ranks agree on each round's choice (see `_judge`): every rank
    returns the log of the one-process build."""
    assert ranks is None or keep_verdicts == 0, "a rank holds only its slice's verdicts"
    steps = spec.steps if steps is None else steps
    s_rm = W.Stream(spec.seed, REMOVE_SID)
    types = W.Stream(spec.seed, TYPE_SID).u64(steps) % np.uint64(max(spec.n_types, 1))
    sigmas = spec.ls_sigmas()
    placements, removals, free_counts, vkeep = [], [], [], []
    live = []   # keys of placed items, in placement order
    n_uni = spec.uniform_rounds
    for step in range(steps):
        t = int(spec.item_seq[step]) if spec.item_seq is not None else int(types[step])
        rec, n_free = None, 0
        for u in range(n_uni):
            # LBFLoss::tighten_sample_bbox (loss.rs:34-44) by the best so far
            x1 = spec.box[2] if rec is None else min(spec.box[2], np.float32(rec[0] / np.float32(10.0)))
            q, uu = _uniform_round(spec, step, u, t, x1)
            b, cb, nf, verdicts = _judge(lay, eng, q, ranks)
            n_free += nf
            if step < keep_verdicts:
                vkeep.append(np.asarray(verdicts).copy())
            if b >= 0 and (rec is None or cb < rec[0]):   # strictly better replaces (search.rs:52 keeps the first)
                rec = (cb, float(uu[b]), q[b].copy(), (u << 24) | b)
        for r, (sg, sth) in enumerate(sigmas, start=1):
            if rec is None:
                break   # nothing to search around (the device marks the round's candidates invalid)
            ql, ul = _local_round(spec, step, r, t, rec[1], rec[2], sg, sth)
            b, cb, nf, _ = _judge(lay, eng, ql, ranks)
            n_free += nf
            if b >= 0 and cb < rec[0]:
                rec = (cb, float(ul[b]), ql[b].copy(), ((n_uni - 1 + r) << 24) | b)
        free_counts.append(n_free)
        if rec is not None:
            r_q = rec[2]
            hz = W.placed_hazard(lay.items[t], t, r_q["cos"], r_q["sin"], r_q["tx"], r_q["ty"])
            key = eng.register_hazard(hz.kind, hz.dynamic, hz.xy, hz.poi, 1_000_000 + step)
            live.append(key)
            placements.append([step, key, rec[3], t] +
                              [int(np.float32(r_q[f]).view(np.uint32)) for f in ("cos", "sin", "tx", "ty")])
        if spec.remove_every and (step + 1) % spec.remove_every == 0 and live:
            j = int(s_rm.randint(0, len(live) - 1, 1)[0])
            key = live.pop(j)
            eng.deregister_hazard(key)
            removals.append([step, key])
        if on_step is not None:
            on_step(step, eng)
    return LbfLog(np.array(placements, dtype=np.uint32).reshape(-1, 8), np.array(removals, dtype=np.uint32).reshape(-1, 2),
                  np.array(free_counts, dtype=np.uint32), vkeep)


def run_device(eng, spec: LbfSpec, steps: int | None = None, steps_per_graph: int = 0, keep_verdicts: int = 0,
               resident=None):
    """The build on the GPU (jcde_lbf_*) from the engine's current state; returns (log, resident)."""
    from .engine import ResidentEngine

    steps = spec.steps if steps is None else steps
    cde = eng.eng if hasattr(eng, "eng") else eng
    r = resident if resident is not None else ResidentEngine(cde)
    r.lbf_begin(spec.seed, spec.n_cand, spec.n_types, spec.remove_every, steps, spec.box, keep_verdicts,
                spec.ls_rounds, spec.ls_cand, spec.ls_sigmas(), spec.uniform_rounds,
                item_sequence=spec.item_seq, orientations=spec.orient)
    r.lbf_steps(steps, steps_per_graph)
    d = r.lbf_read()
    log = LbfLog(d["placements"], d["removals"], d["free_counts"], list(d["verdicts"]))
    return log, r


def main(argv=None) -> int:
    """Run the device build of the strip for some steps and print its counts (a small case for
    profiling one step's kernels): PYTHONPATH=jagua-rs_gb300 python -m jcde.lbf --steps 1501"""
    import argparse

    import jcde

    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--steps", type=int, default=LbfSpec.steps)
    ap.add_argument("--steps-per-graph", type=int, default=0, help="0: every step launched eagerly")
    a = ap.parse_args(argv)
    spec = LbfSpec()
    _, geng = setup(jcde.GpuBackend, spec)
    log, r = run_device(geng, spec, steps=a.steps, steps_per_graph=a.steps_per_graph)
    print(f"steps {len(log.free_counts)} placed {len(log.placements)} removed {len(log.removals)} "
          f"status {r.status()}")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())


def spec_for_instance(setup, **kw) -> LbfSpec:
    """An LBF build of a strip-packing instance (jcde.instance.setup_spp): every item in the placement
    order, the strip as the sampling box, no removals."""
    lay = setup.layout
    return LbfSpec(n_types=len(lay.items), width=setup.width, height=float(lay.hazards[0].xy[:, 1].max()),
                   steps=len(setup.sequence), remove_every=0, item_seq=setup.sequence, orient=setup.orient, **kw)
