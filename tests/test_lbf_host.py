"""The LBF-style build's host definition (oracle side of the on-device build's parity test)."""
import numpy as np

from jcde import lbf
from jcde import workload as W


def test_select_vectorised_equals_scalar(oracle_mod):
    spec = lbf.LbfSpec(n_types=12, n_cand=1024)
    lay, _ = lbf.setup(oracle_mod.OracleBackend, spec)
    rng = np.random.default_rng(3)
    for step in range(6):
        q = lbf.step_queries(spec, step)
        q["item"] = rng.integers(0, spec.n_types, len(q))
        v = (rng.random(len(q)) < (0.02 if step == 0 else 0.4)).astype(np.uint8)
        assert lbf.select_host(lay.items, q, v) == lbf._select_host_scalar(lay.items, q, v)
    q = lbf.step_queries(spec, 0)
    assert lbf.select_host(lay.items, q, np.ones(len(q), np.uint8)) == -1


def test_select_ties_keep_first(oracle_mod):
    spec = lbf.LbfSpec(n_types=4, n_cand=64)
    lay, _ = lbf.setup(oracle_mod.OracleBackend, spec)
    q = lbf.step_queries(spec, 0)
    q[10] = q[3]
    q[20] = q[3]
    v = np.ones(len(q), np.uint8)
    v[[3, 10, 20]] = 0
    assert lbf.select_host(lay.items, q, v) == 3


def test_host_build_small(oracle_mod):
    """A short build: every placement is the least-cost free candidate and the log is reproducible."""
    spec = lbf.LbfSpec(n_types=12, n_cand=512, steps=60, remove_every=20, uniform_rounds=1)
    lay, eng = lbf.setup(oracle_mod.OracleBackend, spec)
    seen = []
    log = lbf.run_host(lay, eng, spec, on_step=lambda s, e: seen.append(s))
    assert seen == list(range(60))
    assert len(log.placements) == 60 and len(log.removals) == 3
    assert len(log.free_counts) == 60 and (log.free_counts > 0).all()
    # the first placement: recompute from the step's candidates on a fresh engine
    lay2, eng2 = lbf.setup(oracle_mod.OracleBackend, spec)
    q = lbf.step_queries(spec, 0)
    v = eng2.detect_batch(q)
    best = lbf.select_host(lay2.items, q, v)
    assert int(log.placements[0, 2]) == best and int(log.placements[0, 3]) == int(q["item"][0])
    lay3, eng3 = lbf.setup(oracle_mod.OracleBackend, spec)
    assert lbf.run_host(lay3, eng3, spec).same_as(log)


def test_step_streams():
    """Candidate draws: rotation n+i, x 2n+i, y 3n+i of stream (seed, 10000 + step); type: draw step of (seed, 2)."""
    spec = lbf.LbfSpec(n_cand=256)
    q = lbf.step_queries(spec, 7)
    st = W.Stream(spec.seed, lbf.CAND_SID_BASE + 7)
    u = st.u64(4 * spec.n_cand)
    x = (u[2 * spec.n_cand :][: spec.n_cand] >> np.uint64(40)).astype(np.float32) * np.float32(2.0**-24)
    assert np.array_equal(q["tx"], np.minimum(np.float32(0) + x * np.float32(spec.width),
                                              np.nextafter(np.float32(spec.width), np.float32(0))))
    t = W.Stream(spec.seed, lbf.TYPE_SID).u64(8)[7] % np.uint64(spec.n_types)
    assert (q["item"] == t).all()


def test_uniform_rounds_tighten_the_sampling_box(oracle_mod):
    """search.rs:62-63 batched per round: after a round with a free candidate, the next rounds draw
    x only up to the best cost / 10 (LBFLoss::tighten_sample_bbox, loss.rs:34-44); the step places
    the least-cost free candidate over all rounds (strictly better replaces, first kept on ties)."""
    spec = lbf.LbfSpec(n_types=12, n_cand=2048, steps=1, remove_every=0, uniform_rounds=4)
    lay, eng = lbf.setup(oracle_mod.OracleBackend, spec)
    t = int(W.Stream(spec.seed, lbf.TYPE_SID).u64(1)[0] % np.uint64(spec.n_types))
    best, x1, tightened = None, spec.box[2], 0
    for u in range(spec.uniform_rounds):
        q, _ = lbf._uniform_round(spec, 0, u, t, x1)
        assert len(q) == 512 and (q["tx"] < x1).all()
        b, c = lbf.select_host_cost(lay.items, q, eng.detect_batch(q))
        if b >= 0 and (best is None or c < best[0]):
            best = (c, (u << 24) | b)
        if best is not None:
            nx = min(spec.box[2], np.float32(best[0] / np.float32(10.0)))
            tightened += int(nx < x1)
            x1 = nx
    assert best is not None and tightened >= 1
    lay2, eng2 = lbf.setup(oracle_mod.OracleBackend, spec)
    log = lbf.run_host(lay2, eng2, spec)
    assert int(log.placements[0, 2]) == best[1]


def test_host_build_with_local_search(oracle_mod):
    """Local search never places worse than the same build's uniform rounds alone."""
    base = dict(n_types=12, n_cand=512, steps=30, remove_every=0)
    spec0 = lbf.LbfSpec(**base)
    spec1 = lbf.LbfSpec(**base, ls_rounds=2, ls_cand=256)
    lay0, eng0 = lbf.setup(oracle_mod.OracleBackend, spec0)
    lay1, eng1 = lbf.setup(oracle_mod.OracleBackend, spec1)
    costs = []
    for lay, eng, spec in ((lay0, eng0, spec0), (lay1, eng1, spec1)):
        p = lbf.run_host(lay, eng, spec, steps=1).placements[0]
        xy = W.transform_points(lay.items[int(p[3])].xy, *[np.uint32(v).view(np.float32) for v in p[4:8]])
        costs.append(lbf.lbf_cost(xy))
    assert costs[1] <= costs[0]
    assert len(lbf.run_host(lay0, eng0, spec0, steps=5).placements) == 5
    # LSSampler's deviations: 1% -> 0.05% of the CDE box's largest side, 2 -> 0.5 degrees (ls_sampler.rs:9-13)
    sig = lbf.LbfSpec(ls_rounds=4, ls_cand=64).ls_sigmas()
    assert np.isclose(sig[0][0], 200.0) and np.isclose(sig[0][1] * 360.0, 2.0)
    assert all(a[0] > b[0] and a[1] > b[1] for a, b in zip(sig, sig[1:]))


def test_deterministic_normal_sampler():
    """The Box-Muller generator shared by the host definition and the device: its logarithm against
    numpy's (a few ULPs), and the moments of its normals."""
    x = np.concatenate([W.Stream(9, 1).f64(100000) + 2.0**-53, [1.0, 0.5, 2.0**-53, 0.7071067811865476]])
    ref = np.log(x)
    assert np.max(np.abs(W.ln_f64(x) - ref) / np.maximum(np.abs(ref), 1e-300)) < 1e-15 and W.ln_f64(np.ones(1))[0] == 0.0
    d = W.Stream(9, 2).f64(400000)
    z0, z1 = W.normal_pair(1.0 - d[:200000], d[200000:])
    for z in (z0, z1):
        assert abs(z.mean()) < 0.01 and abs(z.std() - 1.0) < 0.01
    assert abs(np.corrcoef(z0, z1)[0, 1]) < 0.01


def test_detect_with_surrogate_counts(oracle_mod):
    """The oracle's one-pass verdicts-with-surrogate-count equal the separate full and surrogate passes."""
    spec = lbf.LbfSpec(n_types=12, n_cand=2048)
    lay, eng = lbf.setup(oracle_mod.OracleBackend, spec)
    q = lbf.step_queries(spec, 3)
    q["item"][::97] = 999   # invalid items: verdict 2, never counted
    v, n_und = eng.detect_with_surrogate(q)
    assert np.array_equal(v, eng.detect_batch(q))
    sv = eng.detect_batch(q, mode=1)
    assert n_und == int((sv == 0).sum())
