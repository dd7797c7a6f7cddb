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
    spec = lbf.LbfSpec(n_types=12, n_cand=512, steps=60, remove_every=20)
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


def test_host_build_with_local_search(oracle_mod):
    """Local search never places worse than the uniform round's choice of the same step."""
    base = dict(n_types=12, n_cand=512, steps=30, remove_every=0)
    spec0 = lbf.LbfSpec(**base)
    spec1 = lbf.LbfSpec(**base, ls_rounds=2, ls_cand=256, ls_sigma_t=100.0, ls_sigma_turns=0.05)
    lay0, eng0 = lbf.setup(oracle_mod.OracleBackend, spec0)
    lay1, eng1 = lbf.setup(oracle_mod.OracleBackend, spec1)
    q, _ = lbf._uniform_round(spec1, 0, int(lbf.step_queries(spec1, 0)["item"][0]))
    b, cost0 = lbf.select_host_cost(lay1.items, q, eng1.detect_batch(q))
    log1 = lbf.run_host(lay1, eng1, spec1, steps=1)
    p = log1.placements[0]
    xy = W.transform_points(lay1.items[int(p[3])].xy, *[np.uint32(v).view(np.float32) for v in p[4:8]])
    assert lbf.lbf_cost(xy) <= cost0
    assert len(lbf.run_host(lay0, eng0, spec0, steps=5).placements) == 5


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
