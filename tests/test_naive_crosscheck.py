"""The oracle (and the GPU) against a tree-free checker written apart from both (oracle/naive.cpp).

The oracle and the product were written from the same reading of the reference's quadtree
(qt_node.rs, qt_hazard.rs, qt_traits.rs), so a shared misreading would pass every oracle-vs-GPU
test.  The naive checker uses no quadtree at all: every query against every edge of every relevant
hazard, the containment rule of cd_engine.rs:231-255 and the surrogate's poles against every
hazard.  Verdicts and collected sets must agree.

The one kind of disagreement seen is a near-touch that only rounding creates: edge_intersection
(edge.rs:180-228) rounds t or u into [0, 1] for two edges that miss each other by about one ULP,
while the closed box of the hazard edge (rect.rs:301-345), through which the engine reaches every
hazard edge (QTHazPartial::collides_with, qt_partial_hazard.rs:67-71), rejects the item edge.  The
checker names such a pair (flag 8 of ``NaiveChecker.explain``).  Every disagreement must be that,
must be a hazard the naive checker reports and the engine does not, and must be rare.
"""
import numpy as np
import pytest

from jcde import workload as W
from oracle import naive as N

f32 = np.float32
ROUNDING_ONLY = 8


def nxt(x, k=1, to=np.inf):
    x = f32(x)
    for _ in range(k):
        x = np.nextafter(x, f32(to))
    return x


DENORM = float(np.frombuffer(np.uint32(1).tobytes(), np.float32)[0])   # 1.4e-45, the least denormal
FPA_CASES = [
    (0.0, -0.0, True),                       # +0 == -0 exactly
    (-0.0, -0.0, True),
    (DENORM, -DENORM, True),                 # across zero, within f32::EPSILON
    (1e-38, -1e-38, True),                   # normal tiny values across zero
    (6e-8, -5.9e-8, True),                   # |a-b| = 1.19e-7 <= f32::EPSILON
    (6e-8, -6e-8, False),                    # |a-b| = 1.2e-7 > f32::EPSILON, ULP distance wraps to huge
    (1.0, -1.0, False),                      # bit patterns differ by exactly 2^31: i32::MIN saturates to i32::MAX
    (float(nxt(0.0, 4)), 0.0, True),          # denormals 4 ULPs apart (also within epsilon)
    (2.0, float(nxt(2.0, 4)), True),         # 4 ULPs above 2 (epsilon alone would say no)
    (2.0, float(nxt(2.0, 5)), False),
    (-2.0, float(nxt(-2.0, 4, -np.inf)), True),  # 4 ULPs on the negative side
    (-2.0, float(nxt(-2.0, 5, -np.inf)), False),
    (float(nxt(1.0, 1, 0.0)), float(nxt(1.0, 3)), True),   # across an exponent boundary, 4 ULPs
    (float(nxt(1.0, 2, 0.0)), float(nxt(1.0, 3)), False),
    (3.4028234663852886e38, float(nxt(3.4028234663852886e38, 4, 0.0)), True),   # f32::MAX
]


@pytest.mark.parametrize("a,b,eq", FPA_CASES)
def test_fpa_eq_across_zero_and_boundaries(oracle_mod, a, b, eq):
    """float-cmp's approx_eq!(f32) default margin (util/fpa.rs:18-23): oracle and naive checker."""
    for fn in (oracle_mod.fpa_eq, N.fpa_eq):
        assert fn(a, b) == eq and fn(b, a) == eq, (fn, a, b)


def compare(nc, q, ref_counts, ref_ids, ignored=None, max_rate=2e-4):
    """Naive collected sets vs the engine's: returns the explained corners [(query, key)]."""
    nc_counts, nc_ids = nc.collect_batch(q, ignored=ignored)
    ref = np.split(np.asarray(ref_ids), np.cumsum(ref_counts)[:-1])
    got = np.split(np.asarray(nc_ids), np.cumsum(nc_counts)[:-1])
    corners = []
    for i in np.flatnonzero((np.asarray(ref_counts) != nc_counts) | np.array(
            [not np.array_equal(a, b) for a, b in zip(ref, got)])):
        only_engine = set(ref[i].tolist()) - set(got[i].tolist())
        only_naive = set(got[i].tolist()) - set(ref[i].tolist())
        assert not only_engine, (i, q[i], sorted(only_engine))
        for k in sorted(only_naive):
            assert nc.explain(q[i], k) == ROUNDING_ONLY, (i, q[i], k, nc.explain(q[i], k))
            corners.append((int(i), int(k)))
    assert len(corners) <= max(1, max_rate * len(q)), corners
    return corners


def compare_verdicts(nc, q, ref_verdicts, ignored=None):
    """Naive verdicts vs the engine's; a disagreement must be a query the naive checker calls a
    collision only through rounding-only edge pairs."""
    got = nc.detect_batch(q, ignored=ignored)
    bad = np.flatnonzero(got != ref_verdicts)
    for i in bad:
        assert ref_verdicts[i] == 0 and got[i] == 1, (i, q[i])
        c, ids = nc.collect_batch(q[i : i + 1], ignored=ignored)
        assert all(nc.explain(q[i], k) == ROUNDING_ONLY for k in ids), (i, q[i], ids)
    assert len(bad) <= max(1, 2e-4 * len(q))
    return bad.tolist()


@pytest.fixture(scope="module")
def strip_nc(strip_layout):
    return N.NaiveChecker.from_layout(strip_layout[0])


@pytest.fixture(scope="module")
def star_nc(star_layout):
    return N.NaiveChecker.from_layout(star_layout[0])


def test_strip_uniform_queries(strip_layout, strip_nc):
    """The strip workload (65,536 uniform queries, NoFilter): verdicts and collected sets agree exactly."""
    lay, oeng = strip_layout
    q = W.queries_for(lay, 65536, 0xC0)
    assert compare_verdicts(strip_nc, q, oeng.detect_batch(q)) == []
    sub = q[:16384]
    assert compare(strip_nc, sub, *oeng.collect_batch(sub)) == []


def test_star_uniform_sample(star_layout, star_nc):
    """The star benchmark layout with its zone filter: a 16,384-query sample agrees exactly."""
    lay, oeng = star_layout
    q = W.queries_for(lay, 16384, 0xC1, sid=21)
    assert compare_verdicts(star_nc, q, oeng.detect_batch(q, ignored=lay.filter_keys), lay.filter_keys) == []
    assert compare(star_nc, q, *oeng.collect_batch(q, ignored=lay.filter_keys), ignored=lay.filter_keys) == []


@pytest.mark.parametrize("which", ["strip", "star"])
def test_boundary_queries(which, strip_layout, star_layout, strip_nc, star_nc):
    """Queries on the quadtree's split lines at right angles, some nudged by one ULP."""
    lay, oeng = strip_layout if which == "strip" else star_layout
    nc = strip_nc if which == "strip" else star_nc
    ign = lay.filter_keys or None
    q = W.boundary_queries(lay, 16384, 0xB1)
    compare_verdicts(nc, q, oeng.detect_batch(q, ignored=ign), ign)
    compare(nc, q, *oeng.collect_batch(q, ignored=ign), ignored=ign)


def test_touch_queries(strip_layout, star_layout, strip_nc, star_nc):
    """Item vertices put on hazard vertices and edges (exact touches and one-ULP misses): the
    rounding-only corners appear here and nowhere else, and each is explained."""
    lay, oeng = strip_layout
    q = W.touch_queries(lay, 1 << 16, 0x70)
    assert compare_verdicts(strip_nc, q, oeng.detect_batch(q)) == []
    compare(strip_nc, q[:16384], *oeng.collect_batch(q[:16384]))
    lay, oeng = star_layout
    q = W.touch_queries(lay, 1 << 19, 0x70)
    bad = compare_verdicts(star_nc, q, oeng.detect_batch(q, ignored=lay.filter_keys), lay.filter_keys)
    sub = q[:49152]
    corners = compare(star_nc, sub, *oeng.collect_batch(sub, ignored=lay.filter_keys), ignored=lay.filter_keys)
    # the corners this seeded set holds (listed so that a change in either checker shows up here)
    assert corners == [(44384, 4)], corners
    assert len(bad) <= 4, bad


@pytest.fixture(scope="module")
def bin_layouts(oracle_mod):
    """Three bins of the batched multi-layout workload: star containers of 32-128 vertices holding
    log-uniform 20-160 items drawn from 40 star types of 8-200 vertices."""
    return W.multi_layouts(oracle_mod.OracleBackend, seed=0x7C2, n_layouts=3, items_range=(20, 160))


def test_bin_layouts(bin_layouts):
    """Random star containers and items of up to 200 vertices: queries inside the container, on the
    quadtree's split lines and touching hazards agree, verdicts and collected sets."""
    for l, (lay, oeng) in enumerate(bin_layouts):
        nc = N.NaiveChecker.from_layout(lay)
        xy = lay.hazards[0].xy
        cx, cy = (xy[:, 0].min() + xy[:, 0].max()) / 2, (xy[:, 1].min() + xy[:, 1].max()) / 2
        h = 0.6 * (xy[:, 0].max() - xy[:, 0].min()) / 2
        box = np.array([cx - h, cy - h, cx + h, cy + h], np.float32)
        q = W.make_queries(W.Stream(0x7C4 + l, 1), 8192, len(lay.items), box)
        assert compare_verdicts(nc, q, oeng.detect_batch(q)) == []
        assert compare(nc, q[:4096], *oeng.collect_batch(q[:4096])) == []
        qb = W.boundary_queries(lay, 8192, 0xB2 + l)
        compare_verdicts(nc, qb, oeng.detect_batch(qb))
        compare(nc, qb[:4096], *oeng.collect_batch(qb[:4096]))
        qt = W.touch_queries(lay, 16384, 0x71 + l)
        compare_verdicts(nc, qt, oeng.detect_batch(qt))
        compare(nc, qt[:4096], *oeng.collect_batch(qt[:4096]))


def test_lbf_end_state_after_registrations_and_removals(oracle_mod):
    """The oracle's quadtree after 300 LBF steps (300 registrations, a deregistration every 50 steps,
    freed keys reused by later placements) against the tree-free checker built from the hazards
    still live: what register_hazard / deregister_hazard_by_key (cd_engine.rs:59-96) leave behind
    answers like the live set alone."""
    from jcde import lbf

    spec = lbf.LbfSpec(steps=300, n_cand=2048)
    lay, eng = lbf.setup(oracle_mod.OracleBackend, spec)
    log = lbf.run_host(lay, eng, spec)
    keys = log.placements[:, 1].astype(np.int64)
    assert len(log.removals) == 6 and len(set(keys.tolist())) < len(keys)   # keys were reused
    placed = {int(r[0]): r for r in log.placements}
    removed = {int(s): int(k) for s, k in log.removals}
    live = {}
    for step in range(spec.steps):   # a step places, then removes
        if step in placed:
            r = placed[step]
            t = int(r[3])
            c, s, tx, ty = np.asarray(r[4:8], np.uint32).view(np.float32)
            hz = W.placed_hazard(lay.items[t], t, c, s, tx, ty)
            hz.key = int(r[1])
            assert hz.key not in live
            live[hz.key] = hz
        if step in removed:
            del live[removed[step]]
    assert len(live) == len(keys) - len(log.removals)
    end = W.Layout(lay.name, lay.depth, lay.cd_threshold, lay.cde_bbox, items=lay.items,
                   hazards=[lay.hazards[0]] + list(live.values()))
    nc = N.NaiveChecker.from_layout(end)
    q = W.make_queries(W.Stream(0x1BF, 5), 16384, len(lay.items), np.array([0, 0, 4000, 2000], np.float32))
    v = eng.detect_batch(q)
    assert 0.1 < v.mean() < 0.9
    assert compare_verdicts(nc, q, v) == []
    assert compare(nc, q[:8192], *eng.collect_batch(q[:8192])) == []
    qt = W.touch_queries(end, 32768, 0x72)
    compare_verdicts(nc, qt, eng.detect_batch(qt))
    compare(nc, qt[:8192], *eng.collect_batch(qt[:8192]))
    qb = W.boundary_queries(end, 16384, 0xB3)
    compare_verdicts(nc, qb, eng.detect_batch(qb))
    compare(nc, qb[:8192], *eng.collect_batch(qb[:8192]))


# ----------------------------------------------------------------------------------------------
# GPU: the sm_103a kernels against the oracle (bit-exact) and the naive checker (as above)
# ----------------------------------------------------------------------------------------------
@pytest.fixture(scope="module")
def gpu_engines(strip_layout, star_layout, jcde_mod):
    from helpers import gpu_engine

    return gpu_engine(strip_layout[0]), gpu_engine(star_layout[0])


def _three_way(geng, oeng, nc, q, ign, collect_n):
    from helpers import csr_lists, gpu_collect, gpu_detect

    ref = oeng.detect_batch(q, ignored=ign)
    got = gpu_detect(geng, q, filter=ign)
    assert np.array_equal(got, ref), np.flatnonzero(got != ref)[:20]
    bad = compare_verdicts(nc, q, ref, ign)
    sub = q[:collect_n]
    rc, rids = oeng.collect_batch(sub, ignored=ign)
    assert gpu_collect(geng, sub, filter=ign) == csr_lists(rc, rids)
    corners = compare(nc, sub, rc, rids, ignored=ign)
    return bad, corners


@pytest.mark.gpu
def test_gpu_three_way_strip(strip_layout, strip_nc, gpu_engines):
    """The strip workload: all 65,536 queries, the oracle, the GPU and the naive checker agree."""
    lay, oeng = strip_layout
    bad, corners = _three_way(gpu_engines[0], oeng, strip_nc, W.queries_for(lay, 65536, 0xC0), None, 65536)
    assert bad == [] and corners == []


@pytest.mark.gpu
def test_gpu_three_way_star_sample(star_layout, star_nc, gpu_engines):
    """The star benchmark: a 65,536-query sample of its batch, with the zone filter."""
    lay, oeng = star_layout
    q = W.queries_for(lay, 1 << 20, 0xC1)[:65536]
    bad, corners = _three_way(gpu_engines[1], oeng, star_nc, q, lay.filter_keys, 65536)
    assert bad == [] and corners == []


@pytest.mark.gpu
def test_gpu_three_way_boundary_and_touch(strip_layout, star_layout, strip_nc, star_nc, gpu_engines):
    """Boundary queries (65,536 per layout) and touch queries (2^19 on the star layout)."""
    for (lay, oeng), nc, geng in ((strip_layout, strip_nc, gpu_engines[0]), (star_layout, star_nc, gpu_engines[1])):
        ign = lay.filter_keys or None
        _three_way(geng, oeng, nc, W.boundary_queries(lay, 1 << 16, 0xB0), ign, 16384)
    lay, oeng = star_layout
    bad, corners = _three_way(gpu_engines[1], oeng, star_nc, W.touch_queries(lay, 1 << 19, 0x70), lay.filter_keys,
                              49152)
    assert corners == [(44384, 4)] and len(bad) <= 4
