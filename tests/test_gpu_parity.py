"""GPU parity: every verdict and every collected hazard set of the sm_103a kernels equals the oracle's.

Bit-exact comparisons only (integer verdicts and key sets).  Layouts come from the seeded
generator driven by the oracle; the same hazards are replayed into the GPU engine.
"""
import numpy as np
import pytest

import jcde
from jcde import workload as W

pytestmark = pytest.mark.gpu


from helpers import csr_lists as oracle_sets, gpu_collect, gpu_detect, gpu_engine, torch_queries  # noqa: E402


@pytest.fixture(scope="module")
def strip(strip_layout, jcde_mod):
    lay, oeng = strip_layout
    return lay, oeng, gpu_engine(lay)


@pytest.fixture(scope="module")
def star(star_layout, jcde_mod):
    lay, oeng = star_layout
    return lay, oeng, gpu_engine(lay)


def test_strip_detect_all_queries(strip):
    """The small workload: 65,536 uniform queries, verdicts bit-exact (NoFilter)."""
    lay, oeng, geng = strip
    q = W.queries_for(lay, 65536, 0xC0)
    ref = oeng.detect_batch(q)
    got = gpu_detect(geng, q)
    assert np.array_equal(ref, got), np.flatnonzero(ref != got)[:20]


@pytest.mark.parametrize("mode,omode", [("surrogate", 1), ("poly", 2)])
def test_strip_detect_halves(strip, mode, omode):
    """detect_surrogate_collision and detect_poly_collision separately (cd_engine.rs:204, :160)."""
    lay, oeng, geng = strip
    q = W.queries_for(lay, 16384, 0xC0, sid=11)
    assert np.array_equal(oeng.detect_batch(q, mode=omode), gpu_detect(geng, q, mode=mode))


def test_strip_detect_with_self_filter(strip):
    """HazKey self-filter, as Layout::is_feasible uses it (layout.rs:128-136): every placed item
    tested at its own placement with its own key ignored."""
    lay, oeng, geng = strip
    placed = [hz for hz in lay.hazards if hz.placement is not None]
    for hz in placed[:10]:
        t, c, s, tx, ty = hz.placement
        q = np.zeros(1, W.QUERY_DTYPE)
        q[0] = (t, c, s, tx, ty)
        assert oeng.detect_batch(q, ignored=[hz.key])[0] == gpu_detect(geng, q, filter=[hz.key])[0] == 0
        assert gpu_detect(geng, q)[0] == 1   # without the filter it collides with itself


def test_star_detect_with_zone_filter(star):
    """The large workload with HazKeyFilter::from_irrelevant_qzones (filter.rs:21-41)."""
    lay, oeng, geng = star
    q = W.queries_for(lay, 1 << 18, 0xC1)
    ref = oeng.detect_batch(q, ignored=lay.filter_keys)
    got = gpu_detect(geng, q, filter=lay.filter_keys)
    assert np.array_equal(ref, got), np.flatnonzero(ref != got)[:20]
    # without the filter the answers differ somewhere (the zone matters)
    ref2 = oeng.detect_batch(q[:65536])
    assert np.array_equal(ref2, gpu_detect(geng, q[:65536]))


def test_star_detect_full_size(star):
    """1,048,576 queries (the benchmarked batch), bit-exact against the oracle."""
    lay, oeng, geng = star
    q = W.queries_for(lay, 1 << 20, 0xC1)
    ref = oeng.detect_batch(q, ignored=lay.filter_keys)
    got = gpu_detect(geng, q, filter=lay.filter_keys)
    assert np.array_equal(ref, got), int((ref != got).sum())


def test_host_path_equals_device_path(star):
    lay, oeng, geng = star
    q = W.queries_for(lay, 300_000, 0xC1, sid=5)
    h = geng.detect_batch(q, filter=lay.filter_keys)
    d = gpu_detect(geng, q, filter=lay.filter_keys)
    assert np.array_equal(h, d)


def test_strip_collect(strip):
    """collect_surrogate_collisions + collect_poly_collisions into one collector (ci_bench.rs:56-68)."""
    lay, oeng, geng = strip
    q = W.queries_for(lay, 16384, 0xC0, sid=21)
    ref = oracle_sets(*oeng.collect_batch(q))
    got = gpu_collect(geng, q)
    bad = [i for i in range(len(q)) if ref[i] != got[i]]
    assert not bad, [(i, ref[i], got[i]) for i in bad[:5]]


def test_star_collect_with_filter(star):
    lay, oeng, geng = star
    q = W.queries_for(lay, 65536, 0xC1, sid=22)
    ref = oracle_sets(*oeng.collect_batch(q, ignored=lay.filter_keys))
    got = gpu_collect(geng, q, filter=lay.filter_keys)
    bad = [i for i in range(len(q)) if ref[i] != got[i]]
    assert not bad, [(i, ref[i], got[i]) for i in bad[:5]]
    # collect is non-empty exactly when detect reports a collision
    v = gpu_detect(geng, q, filter=lay.filter_keys)
    assert np.array_equal(v.astype(bool), np.array([len(s) > 0 for s in got]))


def test_collect_capacity_overflow(strip):
    """A too-small id buffer reports the total needed and writes only whole runs."""
    import torch

    lay, oeng, geng = strip
    q = W.queries_for(lay, 4096, 0xC0, sid=23)
    off, cnt, ids, total = geng.collect_batch(torch_queries(q), ids_cap=16)   # retries with the right size
    assert total == int(cnt.sum().item())
    ref = oracle_sets(*oeng.collect_batch(q))
    assert sum(len(s) for s in ref) == total


def test_single_query_entry_points(strip):
    """The reference-shaped single calls: detect/collect on a transformed shape or a surrogate."""
    lay, oeng, geng = strip
    q = W.queries_for(lay, 200, 0xC0, sid=31)
    for row in q:
        it = lay.items[int(row["item"])]
        t = (row["cos"], row["sin"], row["tx"], row["ty"])
        xy = W.transform_points(it.xy, *t)
        p = W.transform_points(it.poi[None, :2], *t)[0]
        poi = np.array([p[0], p[1], it.poi[2]], np.float32)
        assert geng.detect_poly_collision(xy, poi) == oeng.detect_poly(xy, poi)
        assert geng.detect_surrogate_collision(int(row["item"]), t) == oeng.detect_surrogate(int(row["item"]), t)
        assert geng.collect_poly_collisions(xy, poi) == oeng.collect_poly(xy, poi)
        assert geng.collect_surrogate_collisions(int(row["item"]), t) == oeng.collect_surrogate(int(row["item"]), t)


def test_invalid_item_and_empty_batch(strip):
    import torch

    lay, oeng, geng = strip
    q = W.queries_for(lay, 64, 0xC0)
    q["item"][::7] = 1000
    got = gpu_detect(geng, q)
    assert (got[::7] == 2).all()
    ok = np.ones(len(q), bool)
    ok[::7] = False
    assert np.array_equal(got[ok], oeng.detect_batch(q[ok]))
    empty = geng.detect_batch(torch.zeros(0, dtype=torch.uint8, device="cuda"))
    assert empty.numel() == 0


def test_updates_then_queries(strip_layout, jcde_mod, oracle_mod):
    """Deregister / re-register between query batches: the device mirror follows every update."""
    lay, _ = strip_layout
    oeng = W.replay(oracle_mod.OracleBackend, lay)
    geng = gpu_engine(lay)
    q = W.queries_for(lay, 8192, 0xC0, sid=41)
    rng = np.random.default_rng(3)
    live = [hz for hz in lay.hazards if hz.dynamic]
    for step in range(6):
        hz = live.pop(int(rng.integers(len(live))))
        oeng.deregister_hazard(hz.key)
        geng.deregister_hazard_by_key(hz.key)
        assert np.array_equal(oeng.detect_batch(q), gpu_detect(geng, q))
    snap = geng.save()
    for hz in live[:5]:
        geng.deregister_hazard_by_key(hz.key)
    geng.restore(snap)
    assert np.array_equal(oeng.detect_batch(q), gpu_detect(geng, q))


def test_gpu_generated_layout_equals_oracle_layout(strip_layout, jcde_mod):
    """Rejection placement driven by the GPU engine picks exactly the oracle's placements."""
    lay_o, _ = strip_layout
    lay_g, _ = W.strip_layout(jcde_mod.GpuBackend)
    assert len(lay_g.hazards) == len(lay_o.hazards)
    for a, b in zip(lay_o.hazards, lay_g.hazards):
        assert a.key == b.key and a.xy.tobytes() == b.xy.tobytes() and a.poi.tobytes() == b.poi.tobytes()


def test_autotune_keeps_verdicts(star, oracle_mod):
    """Every launch choice the autotuner times gives the oracle's verdicts; the chosen one is kept."""
    lay, oeng, geng = star
    q = W.queries_for(lay, 1 << 17, 0xA7, sid=9)
    saved = geng.get_tuning()
    try:
        t, ms = geng.autotune(torch_queries(q), filter=lay.filter_keys)
        assert ms > 0 and geng.get_tuning() == t
        assert np.array_equal(gpu_detect(geng, q, filter=lay.filter_keys), oeng.detect_batch(q, ignored=lay.filter_keys))
    finally:
        geng.set_tuning(**saved)


@pytest.mark.parametrize("knob,values", [("edge_tile", (4, 8, 16)), ("staging_depth", (0, 1, 2, 3, 4)),
                                         ("surrogate_lanes", (8, 16, 32))])
def test_tuning_knobs_keep_verdicts(star, knob, values):
    """Every value of the autotuner's knobs (edge tile, tree levels staged in shared memory, lanes
    per query of the warp surrogate pass) gives the oracle's verdicts, in a small batch (leaf-table
    polygon pass, warp surrogate pass) and a large one (staged large-batch polygon pass)."""
    lay, oeng, geng = star
    saved = geng.get_tuning()
    try:
        for n, sid in ((4096, 31), (1 << 18, 32)):
            q = W.queries_for(lay, n, 0xC1, sid=sid)
            ref = oeng.detect_batch(q, ignored=lay.filter_keys)
            for val in values:
                geng.set_tuning(**{knob: val})
                got = gpu_detect(geng, q, filter=lay.filter_keys)
                assert np.array_equal(got, ref), (knob, val, n, int((got != ref).sum()))
    finally:
        geng.set_tuning(**saved)


def test_autotune_reports_the_three_knobs(star):
    lay, oeng, geng = star
    q = W.queries_for(lay, 1 << 17, 0xA8, sid=9)
    saved = geng.get_tuning()
    try:
        t, ms = geng.autotune(torch_queries(q), filter=lay.filter_keys)
        assert t["edge_tile"] in (4, 8, 16) and t["surrogate_lanes"] in (8, 16, 32) and 0 <= t["staging_depth"] <= 4
        assert np.array_equal(gpu_detect(geng, q, filter=lay.filter_keys), oeng.detect_batch(q, ignored=lay.filter_keys))
    finally:
        geng.set_tuning(**saved)


def test_boundary_queries_detect_and_collect(star, oracle_mod):
    lay, oeng, geng = star
    q = W.boundary_queries(lay, 1 << 16, 0xB0)
    got = gpu_detect(geng, q, filter=lay.filter_keys)
    assert np.array_equal(got, oeng.detect_batch(q, ignored=lay.filter_keys))
    assert 0.05 < got.mean() < 0.99
    sub = q[:8192]
    rc, rids = oeng.collect_batch(sub, ignored=lay.filter_keys)
    assert gpu_collect(geng, sub, filter=lay.filter_keys) == oracle_sets(rc, rids)
