"""Shape preparation on the device (jcde.prep): poi and surrogate poles of many shapes per launch,
bit-exact with the oracle's compute_pole / generate_surrogate_poles (fail_fast/pole.rs:12-77)."""
import numpy as np
import pytest

from jcde import workload as W

gpu = pytest.mark.gpu


def _shapes():
    """Star items as in the star-container layout (8-200 vertices), shapes with exact distance ties
    (rectangles, a square, regular polygons, an L), a thin sliver and a 64-vertex container."""
    st = W.Stream(0xC1, 1)
    out = []
    for _ in range(24):
        nv = int(st.randint(8, 200, 1)[0])
        out.append(W.star_polygon(st, nv, 20.0, 60.0))
    out.append(W.rect_polygon(0.0, 0.0, 40.0, 25.0))
    out.append(W.rect_polygon(-10.0, -10.0, 10.0, 10.0))
    out.append(W.rect_polygon(5.0, -3.0, 45.0, 22.0))
    for k in (3, 6, 8, 12):
        a = np.arange(k) * (2 * np.pi / k)
        out.append(np.stack([30 * np.cos(a), 30 * np.sin(a)], 1).astype(np.float32))
    out.append(np.array([[0, 0], [60, 0], [60, 20], [20, 20], [20, 50], [0, 50]], np.float32))
    out.append(np.array([[0, 0], [200, 0], [200, 1.5], [0, 2.0]], np.float32))
    out.append(W.star_polygon(W.Stream(0xC1, 9), 64, 2000.0, 2000.0))
    return out


@gpu
def test_poi_batch_matches_oracle(oracle_mod, jcde_mod):
    from jcde import prep

    raws = _shapes()
    shapes = [prep.spolygon_shape(r) for r in raws]
    got = prep.poi_batch([s[0] for s in shapes])
    for i, r in enumerate(raws):
        xy, bbox, area, diam, poi = oracle_mod.OracleBackend.spolygon_new(r)
        assert np.array_equal(shapes[i][0], xy) and np.array_equal(shapes[i][1], bbox)
        assert shapes[i][2] == area and shapes[i][3] == diam
        assert np.array_equal(got[i].view(np.uint32), poi.view(np.uint32)), (i, got[i], poi)


@gpu
def test_import_items_matches_oracle(oracle_mod, jcde_mod):
    """Importer::import_item on the device batch: every Item field equal to the oracle's, bit for bit."""
    from jcde import prep

    raws = _shapes()
    dev = prep.import_items(raws)
    assert len(dev) == len(raws)
    for i, r in enumerate(raws):
        ref = W.import_item(oracle_mod.OracleBackend, r)
        d = dev[i]
        assert np.array_equal(d.xy.view(np.uint32), ref.xy.view(np.uint32))
        assert np.array_equal(d.poi.view(np.uint32), ref.poi.view(np.uint32))
        assert d.poles.shape == ref.poles.shape, (i, d.poles.shape, ref.poles.shape)
        assert np.array_equal(d.poles.view(np.uint32), ref.poles.view(np.uint32)), i
        assert (d.n_ff_poles, d.area, d.diameter, d.centroid) == (ref.n_ff_poles, ref.area, ref.diameter, ref.centroid)


@gpu
def test_pole_limits_and_capacity(oracle_mod, jcde_mod):
    """Other coverage limits, an output too small for the poles (status 5, then the retry), and the
    per-shape status of an invalid shape."""
    import torch

    from jcde import prep

    raws = _shapes()[:6]
    items = [W.import_item(oracle_mod.OracleBackend, r) for r in raws]
    limits = ((40, 0.0), (6, 0.5))
    ref = [oracle_mod.OracleBackend.surrogate_poles(it.xy, it.area, it.poi, limits) for it in items]
    got = prep.surrogate_poles_batch([it.xy for it in items], [it.area for it in items],
                                     np.stack([it.poi for it in items]), limits, cap=2)
    for g, r in zip(got, ref):
        assert np.array_equal(g.view(np.uint32), r.view(np.uint32))
    b = prep.ShapeBatch([items[0].xy, items[1].xy[:2], items[2].xy])
    area = torch.tensor([items[0].area, 1.0, items[2].area], dtype=torch.float32, device="cuda")
    poi = torch.from_numpy(np.stack([items[0].poi, items[0].poi, items[2].poi])).cuda()
    out, cnt, st = b.poles(area, poi, limits, cap=64)
    assert st.cpu().tolist() == [0, 1, 0] and cnt.cpu().tolist()[1] == 0
    assert np.array_equal(out[2, : int(cnt[2])].cpu().numpy().view(np.uint32), ref[2].view(np.uint32))
    with pytest.raises(Exception):
        prep.poi_batch([items[0].xy, items[1].xy[:2]])


@gpu
def test_item_pool_of_the_lbf_build(oracle_mod, jcde_mod):
    """The 60 item types of the LBF build (8-120 vertices) prepared on the device give the same
    layout items as the host preparation."""
    from jcde import lbf, prep

    spec = lbf.LbfSpec()
    lay, _ = lbf.setup(oracle_mod.OracleBackend, spec)
    raws = lbf.raw_shapes(spec)
    dev = prep.import_items(raws)
    for d, ref in zip(dev, lay.items):
        assert np.array_equal(d.poles.view(np.uint32), ref.poles.view(np.uint32))
        assert np.array_equal(d.xy.view(np.uint32), ref.xy.view(np.uint32))


@gpu
@pytest.mark.parametrize("tol", [0.0, 0.001, 0.01, 0.05, 0.3])
def test_simplify_batch_matches_oracle(oracle_mod, jcde_mod, tol):
    """simplify_shape on the device (one warp per shape), both modes, bit-exact with the oracle."""
    from jcde import prep

    raws = _shapes()
    shapes, areas = [], []
    for r in raws:
        xy, _, area, _, _ = oracle_mod.OracleBackend.spolygon_new(r)
        shapes.append(xy)
        areas.append(area)
    for deflate in (False, True):
        got = prep.simplify_batch(shapes, areas, deflate, tol)
        for i, (xy, a) in enumerate(zip(shapes, areas)):
            ref = oracle_mod.OracleBackend.simplify_shape(xy, a, deflate, tol)
            assert got[i].shape == ref.shape and np.array_equal(got[i].view(np.uint32), ref.view(np.uint32)), \
                (i, deflate, len(got[i]), len(ref))


@gpu
def test_import_items_simplified_matches_oracle(oracle_mod, jcde_mod):
    """Importer::import_item with lbf's default simplification (0.001) and a coarse one: simplified
    shape, recomputed poi, poles, area and diameter all equal to the oracle's import."""
    from jcde import prep

    raws = _shapes()[:16] + _shapes()[24:]
    for tol in (0.001, 0.05):
        dev = prep.import_items(raws, simplify_tolerance=tol)
        for i, r in enumerate(raws):
            ref = W.import_item(oracle_mod.OracleBackend, r, simplify_tolerance=tol)
            d = dev[i]
            assert np.array_equal(d.xy.view(np.uint32), ref.xy.view(np.uint32)), (tol, i)
            assert np.array_equal(d.poi.view(np.uint32), ref.poi.view(np.uint32)), (tol, i)
            assert np.array_equal(d.poles.view(np.uint32), ref.poles.view(np.uint32)), (tol, i)
            assert (d.area, d.diameter, d.centroid) == (ref.area, ref.diameter, ref.centroid)


@gpu
def test_batch_wider_than_the_gpu(oracle_mod, jcde_mod):
    """More shapes than SMs: the 512-thread CTAs, several shapes per CTA from the counter."""
    from jcde import prep

    st = W.Stream(0xC0, 3)
    raws = [W.star_polygon(st, int(st.randint(8, 24, 1)[0]), 20.0, 60.0) for _ in range(200)]
    dev = prep.import_items(raws)
    for d, r in zip(dev, raws):
        ref = W.import_item(oracle_mod.OracleBackend, r)
        assert np.array_equal(d.poi.view(np.uint32), ref.poi.view(np.uint32))
        assert np.array_equal(d.poles.view(np.uint32), ref.poles.view(np.uint32))


@gpu
def test_import_items_lbf_default_matches_oracle(oracle_mod, jcde_mod):
    """lbf's default import (simplify 0.001, close concavities at 1% and 20% of the diameter,
    simplify again at a tenth): the device batch import equals the oracle's, bit for bit."""
    from jcde import prep

    raws = _shapes()[:12]
    for ratio in (0.01, 0.2):
        dev = prep.import_items(raws, simplify_tolerance=0.001, narrow_concavity_ratio=ratio)
        for i, r in enumerate(raws):
            ref = W.import_item(oracle_mod.OracleBackend, r, simplify_tolerance=0.001, narrow_concavity_ratio=ratio)
            assert np.array_equal(dev[i].xy.view(np.uint32), ref.xy.view(np.uint32)), (ratio, i)
            assert np.array_equal(dev[i].poles.view(np.uint32), ref.poles.view(np.uint32)), (ratio, i)
