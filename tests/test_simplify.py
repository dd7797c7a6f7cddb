"""Shape simplification (shape_modification.rs:48-144) in the oracle: the invariants the reference
states for it, on star items, concave shapes and the reference's own instances."""
import glob
import json
import os

import numpy as np
import pytest

from jcde import workload as W

from helpers import REFERENCE_ASSETS as REF_ASSETS  # noqa: E402


def _stars(n=24, seed=0xC2):
    st = W.Stream(seed, 7)
    return [W.star_polygon(st, int(st.randint(8, 200, 1)[0]), 20.0, 60.0) for _ in range(n)]


@pytest.mark.parametrize("tol", [0.001, 0.01, 0.05, 0.2])
def test_simplify_invariants(oracle_mod, tol):
    """Fewer or equal vertices, area change within the tolerance, Inflate never shrinks and Deflate
    never grows the shape, and the result is a valid simple polygon (SPolygon::new accepts it)."""
    B = oracle_mod.OracleBackend
    for raw in _stars():
        xy, _, area, _, _ = B.spolygon_new(raw)
        for deflate in (False, True):
            s = B.simplify_shape(xy, area, deflate, tol)
            assert 3 <= len(s) <= len(xy)
            s_xy, _, s_area, _, _ = B.spolygon_new(s)
            assert abs(float(s_area) - float(area)) / float(area) <= tol * (1 + 1e-5)
            assert (s_area <= area) if deflate else (s_area >= area)
            assert np.array_equal(s_xy, s)   # stays counter-clockwise


def test_simplify_keeps_what_it_cannot_change(oracle_mod):
    B = oracle_mod.OracleBackend
    rect = W.rect_polygon(0.0, 0.0, 10.0, 5.0)
    assert np.array_equal(B.simplify_shape(rect, 50.0, False, 0.5), rect)   # 4 convex corners, no 4th-vertex removal
    tri = np.array([[0, 0], [4, 0], [0, 3]], np.float32)
    assert np.array_equal(B.simplify_shape(tri, 6.0, False, 0.5), tri)      # fewer than 4 vertices
    # a collinear vertex costs no area: removed at any tolerance
    sq = np.array([[0, 0], [5, 0], [10, 0], [10, 10], [0, 10]], np.float32)
    out = B.simplify_shape(sq, 100.0, False, 0.0)
    assert len(out) == 4 and not any((out == [5, 0]).all(1))
    # tolerance 0 keeps every corner that changes the area
    star = _stars(1)[0]
    xy, _, area, _, _ = B.spolygon_new(star)
    assert len(B.simplify_shape(xy, area, False, 0.0)) == len(xy)


def test_import_item_with_simplification(oracle_mod):
    """lbf's default import (tolerance 0.001): the internal shape is simplified, its poi recomputed,
    the item keeps the original area."""
    B = oracle_mod.OracleBackend
    raw = _stars(1)[0]
    plain = W.import_item(B, raw)
    simp = W.import_item(B, raw, simplify_tolerance=0.05)
    assert len(simp.xy) < len(plain.xy) and simp.area == plain.area
    assert simp.poles[0].tolist() == simp.poi.tolist()


def _ref_instances():
    return sorted(glob.glob(os.path.join(REF_ASSETS, "*.json")))


@pytest.mark.skipif(not (REF_ASSETS and os.path.isdir(REF_ASSETS)), reason="JCDE_REFERENCE_ASSETS not set")
def test_reference_instances_simplify(oracle_mod):
    """Every simple-polygon item of the reference's instances (read in place) simplifies at lbf's
    default tolerance within its invariants."""
    from jcde import instance as I

    B = oracle_mod.OracleBackend
    seen = 0
    for path in _ref_instances():
        try:
            inst = I.load_spp(path)
        except (KeyError, ValueError, json.JSONDecodeError):
            continue   # bin-packing or other formats
        for it in inst.items[:8]:
            xy, _, area, _, _ = B.spolygon_new(it.xy)
            s = B.simplify_shape(xy, area, False, 0.001)
            _, _, s_area, _, _ = B.spolygon_new(s)
            assert len(s) <= len(xy) and s_area >= area
            assert abs(float(s_area) - float(area)) / float(area) <= 0.001 * (1 + 1e-5)
            seen += 1
    assert seen > 0


@pytest.mark.parametrize("ratio", [0.01, 0.05, 0.2])
def test_close_concavities_product_equals_oracle(oracle_mod, jcde_mod, ratio):
    """close_narrow_concavities: the product's host implementation (jcde_close_concavities) and
    the oracle's give the same vertices, in both modes; bridges only ever remove vertices."""
    from jcde import prep

    B = oracle_mod.OracleBackend
    shapes = _stars(16, seed=0xCC)
    shapes.append(np.array([[0, 0], [60, 0], [60, 20], [21, 20], [21, 50], [19, 50], [19, 20], [0, 20]], np.float32))
    changed = 0
    for raw in shapes:
        xy, _, area, _, _ = B.spolygon_new(raw)
        for deflate in (False, True):
            a = B.close_concavities(xy, deflate, ratio)
            b = prep.close_concavities(xy, deflate, ratio)
            assert a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))
            assert len(a) <= len(xy)
            changed += len(a) < len(xy)
    if ratio >= 0.05:
        assert changed > 0


def test_lbf_default_import(oracle_mod):
    """lbf's default import: simplify 0.001, close concavities under 1% of the diameter, simplify
    0.0001; the result never has more vertices than the plain simplification."""
    B = oracle_mod.OracleBackend
    for raw in _stars(6, seed=0xCD):
        a = W.import_item(B, raw, simplify_tolerance=0.001)
        b = W.import_item(B, raw, simplify_tolerance=0.001, narrow_concavity_ratio=0.01)
        assert len(b.xy) <= len(a.xy) and b.area == a.area


def test_known_answers(oracle_mod):
    """Hand-derived cases.  A notch 1 unit wide and 10 deep in a 20 x 20 square: at a 20% cutoff
    (diameter 28.3, so bridges up to 5.66) the notch is bridged (Inflate) and its two inner
    vertices go; at 1% nothing is short enough.  Deflate never bridges outside the shape."""
    B = oracle_mod.OracleBackend
    notch = np.array([[0, 0], [20, 0], [20, 20], [10.5, 20], [10.5, 10], [9.5, 10], [9.5, 20], [0, 20]],
                     np.float32)
    xy, _, area, diam, _ = B.spolygon_new(notch)
    assert abs(float(diam) - 20 * np.sqrt(2)) < 1e-3
    closed = B.close_concavities(xy, False, 0.2)
    assert len(closed) == 6
    assert not any((closed == [10.5, 10]).all(1)) and not any((closed == [9.5, 10]).all(1))
    assert len(B.close_concavities(xy, False, 0.01)) == 8
    assert len(B.close_concavities(xy, True, 0.2)) == 8
    # simplify_shape on the notch: the concave corners are the cheapest candidates; removing one
    # changes the area by 5 (a triangle of half 1 x 10), 1.25% of 395
    s1 = B.simplify_shape(xy, area, False, 0.02)
    _, _, a1, _, _ = B.spolygon_new(s1)
    assert len(s1) < 8 and float(a1) > float(area)
    assert len(B.simplify_shape(xy, area, False, 0.001)) == 8
