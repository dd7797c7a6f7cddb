"""Known-answer tests of the oracle's primitives (hand-derived cases).

The reference ships no unit tests or golden vectors for these functions, so each case below is
worked out by hand from the reference source (file:line in each test) — they pin the restatement.
"""
import numpy as np
import pytest

f32 = np.float32


def nxt(x, k=1):
    x = f32(x)
    for _ in range(k):
        x = np.nextafter(x, f32(np.inf))
    return x


@pytest.mark.parametrize(
    "a,b,eq",
    [
        (1.0, 1.0, True),
        (-0.0, 0.0, True),                    # exact equality first (float-cmp approx_eq)
        (0.0, 1e-7, True),                    # |a-b| <= f32::EPSILON
        (0.0, 2e-7, False),                   # beyond epsilon, and billions of ULPs apart
        (1e-40, -1e-40, True),                # opposite signs but within epsilon
        (1000.0, float(nxt(1000.0, 4)), True),   # 4 ULPs
        (1000.0, float(nxt(1000.0, 5)), False),  # 5 ULPs, 3e-4 > epsilon
        (1.0, -1.0, False),
    ],
)
def test_fpa_eq(oracle_mod, a, b, eq):
    """util/fpa.rs:18-23 with float-cmp's default F32Margin (epsilon, 4 ULPs)."""
    assert oracle_mod.fpa_eq(a, b) == eq
    assert oracle_mod.fpa_eq(b, a) == eq


@pytest.mark.parametrize(
    "e1,e2,hit",
    [
        ((0, 0, 2, 2), (0, 2, 2, 0), True),      # proper crossing
        ((0, 0, 1, 0), (0, 1, 1, 1), False),     # parallel, bboxes apart
        ((0, 0, 2, 0), (1, 0, 3, 0), False),     # collinear overlap: t_denom == 0 -> "parallel"
        ((0, 0, 1, 1), (1, 1, 2, 0), True),      # shared endpoint: t, u in {0, 1}
        ((0, 0, 2, 0), (1, 0, 1, 1), True),      # T-junction
        ((0, 0, 1, 0), (2, -1, 2, 1), False),    # bbox early-out (edge.rs:187-204)
        ((0, 0, 4, 4), (0, 4, 1, 3), False),     # lines cross at (2,2), outside e2
    ],
)
def test_edge_intersection(oracle_mod, e1, e2, hit):
    """geometry/primitives/edge.rs:180-228."""
    assert oracle_mod.edge_intersection(e1, e2) == hit


@pytest.mark.parametrize(
    "edge,hit",
    [
        ((-1, 0.5, 2, 0.5), True),      # crosses, no endpoint inside
        ((2, 2, 3, 3), False),          # bbox disjoint
        ((-1, -1, 2, 2), True),         # diagonal through
        ((0.5, 0.5, 0.7, 0.7), True),   # endpoint inside
        ((0.5, 2, 2, 0.5), False),      # bboxes overlap, all corners on one side (x+y=2.5)
        ((-1, 1.5, 1.5, -1), True),     # x+y=0.5 cuts the corner region
    ],
)
def test_rect_collides_edge(oracle_mod, edge, hit):
    """geometry/primitives/rect.rs:301-345 against the unit square."""
    assert oracle_mod.rect_collides_edge((0, 0, 1, 1), edge) == hit


SQUARE = [(0, 0), (1, 0), (1, 1), (0, 1)]
DIAMOND = [(1, 0), (2, 1), (1, 2), (0, 1)]
L_SHAPE = [(0, 0), (3, 0), (3, 1), (1, 1), (1, 3), (0, 3)]


@pytest.mark.parametrize(
    "poly,p,inside",
    [
        (SQUARE, (0.5, 0.5), True),
        (SQUARE, (1.5, 0.5), False),     # outside the bbox (simple_polygon.rs:258)
        (SQUARE, (0.5, 0.0), False),     # on the bottom edge: vertex guard counts nothing
        (DIAMOND, (1.0, 1.0), True),     # ray through vertex (2,1): counted once, edge below the ray
        (L_SHAPE, (2.0, 2.0), False),    # in the notch of the L
        (L_SHAPE, (0.5, 2.0), True),
        (L_SHAPE, (2.0, 0.5), True),
    ],
)
def test_point_in_polygon(oracle_mod, poly, p, inside):
    """Ray casting with the FPA vertex guard (simple_polygon.rs:255-292)."""
    assert oracle_mod.point_in_poly(poly, p) == inside


@pytest.mark.parametrize(
    "a,b,rel",
    [
        ((0, 0, 10, 10), (1, 1, 2, 2), 2),                    # Surrounding
        ((0, 0, 10, 10), (0, 0, 10, float(nxt(10.0))), 2),    # 1 ULP over: still Surrounding
        ((0, 0, 1, 1), (2, 2, 3, 3), 3),                      # Disjoint
        ((0, 0, 2, 2), (1, 1, 3, 3), 0),                      # Intersecting
        ((1, 1, 2, 2), (0, 0, 3, 3), 1),                      # Enclosed
        ((0, 0, 1, 1), (float(nxt(1.0, 3)), 0, 2, 1), 0),     # 3 ULPs apart: almost touching
    ],
)
def test_almost_relation(oracle_mod, a, b, rel):
    """geometry/primitives/rect.rs:70-89 (0 Intersecting, 1 Enclosed, 2 Surrounding, 3 Disjoint)."""
    assert oracle_mod.almost_relation(a, b) == rel


@pytest.mark.parametrize(
    "edge,expect",
    [
        ((1, 1, 3, 1), [False, False, True, True]),      # endpoints in q2 and q3
        ((0.5, 3.9, 3.9, 0.5), [True, True, False, True]),  # q0 found by the h-bisector half test
        ((1, 3, 1.5, 3.5), [False, True, False, False]),
        ((-1, 2.5, 5, 2.5), [True, True, False, False]),   # no endpoint inside: side tests
    ],
)
def test_edge_quadrants_known(oracle_mod, edge, expect):
    """Edge::collides_with_quadrants (qt_traits.rs:19-106) over the box (0,0,4,4)."""
    assert oracle_mod.edge_quadrants(edge, (0, 0, 4, 4)) == expect


def test_edge_quadrants_cover_individual_tests(oracle_mod):
    """The debug assertion of qt_traits.rs:87-102: every quadrant an edge collides with is flagged."""
    rng = np.random.default_rng(0)
    for _ in range(3000):
        r = np.sort(rng.uniform(-10, 10, 2))
        s = np.sort(rng.uniform(-10, 10, 2))
        box = (r[0], s[0], r[1], s[1])
        e = rng.uniform(-12, 12, 4)
        got = oracle_mod.edge_quadrants(e, box)
        cx, cy = (f32(box[0]) + f32(box[2])) / f32(2), (f32(box[1]) + f32(box[3])) / f32(2)
        corners = [(box[2], box[3]), (box[0], box[3]), (box[0], box[1]), (box[2], box[1])]
        for i, (x, y) in enumerate(corners):
            q = (min(x, cx), min(y, cy), max(x, cx), max(y, cy))
            if oracle_mod.rect_collides_edge(q, e):
                assert got[i], (e, box, i)


def test_centroid_matches_generator(oracle_mod):
    """SPolygon::centroid (simple_polygon.rs:173-192): oracle vs the workload generator's f32 loop."""
    from jcde import workload as W

    st = W.Stream(1, 1)
    for _ in range(20):
        xy = W.star_polygon(st, int(st.randint(8, 60, 1)[0]), 20.0, 60.0)
        xo, _, area, _, _ = oracle_mod.OracleBackend.spolygon_new(xy)
        a = oracle_mod.centroid(xo, area)
        b = W.centroid_f32(xo, area)
        assert a[0] == b[0] and a[1] == b[1]
