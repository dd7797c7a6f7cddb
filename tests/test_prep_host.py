"""Host side of the batched item preparation (jcde.prep): SPolygon::new without its poi over many
shapes in one call, and the centroids / centring vectorised across shapes."""
import numpy as np

from jcde import prep
from jcde import workload as W


def _raws():
    st = W.Stream(0xC2, 7)
    raws = [W.star_polygon(st, int(st.randint(3, 200, 1)[0]), 20.0, 60.0) for _ in range(96)]
    raws.append(raws[0][::-1].copy())   # clockwise: reversed into the internal order
    raws.append(W.rect_polygon(5.0, -3.0, 45.0, 22.0))
    return raws


def test_spolygon_batch_equals_single(jcde_mod):
    raws = _raws()
    flat, off, bb, ad = prep.spolygon_batch(raws, n_threads=4)
    for i, r in enumerate(raws):
        xo, b, a, d = prep.spolygon_shape(r)
        full = jcde_mod.spolygon_new(r)
        assert np.array_equal(xo, flat[off[i]: off[i + 1]]) and np.array_equal(xo, full[0])
        assert np.array_equal(b, bb[i]) and a == ad[i, 0] == full[2] and d == ad[i, 1] == full[3]


def test_spolygon_batch_rejects_invalid(jcde_mod):
    import pytest

    bad = np.array([[0, 0], [1, 0], [0, 0], [0, 1]], np.float32)   # a repeated vertex
    with pytest.raises(Exception):
        prep.spolygon_batch([W.rect_polygon(0, 0, 1, 1), bad])


def test_centroids_vectorised(jcde_mod):
    """The centroids of the batch call (C++) and of the vectorised numpy form equal the scalar
    float32 sums of workload.centroid_f32 bit for bit."""
    raws = _raws()
    flat, off, _, ad, cen = prep.spolygon_batch(raws, centroids=True)
    shapes = [flat[off[i]: off[i + 1]] for i in range(len(raws))]
    cv = W.centroids_f32(shapes, ad[:, 0])
    ref = np.array([W.centroid_f32(s, a) for s, a in zip(shapes, ad[:, 0])], np.float32)
    assert np.array_equal(cv.view(np.uint32), ref.view(np.uint32))
    assert np.array_equal(cen.view(np.uint32), ref.view(np.uint32))
