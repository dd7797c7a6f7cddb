"""Strip-packing instances in the reference's JSON format (jcde.instance) and their LBF build."""
import json
import os

import numpy as np
import pytest

from jcde import instance as I
from jcde import lbf
from jcde import workload as W

# A small instance of our own in the reference's format: every shape kind and orientation rule.
DEMO = {
    "name": "demo",
    "strip_height": 200.0,
    "items": [
        {"id": 0, "demand": 3, "allowed_orientations": [0.0, 90.0, 180.0, 270.0],
         "shape": {"type": "simple_polygon", "data": [[0, 0], [60, 0], [60, 20], [20, 20], [20, 50], [0, 50]]}},
        {"id": 1, "demand": 2, "shape": {"type": "rectangle", "data": {"x_min": 5.0, "y_min": -3.0, "width": 40.0,
                                                                        "height": 25.0}}},
        {"id": 2, "demand": 4, "allowed_orientations": [0.0],
         "shape": {"type": "simple_polygon", "data": [[0, 0], [45, 0], [10, 35]]}},
        {"id": 3, "demand": 2, "allowed_orientations": [45.0, 135.0],
         "shape": {"type": "polygon", "data": {"outer": [[0, 0], [50, 0], [50, 50], [0, 50]],
                                               "inner": [[[10, 10], [40, 10], [40, 40], [10, 40]]]}}},
        {"id": 4, "demand": 1, "allowed_orientations": [],
         "shape": {"type": "simple_polygon", "data": [[0, 0], [70, 10], [65, 40], [10, 30]]}},
    ],
}


def test_load_and_setup(oracle_mod):
    inst = I.load_spp(json.dumps(DEMO))
    assert inst.name == "demo" and inst.strip_height == 200.0 and len(inst.items) == 5
    assert inst.items[1].orientations is None and inst.items[2].orientations == [] and inst.items[4].orientations == []
    assert np.array_equal(inst.items[1].xy, W.rect_polygon(5.0, -3.0, 45.0, 22.0))
    assert len(inst.items[3].xy) == 4   # the outer boundary only (the importer ignores item holes)
    with pytest.raises(ValueError):
        I.load_spp({"strip_height": 1, "items": [{"id": 0, "shape": {"type": "multi_polygon", "data": []}}]})
    su = I.setup_spp(oracle_mod.OracleBackend, inst, 800.0)
    assert len(su.sequence) == 12
    diam = [float(np.float32(it.diameter)) for it in su.layout.items]
    order = [int(su.sequence[0])] + [int(b) for a, b in zip(su.sequence, su.sequence[1:]) if a != b]
    assert [diam[i] for i in order] == sorted(diam, reverse=True)   # descending diameter
    assert su.orient[1] is None and len(su.orient[0]) == 4 and len(su.orient[2]) == 1
    cs = I.orientation_cs([0.0, 90.0, 180.0, 270.0])
    assert np.array_equal(np.abs(cs), np.array([[1, 0], [0, 1], [1, 0], [0, 1]], np.float32))
    assert np.array_equal(np.sign(cs[:, 1]), [0, 1, 0, -1])


def test_instance_build_on_the_oracle(oracle_mod):
    su = I.setup_spp(oracle_mod.OracleBackend, I.load_spp(DEMO), 800.0)
    spec = lbf.spec_for_instance(su, n_cand=1024, ls_rounds=2, ls_cand=256)
    log = lbf.run_host(su.layout, su.engine, spec)
    assert len(log.placements) == 12
    o0 = su.orient[0]
    for p in log.placements:
        if int(p[3]) == 0:   # a discrete item keeps one of its allowed orientations
            cs = np.array([np.uint32(p[4]).view(np.float32), np.uint32(p[5]).view(np.float32)])
            assert (o0 == cs).all(axis=1).any()


from helpers import reference_asset  # noqa: E402

REF_ASSET = reference_asset("swim.json")


@pytest.mark.skipif(not (REF_ASSET and os.path.exists(REF_ASSET)), reason="JCDE_REFERENCE_ASSETS not set")
def test_reference_instance_imports(oracle_mod):
    """A reference instance read in place: parsed, imported, and a few LBF steps run on the oracle."""
    inst = I.load_spp(REF_ASSET)
    assert len(inst.items) > 0 and inst.strip_height > 0
    su = I.setup_spp(oracle_mod.OracleBackend, inst, 4.0 * inst.strip_height)
    assert len(su.sequence) == sum(it.demand for it in inst.items)
    spec = lbf.spec_for_instance(su, n_cand=512)
    log = lbf.run_host(su.layout, su.engine, spec, steps=4)
    assert len(log.placements) == 4


def test_import_simple_polygon_rules(oracle_mod):
    closed = [[0, 0], [10, 0], [10, 10], [10, 10], [0, 10], [0, 0]]
    xy = I.import_simple_polygon(closed)
    assert xy.tolist() == [[0, 0], [10, 0], [10, 10], [0, 10]]
    near = [[0, 0], [10, 0], [10, np.nextafter(np.float32(0), np.float32(1))], [10, 10], [0, 10]]
    assert len(I.import_simple_polygon(near)) == 4   # 1 ULP apart counts as the same vertex
    with pytest.raises(ValueError):
        I.import_simple_polygon([[0, 0], [10, 0], [5, 5], [10, 10], [5, 5], [0, 10]])
    for a, b in ((1.0, 1.0), (0.0, 1e-8), (1.0, float(np.nextafter(np.float32(1), np.float32(2))))):
        assert I.fpa_eq32(a, b) == oracle_mod.fpa_eq(a, b)
    assert not I.fpa_eq32(1.0, 1.001) and not oracle_mod.fpa_eq(1.0, 1.001)


def test_export_solution_moves_the_original_shapes(oracle_mod):
    """Exported transformations applied to the original shapes give the placed hazards' vertices."""
    inst = I.load_spp(DEMO)
    su = I.setup_spp(oracle_mod.OracleBackend, inst, 800.0)
    spec = lbf.spec_for_instance(su, n_cand=1024)
    log = lbf.run_host(su.layout, su.engine, spec)
    sol = I.export_solution(su, inst, log.placements)
    assert len(sol["placed_items"]) == 12 and 0.0 < sol["density"] < 1.0
    for p, e in zip(log.placements, sol["placed_items"]):
        t = int(p[3])
        assert e["item_id"] == inst.items[t].id
        c, s, tx, ty = (np.uint32(v).view(np.float32) for v in p[4:8])
        want = W.transform_points(su.layout.items[t].xy, c, s, tx, ty).astype(np.float64)
        raw = inst.items[t].xy.astype(np.float64)
        a = np.radians(e["transformation"]["rotation"])
        got = raw @ np.array([[np.cos(a), np.sin(a)], [-np.sin(a), np.cos(a)]]) + e["transformation"]["translation"]
        # the importer may reverse a clockwise outline: compare as point sets
        assert np.abs(np.sort(got, axis=0) - np.sort(want, axis=0)).max() < 1e-2
