"""Bin packing (jcde.bpp): the reference's ExtBPInstance import and the lbf_bpp.rs optimizer on the
oracle engine."""
import os

import numpy as np
import pytest

from jcde import bpp
from jcde import workload as W

from helpers import reference_asset  # noqa: E402

REF_BALDACCI = reference_asset("baldacci1.json")


def test_load_rules():
    d = bpp.synthetic_instance(n_types=6, n_bins=3)
    inst = bpp.load_bpp(d)
    assert [it.id for it in inst.items] == list(range(6)) and len(inst.bins) == 3
    assert inst.items[4].min_quality == 1 and inst.items[0].min_quality is None
    # holes become quality-0 zones, zones sorted by quality
    assert [q for q, _ in inst.bins[1].zones] == [0, 1, 2] and [q for q, _ in inst.bins[0].zones] == [1, 2]
    # zero demand / stock are dropped; the remaining ids must be 0..n-1
    d["items"][5]["demand"] = 0
    assert len(bpp.load_bpp(d).items) == 5
    d["items"][2]["demand"] = 0
    with pytest.raises(ValueError):
        bpp.load_bpp(d)


def _replay_free(oracle_mod, su, log):
    """Every placement is collision-free in its layout given the items placed there before it."""
    B = oracle_mod.OracleBackend
    engines = {}
    for row in log.placements:
        li, b, t = int(row[1]), int(row[2]), int(row[3])
        if li not in engines:
            engines[li] = bpp._bin_engine(B, su, b)
        eng, keys = engines[li]
        c, s, tx, ty = (np.uint32(v).view(np.float32) for v in row[5:9])
        q = np.zeros(1, dtype=W.QUERY_DTYPE)
        q["item"], q["cos"], q["sin"], q["tx"], q["ty"] = t, c, s, tx, ty
        filt = bpp.quality_filter(su.bins[b], keys, su.instance.items[t].min_quality)
        assert int(eng.detect_batch(q, filt)[0]) == 0
        hz = W.placed_hazard(su.items[t], t, c, s, tx, ty)
        eng.register_hazard(hz.kind, hz.dynamic, hz.xy, hz.poi, 1)


def test_run_on_the_oracle(oracle_mod):
    inst = bpp.load_bpp(bpp.synthetic_instance(n_types=12, n_bins=3))
    su = bpp.setup_bpp(oracle_mod.OracleBackend, inst)
    log = bpp.run_bpp(oracle_mod.OracleBackend, su, bpp.BppSpec(n_cand=512))
    placed = len(log.placements) + sum(log.unplaced.values())
    assert len(log.placements) > 0 and placed <= sum(it.demand for it in inst.items)
    # bins are opened within their stock, the item order is the placement order
    for b in range(len(inst.bins)):
        assert log.layouts.count(b) <= inst.bins[b].stock
    seen = [int(r[3]) for r in log.placements]
    ranks = {t: k for k, t in enumerate(su.order)}
    assert all(ranks[a] <= ranks[b] for a, b in zip(seen, seen[1:]))
    _replay_free(oracle_mod, su, log)
    sol = bpp.export_solution(su, log)
    assert sol["cost"] == sum(inst.bins[b].cost for b in log.layouts)
    assert 0.0 < sol["density"] <= 1.0 and sum(len(l["placed_items"]) for l in sol["layouts"]) == len(log.placements)
    # reproducible
    log2 = bpp.run_bpp(oracle_mod.OracleBackend, bpp.setup_bpp(oracle_mod.OracleBackend, inst), bpp.BppSpec(n_cand=512))
    assert log2.same_as(log)


def test_items_that_fit_nowhere(oracle_mod):
    """A type too large for every bin is skipped with its copies (lbf_bpp.rs:70), the rest placed."""
    d = bpp.synthetic_instance(n_types=4, n_bins=1)
    d["items"][0]["shape"] = {"type": "rectangle", "data": {"x_min": 0, "y_min": 0, "width": 5000, "height": 5000}}
    inst = bpp.load_bpp(d)
    su = bpp.setup_bpp(oracle_mod.OracleBackend, inst)
    log = bpp.run_bpp(oracle_mod.OracleBackend, su, bpp.BppSpec(n_cand=256))
    assert log.unplaced.get(0) == inst.items[0].demand
    assert 0 not in [int(r[3]) for r in log.placements]


@pytest.mark.skipif(not (REF_BALDACCI and os.path.exists(REF_BALDACCI)), reason="JCDE_REFERENCE_ASSETS not set")
def test_reference_instance_on_the_oracle(oracle_mod):
    """A reference bin-packing instance with quality zones, read in place, packed on the oracle."""
    inst = bpp.load_bpp(REF_BALDACCI)
    assert any(it.min_quality is not None for it in inst.items) and all(b.zones for b in inst.bins)
    su = bpp.setup_bpp(oracle_mod.OracleBackend, inst)
    log = bpp.run_bpp(oracle_mod.OracleBackend, su, bpp.BppSpec(n_cand=512))
    assert len(log.placements) + sum(log.unplaced.values()) == sum(it.demand for it in inst.items)
    _replay_free(oracle_mod, su, log)


@pytest.mark.skipif(not (REF_BALDACCI and os.path.exists(REF_BALDACCI)), reason="JCDE_REFERENCE_ASSETS not set")
def test_reference_instance_lbf_default_import(oracle_mod):
    """The reference instance imported as lbf's default config does (simplification 0.001 and
    concavities under 1% closed, items inflated, the container outers deflated) still packs."""
    inst = bpp.load_bpp(REF_BALDACCI)
    su = bpp.setup_bpp(oracle_mod.OracleBackend, inst, simplify_tolerance=0.001, narrow_concavity_ratio=0.01)
    log = bpp.run_bpp(oracle_mod.OracleBackend, su, bpp.BppSpec(n_cand=256))
    assert len(log.placements) > 0
    _replay_free(oracle_mod, su, log)
