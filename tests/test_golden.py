"""The committed golden fixtures (tests/golden/golden.npz, written by tests/golden/make_golden.py
from the oracle): the oracle still reproduces every one of them bit for bit (a regression pin of
the oracle; the GPU side of the same fixtures is tests/test_gpu_golden.py)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden as G  # noqa: E402

from jcde import bpp, lbf  # noqa: E402
from jcde import workload as W  # noqa: E402


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(os.path.join(HERE, "golden", "golden.npz")))


def test_strip_layout(oracle_mod, golden):
    B = oracle_mod.OracleBackend
    lay, eng = W.strip_layout(B)
    pl = [h.placement for h in lay.hazards if h.placement is not None]
    got = np.array([[p[0], *[np.float32(x).view(np.uint32) for x in p[1:]]] for p in pl], dtype=np.uint32)
    assert np.array_equal(got, golden["strip_placements"])
    q = W.queries_for(lay, G.N_QUERIES, 0xC0)
    assert np.array_equal(np.packbits(eng.detect_batch(q)), golden["strip_verdicts"])
    counts, ids = eng.collect_batch(q[: G.N_COLLECT])
    assert np.array_equal(counts.astype(np.uint32), golden["strip_collect_counts"])
    assert np.array_equal(ids.astype(np.uint32), golden["strip_collect_ids"])
    assert G.tree_hash(eng.tree_dump()) == bytes(golden["strip_tree_sha256"]).hex()


def test_preparation(oracle_mod, golden):
    B = oracle_mod.OracleBackend
    for i, raw in enumerate(G.prep_shapes()):
        it = W.import_item(B, raw)
        assert np.array_equal(it.poi.view(np.uint32), golden[f"prep{i}_poi"].view(np.uint32))
        assert np.array_equal(it.poles.view(np.uint32), golden[f"prep{i}_poles"].view(np.uint32))
        xy, _, area, _, _ = B.spolygon_new(raw)
        for tol in G.SIMPLIFY_TOLS:
            for deflate in (0, 1):
                s = B.simplify_shape(xy, area, bool(deflate), tol)
                assert np.array_equal(s.view(np.uint32), golden[f"simp{i}_{tol}_{deflate}"].view(np.uint32))


def test_builds(oracle_mod, golden):
    B = oracle_mod.OracleBackend
    spec = G.lbf_spec()
    lay, eng = lbf.setup(B, spec)
    log = lbf.run_host(lay, eng, spec)
    assert np.array_equal(log.placements, golden["lbf_placements"])
    assert np.array_equal(log.removals, golden["lbf_removals"])
    assert np.array_equal(log.free_counts, golden["lbf_free_counts"])
    inst, bspec = G.bpp_case()
    blog = bpp.run_bpp(B, bpp.setup_bpp(B, inst), bspec)
    assert np.array_equal(blog.placements, golden["bpp_placements"])
    assert blog.layouts == golden["bpp_layouts"].tolist()
