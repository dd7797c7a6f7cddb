"""The CUDA path against the committed golden fixtures (tests/golden/golden.npz): the same outputs
bit for bit, with no oracle involved at run time."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden as G  # noqa: E402

from jcde import bpp, lbf  # noqa: E402
from jcde import workload as W  # noqa: E402

gpu = pytest.mark.gpu


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(os.path.join(HERE, "golden", "golden.npz")))


@gpu
def test_strip_layout_gpu(jcde_mod, golden):
    import torch

    import jcde

    lay, eng = W.strip_layout(jcde.GpuBackend)
    pl = [h.placement for h in lay.hazards if h.placement is not None]
    got = np.array([[p[0], *[np.float32(x).view(np.uint32) for x in p[1:]]] for p in pl], dtype=np.uint32)
    assert np.array_equal(got, golden["strip_placements"])
    q = W.queries_for(lay, G.N_QUERIES, 0xC0)
    dq = torch.from_numpy(q.view(np.uint8).copy()).cuda()
    assert np.array_equal(np.packbits(eng.eng.detect_batch(dq).cpu().numpy()), golden["strip_verdicts"])
    off, cnt, ids, _ = eng.eng.collect_batch(dq[: G.N_COLLECT * W.QUERY_DTYPE.itemsize])
    off, cnt, ids = off.cpu().numpy(), cnt.cpu().numpy(), ids.cpu().numpy()
    assert np.array_equal(cnt.astype(np.uint32), golden["strip_collect_counts"])
    flat = np.concatenate([ids[o: o + c] for o, c in zip(off, cnt)]) if len(off) else np.zeros(0, np.int32)
    assert np.array_equal(flat.astype(np.uint32), golden["strip_collect_ids"])
    assert G.tree_hash(eng.tree_dump()) == bytes(golden["strip_tree_sha256"]).hex()


@gpu
def test_preparation_gpu(jcde_mod, golden):
    from jcde import prep

    shapes = G.prep_shapes()
    items = prep.import_items(shapes)
    for i, it in enumerate(items):
        assert np.array_equal(it.poi.view(np.uint32), golden[f"prep{i}_poi"].view(np.uint32))
        assert np.array_equal(it.poles.view(np.uint32), golden[f"prep{i}_poles"].view(np.uint32))
    base = [prep.spolygon_shape(r) for r in shapes]
    for tol in G.SIMPLIFY_TOLS:
        for deflate in (0, 1):
            got = prep.simplify_batch([b[0] for b in base], [b[2] for b in base], bool(deflate), tol)
            for i, g in enumerate(got):
                assert np.array_equal(g.view(np.uint32), golden[f"simp{i}_{tol}_{deflate}"].view(np.uint32))


@gpu
def test_builds_gpu(jcde_mod, golden):
    import jcde

    spec = G.lbf_spec()
    _, geng = lbf.setup(jcde.GpuBackend, spec)
    log, _ = lbf.run_device(geng, spec, steps_per_graph=10)
    assert np.array_equal(log.placements, golden["lbf_placements"])
    assert np.array_equal(log.removals, golden["lbf_removals"])
    assert np.array_equal(log.free_counts, golden["lbf_free_counts"])
    inst, bspec = G.bpp_case()
    blog = bpp.run_bpp(jcde.GpuBackend, bpp.setup_bpp(jcde.GpuBackend, inst), bspec)
    assert np.array_equal(blog.placements, golden["bpp_placements"])
    assert blog.layouts == golden["bpp_layouts"].tolist()
