"""Pole-overlap proxy: FP64 oracle checks (CPU) and the GPU forward/adjoint against it (GPU)."""
import numpy as np
import pytest

from jcde import workload as W


@pytest.fixture(scope="module")
def strip_poles(oracle_mod, strip_layout):
    lay, _ = strip_layout
    return W.hazard_poles(oracle_mod.OracleBackend, lay)


def test_f64_gradient_matches_central_differences(oracle_mod, strip_layout, strip_poles):
    """The analytic adjoint of the FP64 oracle against central finite differences, h = 1e-3."""
    lay, _ = strip_layout
    st = W.Stream(0xF4, 1)
    params, items = W.random_params(st, 4000, len(lay.items), lay.cde_bbox)
    polesets = [it.poles for it in lay.items]
    val, grad = oracle_mod.proxy_f64(params, items, polesets, strip_poles)
    sel = np.flatnonzero(val > 1.0)[:300]
    assert len(sel) > 50
    h = 1e-3
    fd = np.zeros((len(sel), 3))
    base = params[sel].astype(np.float64)
    for k in range(3):
        pp, pm = base.copy(), base.copy()
        pp[:, k] += h
        pm[:, k] -= h
        vp, _ = oracle_mod.proxy_f64(pp, items[sel], polesets, strip_poles)
        vm, _ = oracle_mod.proxy_f64(pm, items[sel], polesets, strip_poles)
        fd[:, k] = (vp - vm) / (2 * h)
    g = grad[sel]
    rel = np.abs(fd - g).max(axis=1) / np.maximum(np.abs(g).max(axis=1), 1e-9)
    assert np.median(rel) < 1e-3 and np.percentile(rel, 90) < 1e-2, (np.median(rel), np.percentile(rel, 90))


@pytest.mark.gpu
def test_gpu_proxy_matches_f64(oracle_mod, jcde_mod, strip_layout, strip_poles):
    import torch

    from helpers import gpu_engine

    lay, _ = strip_layout
    eng = gpu_engine(lay)
    for hz in lay.hazards:
        sel = strip_poles[:, 3].view(np.uint32) == hz.key
        if sel.any():
            eng.set_hazard_poles(hz.key, strip_poles[sel, :3])
    st = W.Stream(0xF4, 2)
    params, items = W.random_params(st, 20000, len(lay.items), lay.cde_bbox)
    val, grad = eng.proxy_batch(torch.from_numpy(params).cuda(), torch.from_numpy(items.astype(np.int32)).cuda())
    val, grad = val.cpu().numpy().astype(np.float64), grad.cpu().numpy().astype(np.float64)
    v64, g64 = oracle_mod.proxy_f64(params, items, [it.poles for it in lay.items], strip_poles)
    on = v64 > 1e-2
    assert on.sum() > 1000
    assert np.array_equal(val > 0, v64 > 0) or ((val > 0) != (v64 > 0)).sum() < 5
    rel_v = np.abs(val[on] - v64[on]) / v64[on]
    rel_g = np.linalg.norm(grad[on] - g64[on], axis=1) / np.linalg.norm(g64[on], axis=1)
    # float-float contact pairs: every candidate within 1e-4 (typically ~1e-8)
    assert rel_v.max() < 1e-5 and rel_g.max() < 1e-4, (rel_v.max(), rel_g.max())


@pytest.mark.gpu
def test_gpu_separation_then_exact_verdict(oracle_mod, jcde_mod, strip_layout, strip_poles):
    """Descent moves colliding candidates; every final placement's verdict is the oracle's."""
    import torch

    from helpers import gpu_engine

    lay, oeng = strip_layout
    eng = gpu_engine(lay)
    for hz in lay.hazards:
        sel = strip_poles[:, 3].view(np.uint32) == hz.key
        if sel.any():
            eng.set_hazard_poles(hz.key, strip_poles[sel, :3])
    st = W.Stream(0xF4, 3)
    params, items = W.random_params(st, 8192, len(lay.items), lay.cde_bbox)
    dp = torch.from_numpy(params).cuda()
    di = torch.from_numpy(items.astype(np.int32)).cuda()
    q0, p0 = eng.separate_batch(dp.clone(), di, steps=0)
    v0 = eng.detect_batch(q0).cpu().numpy()
    q1, p1 = eng.separate_batch(dp, di, steps=20)
    v1 = eng.detect_batch(q1).cpu().numpy()
    host_q = q1.cpu().numpy().view(W.QUERY_DTYPE)
    assert np.array_equal(v1, oeng.detect_batch(host_q))
    p0, p1 = p0.cpu().numpy(), p1.cpu().numpy()
    moved = p0 > 0
    assert (p1[moved] <= p0[moved] + 1e-3).mean() > 0.95   # descent lowers the proxy
    assert v1[moved].mean() < v0[moved].mean()             # and frees some placements


@pytest.mark.gpu
def test_gpu_proxy_forward_backward_pair_and_autograd(oracle_mod, jcde_mod, strip_layout, strip_poles):
    """The forward/backward pair equals the fused call bit for bit, and drives torch autograd."""
    import torch

    import jcde
    from helpers import gpu_engine

    lay, _ = strip_layout
    eng = gpu_engine(lay)
    for hz in lay.hazards:
        sel = strip_poles[:, 3].view(np.uint32) == hz.key
        if sel.any():
            eng.set_hazard_poles(hz.key, strip_poles[sel, :3])
    st = W.Stream(0xF4, 4)
    params, items = W.random_params(st, 4096, len(lay.items), lay.cde_bbox)
    dp = torch.from_numpy(params).cuda()
    di = torch.from_numpy(items.astype(np.int32)).cuda()
    val, grad = eng.proxy_batch(dp, di)
    assert torch.equal(eng.proxy_forward(dp, di), val)
    assert torch.equal(eng.proxy_backward(dp, di), grad)
    w = torch.from_numpy(W.Stream(0xF4, 5).f32(4096)).cuda()
    x = dp.clone().requires_grad_(True)
    p = jcde.pole_overlap(eng, x, di)
    assert torch.equal(p.detach(), val)
    (w * p).sum().backward()
    assert torch.equal(x.grad, w[:, None] * grad)   # the same float32 products
