"""Bin packing on the GPU engines (jcde.bpp): the same layouts, placements and skipped items as the
oracle run, with every search's layouts evaluated in one multi-layout launch sequence or one by one."""
import numpy as np
import pytest

from jcde import bpp

gpu = pytest.mark.gpu


@gpu
@pytest.mark.parametrize("ls", [0, 2])
def test_bpp_matches_oracle(oracle_mod, jcde_mod, ls):
    import jcde

    inst = bpp.load_bpp(bpp.synthetic_instance(n_types=16, n_bins=4))
    spec = bpp.BppSpec(n_cand=2048, ls_rounds=ls, ls_cand=512 if ls else 0)
    ref = bpp.run_bpp(oracle_mod.OracleBackend, bpp.setup_bpp(oracle_mod.OracleBackend, inst), spec)
    su = bpp.setup_bpp(jcde.GpuBackend, inst)
    got = bpp.run_bpp(jcde.GpuBackend, su, spec, batched=True)
    assert got.same_as(ref), (len(got.placements), len(ref.placements), got.layouts, ref.layouts)
    seq = bpp.run_bpp(jcde.GpuBackend, bpp.setup_bpp(jcde.GpuBackend, inst), spec, batched=False)
    assert seq.same_as(ref)
    assert np.isclose(bpp.export_solution(su, got)["density"], bpp.export_solution(su, ref)["density"])


@gpu
def test_device_candidates_equal_host_round(jcde_mod):
    """jcde_gen_candidates draws the host round's candidates bit for bit (continuous rotation and
    allowed orientations)."""
    import torch

    from jcde import instance as I
    from jcde import workload as W
    from jcde._ffi import check, jcde_rect, lib

    spec = bpp.BppSpec(n_cand=3000)
    box = np.array([-5.0, 2.0, 612.5, 480.0], np.float32)
    for orient in (None, I.orientation_cs([0.0, 90.0, 180.0, 270.0])):
        q, u = bpp._round(spec, 7, 2049, 3, box, orient)
        dq = torch.empty(len(q) * W.QUERY_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        du = torch.empty(len(q), dtype=torch.float64, device="cuda")
        do = None if orient is None else torch.from_numpy(np.ascontiguousarray(orient)).cuda()
        check(lib().jcde_gen_candidates(spec.seed, bpp.BPP_SID_BASE + 4096 * 7 + 2049, len(q), 3,
                                        jcde_rect(*[float(v) for v in box]), None if do is None else do.data_ptr(),
                                        0 if do is None else len(do), dq.data_ptr(), du.data_ptr(), None), "gen")
        torch.cuda.synchronize()
        got = dq.cpu().numpy().view(W.QUERY_DTYPE)
        assert np.array_equal(got.view(np.uint8), q.view(np.uint8))
        assert np.array_equal(du.cpu().numpy(), u)


@gpu
def test_device_prep_setup_equals_host(oracle_mod, jcde_mod):
    """setup_bpp with the items prepared on the device gives the host preparation's items."""
    import jcde

    inst = bpp.load_bpp(bpp.synthetic_instance(n_types=10, n_bins=2))
    a = bpp.setup_bpp(oracle_mod.OracleBackend, inst, simplify_tolerance=0.001)
    b = bpp.setup_bpp(jcde.GpuBackend, inst, simplify_tolerance=0.001, device_prep=True)
    for x, y in zip(a.items, b.items):
        assert np.array_equal(x.xy, y.xy) and np.array_equal(x.poles, y.poles) and np.array_equal(x.poi, y.poi)
    assert a.order == b.order


@gpu
def test_segmented_generator_and_choice(jcde_mod):
    """jcde_gen_candidates_segments draws each segment's host round; jcde_lbf_select_segments makes
    each segment's LBF choice as the host does."""
    import ctypes as C

    import torch

    import jcde
    from jcde import lbf
    from jcde import workload as W
    from jcde._ffi import check, jcde_rect, lib

    inst = bpp.load_bpp(bpp.synthetic_instance(n_types=4, n_bins=3))
    su = bpp.setup_bpp(jcde.GpuBackend, inst)
    eng, _ = bpp._bin_engine(jcde.GpuBackend, su, 1)
    spec = bpp.BppSpec(n_cand=1500)
    slots, boxes = [5, 2049, 2050], [su.bins[0].box, su.bins[1].box, su.bins[2].box]
    n = spec.n_cand
    dq = torch.empty(3 * n * W.QUERY_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    du = torch.empty(3 * n, dtype=torch.float64, device="cuda")
    sids = (C.c_uint64 * 3)(*[bpp.BPP_SID_BASE + 4096 * 11 + s for s in slots])
    rects = (jcde_rect * 3)(*[jcde_rect(*[float(x) for x in b]) for b in boxes])
    check(lib().jcde_gen_candidates_segments(spec.seed, sids, rects, 3, n, 2, None, 0, dq.data_ptr(), du.data_ptr(),
                                             None), "gen")
    torch.cuda.synchronize()
    got = dq.cpu().numpy().view(W.QUERY_DTYPE)
    hosts = [bpp._round(spec, 11, s, 2, b, None) for s, b in zip(slots, boxes)]
    for k, (q, u) in enumerate(hosts):
        assert np.array_equal(got[k * n: (k + 1) * n].view(np.uint8), q.view(np.uint8))
        assert np.array_equal(du.cpu().numpy()[k * n: (k + 1) * n], u)
    v = np.concatenate([eng.detect_batch(q) for q, _ in hosts])
    dv = torch.from_numpy(v).cuda()
    best = torch.empty(3, dtype=torch.int64, device="cuda")
    check(lib().jcde_lbf_select_segments(eng.eng.h, dq.data_ptr(), dv.data_ptr(), n, 3, best.data_ptr(), None), "sel")
    b = best.cpu().numpy().view(np.uint64)
    for k, (q, _) in enumerate(hosts):
        ref = lbf.select_host(su.items, q, v[k * n: (k + 1) * n])
        assert (b[k] == np.uint64(0xFFFFFFFFFFFFFFFF)) if ref < 0 else int(b[k] & np.uint64(0xFFFFFFFF)) == ref
