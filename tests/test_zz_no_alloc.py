"""jcde_detect_batch_noalloc: filtered detect that allocates no device memory.

Some callers cannot let a query allocate: a service whose GPU memory is all owned by its own pool
has none to give, and a caller running queries next to other work cannot take cudaMalloc's
device-wide synchronization.  The regular filtered entry point allocates a bitmask and a per-node
table the first time it meets a filter; this one keeps them in a static device array instead.

Checked here through the C ABI, against the regular entry point, on two calls in a row with
different filters (the array keeps the previous call's contents, so the second call also shows that
the first call's state is cleared).  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _engine(lay):
    import jcde

    eng = jcde.CDEngine(lay.cde_bbox, (), jcde.CDEConfig(quadtree_depth=lay.depth, cd_threshold=lay.cd_threshold))
    for it in lay.items:
        eng.register_item(it.xy, it.poi, it.poles)
    for hz in lay.hazards:
        eng.register_hazard(jcde.Hazard(hz.kind, hz.xy, hz.poi, hz.dynamic, hz.tag))
    return eng


def _filter(keys):
    from jcde import _ffi

    arr = np.ascontiguousarray(np.asarray(keys, dtype=np.uint32))
    f = _ffi.jcde_filter()
    f.ignored = arr.ctypes.data_as(C.POINTER(C.c_uint32))
    f.n_ignored = len(arr)
    return f, arr


def test_noalloc_equals_detect_batch_two_calls(star_layout, jcde_mod):
    import torch

    from jcde import _ffi
    from jcde import workload as W

    lay, _ = star_layout
    eng = _engine(lay)
    L = jcde_mod.lib()
    q = W.queries_for(lay, 1 << 17, 0xC1, sid=77)
    dq = torch.from_numpy(q.view(np.uint8).copy()).cuda()
    n = len(q)
    stream = torch.cuda.current_stream().cuda_stream
    placed = [hz.key for hz in lay.hazards if hz.dynamic][:25]
    filters = [lay.filter_keys, placed + lay.filter_keys]   # second call: a different, larger filter
    ref = torch.empty(n, dtype=torch.uint8, device="cuda")
    got = torch.empty(n, dtype=torch.uint8, device="cuda")
    for i, keys in enumerate(filters):
        f, keep = _filter(keys)
        assert L.jcde_detect_batch(eng.h, dq.data_ptr(), n, C.byref(f), ref.data_ptr(), stream) == _ffi.OK
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        got.fill_(0xAB)
        assert L.jcde_detect_batch_noalloc(eng.h, dq.data_ptr(), n, C.byref(f), got.data_ptr(), stream) == _ffi.OK
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        assert torch.equal(ref, got), f"call {i}: {int((ref != got).sum())} verdicts differ"
        if i == 1:   # the first call may load the new kernels' code; the second must not move memory
            assert free_after >= free_before, (free_before, free_after)
    # the two filters give different answers somewhere, so the second call did not reuse the first's
    f0, k0 = _filter(filters[0])
    f1, k1 = _filter(filters[1])
    a = torch.empty_like(got)
    b = torch.empty_like(got)
    L.jcde_detect_batch_noalloc(eng.h, dq.data_ptr(), n, C.byref(f0), a.data_ptr(), stream)
    L.jcde_detect_batch_noalloc(eng.h, dq.data_ptr(), n, C.byref(f1), b.data_ptr(), stream)
    torch.cuda.synchronize()
    assert not torch.equal(a, b)


def test_noalloc_refuses_what_it_cannot_do_without_allocating(strip_layout, jcde_mod):
    import torch

    from jcde import _ffi
    from jcde import workload as W

    lay, _ = strip_layout
    eng = _engine(lay)
    L = jcde_mod.lib()
    q = W.queries_for(lay, 1024, 0xC0, sid=78)
    dq = torch.from_numpy(q.view(np.uint8).copy()).cuda()
    out = torch.empty(len(q), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    f, keep = _filter([1, 2])
    # the device copy of a freshly built engine is not current yet
    assert L.jcde_detect_batch_noalloc(eng.h, dq.data_ptr(), len(q), C.byref(f), out.data_ptr(), stream) == _ffi.ERR_STATE
    assert L.jcde_detect_batch(eng.h, dq.data_ptr(), 0, None, out.data_ptr(), stream) == _ffi.OK
    assert L.jcde_detect_batch_noalloc(eng.h, dq.data_ptr(), len(q), C.byref(f), out.data_ptr(), stream) == _ffi.OK
    # more ignored keys than the static array holds
    big, keep2 = _filter(np.arange(300_000) % 41)
    assert L.jcde_detect_batch_noalloc(eng.h, dq.data_ptr(), len(q), C.byref(big), out.data_ptr(), stream) == _ffi.ERR_CAPACITY
    torch.cuda.synchronize()
