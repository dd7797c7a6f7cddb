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


def _check_two_calls(eng, L, dq, n, filters, stream):
    """jcde_detect_batch_noalloc equals jcde_detect_batch on each filter, called in a row; device
    memory does not move across any call."""
    import torch

    from jcde import _ffi

    ref = torch.empty(n, dtype=torch.uint8, device="cuda")
    got = torch.empty(n, dtype=torch.uint8, device="cuda")
    for i, keys in enumerate(filters):
        f, keep = _filter(keys)
        assert L.jcde_detect_batch(eng.h, dq.data_ptr(), n, C.byref(f), ref.data_ptr(), stream) == _ffi.OK
        torch.cuda.synchronize()
        got.fill_(0xAB)
        free_before = torch.cuda.mem_get_info()[0]
        assert L.jcde_detect_batch_noalloc(eng.h, dq.data_ptr(), n, C.byref(f), got.data_ptr(), stream) == _ffi.OK
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        assert torch.equal(ref, got), f"n={n} call {i}: {int((ref != got).sum())} verdicts differ"
        assert free_after >= free_before, (n, i, free_before, free_after)


@pytest.mark.parametrize("n", [256, 1 << 17, (1 << 18) + 5])
def test_noalloc_equals_detect_batch_two_calls(star_layout, jcde_mod, n):
    """Small batches (leaf-table polygon pass), the largest of those, and a large batch
    (counter-fed large-batch passes)."""
    import torch

    from jcde import workload as W

    lay, _ = star_layout
    eng = _engine(lay)
    L = jcde_mod.lib()
    q = W.queries_for(lay, n, 0xC1, sid=77)
    dq = torch.from_numpy(q.view(np.uint8).copy()).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    placed = [hz.key for hz in lay.hazards if hz.dynamic][:25]
    # second call: a different, larger filter (the array keeps the first call's mask)
    _check_two_calls(eng, L, dq, n, [lay.filter_keys, placed + lay.filter_keys], stream)
    # the two filters give different answers somewhere, so the second call did not reuse the first's
    if n >= 1 << 17:
        f0, k0 = _filter(lay.filter_keys)
        f1, k1 = _filter(placed + lay.filter_keys)
        a = torch.empty(n, dtype=torch.uint8, device="cuda")
        b = torch.empty(n, dtype=torch.uint8, device="cuda")
        L.jcde_detect_batch_noalloc(eng.h, dq.data_ptr(), n, C.byref(f0), a.data_ptr(), stream)
        L.jcde_detect_batch_noalloc(eng.h, dq.data_ptr(), n, C.byref(f1), b.data_ptr(), stream)
        torch.cuda.synchronize()
        assert not torch.equal(a, b)


def test_noalloc_state_and_large_filters(strip_layout, jcde_mod):
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
    # a filter of 300,000 keys (most beyond the engine's slots): the key list is turned into the
    # bitmask on the host, so its length costs no device memory
    _check_two_calls(eng, L, dq, len(q), [np.arange(300_000) % 41, [3, 5, 7]], stream)
    # the caller's key buffer may be reused as soon as the call returns
    keys = np.ascontiguousarray(np.array([1, 2, 3], np.uint32))
    fk = _ffi.jcde_filter()
    fk.ignored = keys.ctypes.data_as(C.POINTER(C.c_uint32))
    fk.n_ignored = 3
    a = torch.empty_like(out)
    assert L.jcde_detect_batch_noalloc(eng.h, dq.data_ptr(), len(q), C.byref(fk), a.data_ptr(), stream) == _ffi.OK
    keys[:] = [4, 5, 6]
    torch.cuda.synchronize()
    f123, k123 = _filter([1, 2, 3])
    ref = torch.empty_like(out)
    assert L.jcde_detect_batch(eng.h, dq.data_ptr(), len(q), C.byref(f123), ref.data_ptr(), stream) == _ffi.OK
    torch.cuda.synchronize()
    assert torch.equal(a, ref)
