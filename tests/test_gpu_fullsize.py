"""Full-size correctness of every benchmark workload against the oracle (bit-exact where the
result is a verdict or a key set; within 1e-4 relative of an FP64 evaluation for the proxy's
gradient), at the sizes the benchmark runs.

Layouts are built through the GPU engine (its item preparation and placements are bit-identical
to the oracle's, tested elsewhere) and replayed into oracle engines for the comparison.
"""
import numpy as np
import pytest

import jcde
from jcde import workload as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _cuda(q):
    import torch

    return torch.from_numpy(np.ascontiguousarray(q).view(np.uint8).copy()).cuda()


@pytest.fixture(scope="module")
def star_gpu(jcde_mod, oracle_mod):
    """The star benchmark layout (300 items of 8-200 vertices, holes, zones), with a GPU and an oracle engine."""
    from helpers import gpu_engine

    lay, _ = W.star_container_layout(jcde.GpuBackend)
    return lay, gpu_engine(lay), W.replay(O.OracleBackend, lay)


def test_multi_64_layouts_every_layout_vs_oracle(jcde_mod, oracle_mod):
    """The batched workload: the 64 default layouts (20-400 items of 8-200 vertices, 32-128-vertex containers,
    4,096-262,144 queries each) in one batched launch sequence with graph replay: every verdict equals
    the per-layout launch's, and the first 4,096 queries of every layout equal the oracle's."""
    import torch

    lays = W.multi_layouts(jcde.GpuBackend)
    assert len(lays) == 64
    q, offs = W.multi_queries(lays)
    engines = [e.eng for _, e in lays]
    m = jcde.MultiEngine(engines)
    dq = _cuda(q)
    st = torch.cuda.Stream()
    got = m.detect(dq, offs, graph=True, stream=st)
    st.synchronize()
    got = got.cpu().numpy()
    qb = W.QUERY_DTYPE.itemsize
    for l, (lay, _) in enumerate(lays):
        a, b = int(offs[l]), int(offs[l + 1])
        assert b - a >= 4096
        plain = engines[l].detect_batch(dq[a * qb : b * qb]).cpu().numpy()
        assert np.array_equal(plain, got[a:b]), l
        oeng = W.replay(O.OracleBackend, lay)
        ref = oeng.detect_batch(q[a : a + 4096])
        assert np.array_equal(ref, got[a : a + 4096]), (l, np.flatnonzero(ref != got[a : a + 4096])[:10])


def test_collect_full_configs1_batch(star_gpu):
    """The star benchmark batch in collect mode: all 1,048,576 queries with the zone filter; every count and every
    sorted key list equals the oracle's."""
    lay, geng, oeng = star_gpu
    q = W.queries_for(lay, 1 << 20, 0xC1)
    off, cnt, ids, total = geng.collect_batch(_cuda(q), filter=lay.filter_keys)
    rc, rids = oeng.collect_batch(q, ignored=lay.filter_keys)
    cnt = cnt.cpu().numpy().astype(np.int64)
    assert np.array_equal(cnt, rc.astype(np.int64))
    assert total == len(rids)
    # each query's keys sit at its own offset (segments are placed by atomics, not in query order)
    off = off.cpu().numpy().astype(np.int64)
    start = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    gather = np.repeat(off, cnt) + (np.arange(total) - np.repeat(start, cnt))
    assert np.array_equal(ids.cpu().numpy()[gather].astype(np.uint32), rids)


@pytest.fixture(scope="module")
def big_items(jcde_mod, oracle_mod):
    """Items of 257-600 vertices (above the polygon pass's shared-memory vertex table)."""
    from helpers import gpu_engine

    from jcde import prep

    lay, _ = W.strip_layout(jcde.GpuBackend, seed=0xB16, n_types=6, v_range=(257, 600), r_range=(30.0, 70.0),
                            n_place=30, import_many=prep.import_items)
    assert min(len(it.xy) for it in lay.items) > 256
    return lay, gpu_engine(lay), W.replay(O.OracleBackend, lay)


@pytest.mark.parametrize("n", [4096, 1 << 18])
def test_big_items_detect(big_items, n):
    """Both batch-size regimes (leaf-table kernel and large-batch kernel), both halves and the verdict."""
    from helpers import gpu_detect

    lay, geng, oeng = big_items
    q = W.queries_for(lay, n, 0xB16)
    assert np.array_equal(gpu_detect(geng, q), oeng.detect_batch(q))
    assert np.array_equal(gpu_detect(geng, q, mode="poly"), oeng.detect_batch(q, mode=2))
    ign = [lay.hazards[3].key]
    assert np.array_equal(gpu_detect(geng, q, filter=ign), oeng.detect_batch(q, ignored=ign))


def test_big_items_collect_and_touch(big_items):
    from helpers import csr_lists, gpu_collect, gpu_detect

    lay, geng, oeng = big_items
    q = W.queries_for(lay, 32768, 0xB17)
    rc, rids = oeng.collect_batch(q)
    assert gpu_collect(geng, q) == csr_lists(rc, rids)
    t = W.touch_queries(lay, 1 << 16, 0xB18)
    assert np.array_equal(gpu_detect(geng, t), oeng.detect_batch(t))


def _proxy_candidates(eng, lay, n_target, filt):
    """The gradient-separation workload's candidate pool: uniform placements that collide (exact verdict) and overlap
    some hazard pole."""
    import torch

    st = W.Stream(0xC4, 1)
    got_p, got_i, have = [], [], 0
    while have < n_target:
        params, items = W.random_params(st, 1 << 21, len(lay.items), lay.cde_bbox)
        dp = torch.from_numpy(params).cuda()
        di = torch.from_numpy(items.astype(np.int32)).cuda()
        q0, p0 = eng.separate_batch(dp.clone(), di, steps=0, filter=filt)
        v0 = eng.detect_batch(q0, filter=filt)
        keep = (v0 == 1) & (p0 > 0)
        got_p.append(dp[keep])
        got_i.append(di[keep])
        have += int(keep.sum().item())
    return torch.cat(got_p)[:n_target].contiguous(), torch.cat(got_i)[:n_target].contiguous()


def test_proxy_gradient_every_configs4_candidate(star_gpu):
    """The gradient-separation workload: 1,048,576 colliding candidates on the star layout; the proxy and its
    gradient d/d(theta, tx, ty) from the GPU against an FP64 evaluation of the same float32 inputs:
    every candidate's gradient within 1e-4 relative (norm-wise), every value within 1e-5."""
    lay, geng, _ = star_gpu
    hp = W.hazard_poles(jcde.GpuBackend, lay)
    keys = hp[:, 3].view(np.uint32)
    for k in np.unique(keys):
        geng.set_hazard_poles(int(k), hp[keys == k, :3])
    P, I = _proxy_candidates(geng, lay, 1 << 20, lay.filter_keys)
    val, grad = geng.proxy_batch(P, I, filter=lay.filter_keys)
    v32, g32 = val.cpu().numpy().astype(np.float64), grad.cpu().numpy().astype(np.float64)
    v64, g64 = O.proxy_f64(P.cpu().numpy(), I.cpu().numpy().astype(np.uint32), [it.poles for it in lay.items], hp,
                           ignored=lay.filter_keys)
    assert np.array_equal(v64 > 0, v32 > 0), int(((v64 > 0) != (v32 > 0)).sum())
    n64 = np.linalg.norm(g64, axis=1)
    on = n64 > 0
    rel_g = np.linalg.norm(g32[on] - g64[on], axis=1) / n64[on]
    assert rel_g.max() <= 1e-4, (rel_g.max(), np.percentile(rel_g, 99.99), int((rel_g > 1e-4).sum()))
    assert np.abs(g32[~on]).max(initial=0.0) <= 1e-6
    rel_v = np.abs(v32 - v64) / np.maximum(v64, 1e-30)
    assert rel_v[v64 > 0].max() <= 1e-5, rel_v.max()


@pytest.mark.parametrize("n", [(1 << 18) + 7, 1 << 20])
def test_host_entry_point_equals_device_path_and_oracle(star_gpu, n):
    """jcde_detect_batch_host (host buffers: copy in, the passes, copy out) at the benchmark's size
    gives the device path's verdicts, with and without a filter, and the oracle's on samples."""
    from helpers import gpu_detect

    lay, geng, oeng = star_gpu
    q = W.queries_for(lay, n, 0xC1, sid=91)
    for filt in (None, lay.filter_keys):
        host = geng.detect_batch(q, filter=filt)
        assert np.array_equal(host, gpu_detect(geng, q, filter=filt)), filt
        assert np.array_equal(host[:8192], oeng.detect_batch(q[:8192], ignored=filt)), filt
        assert np.array_equal(host[-4096:], oeng.detect_batch(q[-4096:], ignored=filt)), filt
