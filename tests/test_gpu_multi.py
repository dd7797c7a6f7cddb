"""Several layouts in one launch sequence: jcde_multi_detect(_graph) equals per-engine detect."""
import numpy as np
import pytest

import jcde
from jcde import workload as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bins(oracle_mod, jcde_mod):
    """Six small bin layouts from the oracle, replayed into GPU engines."""
    lays = W.multi_layouts(oracle_mod.OracleBackend, seed=0x5C2, n_layouts=6, n_types=8, v_range=(8, 60),
                           items_range=(10, 60))
    engines = []
    for lay, _ in lays:
        eng = jcde.CDEngine(lay.cde_bbox, (), jcde.CDEConfig(quadtree_depth=lay.depth, cd_threshold=lay.cd_threshold))
        for it in lay.items:
            eng.register_item(it.xy, it.poi, it.poles)
        for hz in lay.hazards:
            assert eng.register_hazard(jcde.Hazard(hz.kind, hz.xy, hz.poi, hz.dynamic, hz.tag)) == hz.key
        engines.append(eng)
    q, offs = W.multi_queries(lays, seed=0x5C2, q_range=(1000, 20000))
    return lays, engines, q, offs


def _per_engine(engines, q, offs, filters):
    import torch

    outs = []
    for l, eng in enumerate(engines):
        part = q[offs[l]:offs[l + 1]]
        dq = torch.from_numpy(np.ascontiguousarray(part).view(np.uint8).copy()).cuda()
        outs.append(eng.detect_batch(dq, filter=filters[l] if filters else None).cpu().numpy())
    return np.concatenate(outs)


def test_multi_equals_per_engine_and_oracle(bins):
    import torch

    lays, engines, q, offs = bins
    filters = [[1] if l % 2 else [] for l in range(len(engines))]   # ignore a placed item in odd bins
    ref = _per_engine(engines, q, offs, filters)
    m = jcde.MultiEngine(engines)
    dq = torch.from_numpy(q.view(np.uint8).copy()).cuda()
    got = m.detect(dq, offs, filters=filters).cpu().numpy()
    assert np.array_equal(ref, got)
    # spot check against the oracle
    for l in (0, 3):
        part = q[offs[l]:offs[l + 1]]
        o = lays[l][1].detect_batch(part, ignored=filters[l] or None)
        assert np.array_equal(o, got[offs[l]:offs[l + 1]])


def test_multi_graph_replay_and_recapture(bins):
    import torch

    lays, engines, q, offs = bins
    m = jcde.MultiEngine(engines)
    dq = torch.from_numpy(q.view(np.uint8).copy()).cuda()
    s = torch.cuda.Stream()
    out = torch.empty(len(q), dtype=torch.uint8, device="cuda")
    ref = m.detect(dq, offs).cpu().numpy()
    for _ in range(3):   # capture once, replay
        out.fill_(7)
        m.detect(dq, offs, out=out, stream=s, graph=True)
        s.synchronize()
        assert np.array_equal(out.cpu().numpy(), ref)
    # a mutation of one engine changes its device image: the group re-captures
    hz = next(h for h in lays[2][0].hazards if h.dynamic)
    engines[2].deregister_hazard_by_key(hz.key)
    ref2 = _per_engine(engines, q, offs, None)
    m.detect(dq, offs, out=out, stream=s, graph=True)
    s.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref2)
    engines[2].register_hazard(jcde.Hazard(hz.kind, hz.xy, hz.poi, hz.dynamic, hz.tag))


def test_multi_autotune_keeps_verdicts(bins):
    import torch

    lays, engines, q, offs = bins
    ref = _per_engine(engines, q, offs, None)
    m = jcde.MultiEngine(engines)
    dq = torch.from_numpy(q.view(np.uint8).copy()).cuda()
    choice, ms = m.autotune(dq, offs)
    assert ms > 0 and choice["poly_chunk"] in (1, 2, 4, 8)
    assert np.array_equal(m.detect(dq, offs).cpu().numpy(), ref)
    st = torch.cuda.Stream()   # a captured graph needs a stream other than the legacy default one
    got = m.detect(dq, offs, graph=True, stream=st)
    torch.cuda.synchronize()
    assert np.array_equal(got.cpu().numpy(), ref)
