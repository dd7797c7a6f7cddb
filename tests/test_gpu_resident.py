"""Device-resident engine and the on-device LBF-style build against the oracle.

* the resident tree (register / deregister run on the GPU) has the oracle's canonical tree dump —
  node boxes, presences, ff boxes and clipped edge sets bit for bit — after a copy, after placements
  and after removals, and answers detect queries like the oracle;
* the LBF-style build run on the GPU (generation, verdicts, choice, registration and removal without
  a host round trip) logs the same placements, removals and free-candidate counts as the same build
  driven step by step through the oracle, and ends with the oracle's tree.
"""
import numpy as np
import pytest

import jcde
from jcde import lbf
from jcde import workload as W

pytestmark = pytest.mark.gpu


def tq(q):
    import torch

    return torch.from_numpy(np.ascontiguousarray(q, dtype=W.QUERY_DTYPE).view(np.uint8).copy()).cuda()


def resident_detect(r, q):
    import torch

    out = r.detect_batch(tq(q))
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_resident_copy_updates_and_queries(star_layout, oracle_mod, jcde_mod):
    import torch

    lay, _ = star_layout
    oeng = W.replay(oracle_mod.OracleBackend, lay)
    geng = W.replay(jcde.GpuBackend, lay)
    r = jcde.ResidentEngine(geng.eng)
    assert np.array_equal(r.tree_dump(), oeng.tree_dump())
    st = r.status()
    assert st["error"] == 0 and st["n_live"] == len(lay.hazards)

    # placements found free by the oracle, registered on both sides
    q = W.make_queries(W.Stream(0x51, 1), 4096, len(lay.items), lay.cde_bbox)
    free = np.flatnonzero(oeng.detect_batch(q) == 0)[:40]
    assert len(free) >= 20
    key_dev = torch.zeros(1, dtype=torch.int32, device="cuda")
    placed = []
    for i in free:
        hz = W.placed_hazard(lay.items[int(q["item"][i])], int(q["item"][i]), q["cos"][i], q["sin"][i], q["tx"][i],
                             q["ty"][i])
        k = oeng.register_hazard(hz.kind, hz.dynamic, hz.xy, hz.poi, 0)
        r.register_placed(tq(q[i : i + 1]), key_dev)
        assert int(key_dev.item()) == k
        placed.append(k)
    assert np.array_equal(r.tree_dump(), oeng.tree_dump())

    # removals (placed items and a static hazard), then placements that reuse the freed keys
    rng = np.random.default_rng(5)
    gone = list(rng.choice(placed, 12, replace=False)) + [int(lay.hazards[3].key)]
    for k in gone:
        oeng.deregister_hazard(int(k))
        key_dev.fill_(int(k))
        r.deregister(key_dev)
    assert np.array_equal(r.tree_dump(), oeng.tree_dump())
    for i in free[:5]:
        hz = W.placed_hazard(lay.items[int(q["item"][i])], int(q["item"][i]), q["cos"][i], q["sin"][i], q["tx"][i],
                             q["ty"][i])
        k = oeng.register_hazard(hz.kind, hz.dynamic, hz.xy, hz.poi, 0)
        r.register_placed(tq(q[i : i + 1]), key_dev)
        assert int(key_dev.item()) == k
    assert np.array_equal(r.tree_dump(), oeng.tree_dump())

    # an unknown key is counted and ignored
    key_dev.fill_(10_000_000)
    r.deregister(key_dev)
    st = r.status()
    assert st["error"] == 0 and st["not_found"] == 1
    assert np.array_equal(r.tree_dump(), oeng.tree_dump())

    qq = W.make_queries(W.Stream(0x52, 1), 1 << 16, len(lay.items), lay.cde_bbox)
    assert np.array_equal(resident_detect(r, qq), oeng.detect_batch(qq))


def _lbf_pair(oracle_mod, spec, keep_verdicts=0, steps_per_graph=0):
    lay_o, oeng = lbf.setup(oracle_mod.OracleBackend, spec)
    ref = lbf.run_host(lay_o, oeng, spec, keep_verdicts=keep_verdicts)
    lay_g, geng = lbf.setup(jcde.GpuBackend, spec)
    got, r = lbf.run_device(geng, spec, steps_per_graph=steps_per_graph, keep_verdicts=keep_verdicts)
    return ref, oeng, got, r


def test_lbf_device_matches_oracle(oracle_mod, jcde_mod):
    spec = lbf.LbfSpec(steps=300, n_cand=4096, remove_every=25)
    ref, oeng, got, r = _lbf_pair(oracle_mod, spec, keep_verdicts=12)
    assert len(ref.placements) > 250 and len(ref.removals) == 12
    assert np.array_equal(got.free_counts, ref.free_counts)
    assert np.array_equal(got.placements, ref.placements)
    assert np.array_equal(got.removals, ref.removals)
    for a, b in zip(got.verdicts, ref.verdicts):
        assert np.array_equal(a, b)
    assert r.status()["error"] == 0
    assert np.array_equal(r.tree_dump(), oeng.tree_dump())


def test_lbf_graph_replay_matches_eager(oracle_mod, jcde_mod):
    spec = lbf.LbfSpec(steps=120, n_cand=2048, remove_every=10)
    _, geng = lbf.setup(jcde.GpuBackend, spec)
    eager, r1 = lbf.run_device(geng, spec)
    _, geng2 = lbf.setup(jcde.GpuBackend, spec)
    graphed, r2 = lbf.run_device(geng2, spec, steps_per_graph=16)   # 7 graph launches + 8 eager steps
    assert eager.same_as(graphed)
    assert np.array_equal(r1.tree_dump(), r2.tree_dump())
    assert r2.reset() > 0   # back to the engine's hazards: the same build again
    again, _ = lbf.run_device(geng2, spec, steps_per_graph=16, resident=r2)
    assert again.same_as(eager)


def test_lbf_full_size_matches_oracle(oracle_mod, jcde_mod):
    """2000 steps x 16384 candidates, a removal every 50 steps: the same final layout as the oracle."""
    spec = lbf.LbfSpec()
    ref, oeng, got, r = _lbf_pair(oracle_mod, spec, steps_per_graph=25)
    assert len(ref.removals) == 40
    assert got.same_as(ref)
    assert r.status()["error"] == 0
    assert np.array_equal(r.tree_dump(), oeng.tree_dump())


def test_lbf_search_with_box_tightening_and_normal_local_search_matches_oracle(oracle_mod, jcde_mod):
    """lbf's search restated in rounds: 4 uniform rounds, each over the box tightened to the best
    cost so far / 10 (search.rs:62-63, loss.rs:34-44), then 3 local-search rounds with Normal offsets
    on LSSampler's decaying deviations (ls_sampler.rs): the device build equals the oracle-driven
    one (placements, removals, per-step counts, final tree), eagerly and from a CUDA graph."""
    spec = lbf.LbfSpec(steps=240, n_cand=4096, remove_every=40, uniform_rounds=4, ls_rounds=3, ls_cand=1024)
    ref, oeng, got, r = _lbf_pair(oracle_mod, spec, steps_per_graph=16)
    assert len(ref.placements) >= 200
    assert got.same_as(ref)
    assert r.status()["error"] == 0
    assert np.array_equal(r.tree_dump(), oeng.tree_dump())
    # the later rounds did choose (their round index is in the placement log)
    rounds = ref.placements[:, 2] >> 24
    assert (rounds >= 1).sum() > 20 and (rounds >= 4).sum() > 20


def test_resident_capacity_error_is_sticky_and_reset_clears_it(strip_layout, jcde_mod):
    """A pool that runs out sets a sticky capacity error; later updates are skipped; reset recovers."""
    import torch

    lay, oeng = strip_layout
    geng = W.replay(jcde.GpuBackend, lay)
    with pytest.raises(jcde.JcdeError):   # the engine's own edges do not fit in 64
        jcde.ResidentEngine(geng.eng, max_edges=64)
    r = jcde.ResidentEngine(geng.eng, max_edges=6000)
    base = r.status()
    assert base["error"] == 0
    q = W.make_queries(W.Stream(0x61, 1), 256, len(lay.items), lay.cde_bbox)
    key = torch.zeros(1, dtype=torch.int32, device="cuda")
    for i in range(len(q)):
        r.register_placed(tq(q[i : i + 1]), key)
    st = r.status()
    assert st["status"] == -3 and st["error"] == 3   # JCDE_ERR_CAPACITY, edge pool
    assert st["edges"] <= 6000
    n_live = st["n_live"]
    r.register_placed(tq(q[:1]), key)   # skipped
    assert int(key.item()) == -1 and r.status()["n_live"] == n_live
    r.reset()
    assert r.status() == base and np.array_equal(r.tree_dump(), oeng.tree_dump())


def test_lbf_select_entry_point_matches_host_choice(oracle_mod, jcde_mod):
    """jcde_lbf_select picks the host rule's candidate (least cost among free ones, first on ties)."""
    from jcde.engine import lbf_select

    spec = lbf.LbfSpec(n_types=12, n_cand=4096)
    lay, geng = lbf.setup(jcde.GpuBackend, spec)
    rng = np.random.default_rng(11)
    for step in range(4):
        q = lbf.step_queries(spec, step)
        q["item"] = rng.integers(0, spec.n_types, len(q))
        v = (rng.random(len(q)) < 0.5).astype(np.uint8)
        assert lbf_select(geng, q, v) == lbf.select_host(lay.items, q, v)
    q = lbf.step_queries(spec, 0)
    q[7] = q[3]
    v = np.ones(len(q), np.uint8)
    v[[3, 7]] = 0
    assert lbf_select(geng, q, v) == 3
    assert lbf_select(geng, q, np.ones(len(q), np.uint8)) == -1


def test_lbf_with_local_search_matches_oracle(oracle_mod, jcde_mod):
    """Uniform round plus three local-search rounds per step, on the device and through the oracle."""
    spec = lbf.LbfSpec(steps=160, n_cand=4096, remove_every=40, ls_rounds=3, ls_cand=1024)
    ref, oeng, got, r = _lbf_pair(oracle_mod, spec, steps_per_graph=16)
    rounds = ref.placements[:, 2] >> 24
    assert (rounds > 0).sum() > 20   # local search improved many steps
    assert got.same_as(ref)
    assert r.status()["error"] == 0
    assert np.array_equal(r.tree_dump(), oeng.tree_dump())


def test_instance_build_matches_oracle(oracle_mod, jcde_mod):
    """A strip-packing instance (reference JSON format): item sequence, discrete and continuous
    orientations, local search; the device build places what the oracle-driven build places."""
    from jcde import instance as I
    from test_instance import DEMO

    inst = I.load_spp(DEMO)
    su_o = I.setup_spp(oracle_mod.OracleBackend, inst, 800.0)
    su_g = I.setup_spp(jcde.GpuBackend, inst, 800.0)
    spec = lbf.spec_for_instance(su_o, n_cand=2048, ls_rounds=2, ls_cand=512)
    ref = lbf.run_host(su_o.layout, su_o.engine, spec)
    got, r = lbf.run_device(su_g.engine, spec, steps_per_graph=4)
    assert len(ref.placements) == 12 and got.same_as(ref)
    assert np.array_equal(r.tree_dump(), su_o.engine.tree_dump())
