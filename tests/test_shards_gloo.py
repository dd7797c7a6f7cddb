"""The multi-rank paths on CPU with two gloo ranks: the query path (each rank answers its own shard
against its own replica of the layout, then the step-time reduction and the gather; the gathered
verdicts equal one process answering both shards) and the LBF-style build over ranks (each rank
judges a slice of every round's candidates, one all-reduce-min of a 64-bit key per round; every
rank's log equals the one-process build's)."""
import multiprocessing as mp
import os
import socket

import numpy as np


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from jcde import shards
        from jcde import workload as W
        from oracle import oracle as O

        lay, _ = W.strip_layout(O.OracleBackend)
        eng = W.replay(O.OracleBackend, lay)
        r, w, _ = shards.dist_env()
        assert (r, w) == (rank, world)
        q = shards.rank_queries(lay, 4096, 0xC0, r)
        v = eng.detect_batch(q, n_threads=2)
        allv = shards.gather_verdicts(v)
        t = shards.max_over_ranks(0.5 + r)
        if r == 0:
            out.put((allv, t))
    finally:
        dist.destroy_process_group()


def test_two_rank_shards(oracle_mod, strip_layout):
    from jcde import shards
    from jcde import workload as W

    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in ps:
        p.start()
    allv, t = out.get(timeout=300)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    lay, _ = strip_layout
    eng = W.replay(oracle_mod.OracleBackend, lay)
    q0, q1 = (shards.rank_queries(lay, 4096, 0xC0, r) for r in range(2))
    assert not np.array_equal(q0, q1)   # distinct shards
    assert np.array_equal(allv, np.concatenate([eng.detect_batch(q0), eng.detect_batch(q1)]))
    assert t == 1.5   # the slowest rank's time


def test_single_process_fallbacks():
    from jcde import shards

    assert shards.max_over_ranks(2.5) == 2.5
    v = np.arange(10, dtype=np.uint8)
    assert np.array_equal(shards.gather_verdicts(v), v)


# ----------------------------------------------------------------------------------------------
# The LBF-style build over ranks: each rank judges a slice of every round's candidates against its
# own replica; the ranks agree on each round's choice through one all-reduce of a 64-bit key.
# ----------------------------------------------------------------------------------------------
def _lbf_spec():
    from jcde import lbf

    # two tightened uniform rounds and two local-search rounds of 501 (uneven slices)
    return lbf.LbfSpec(steps=120, n_cand=2048, uniform_rounds=2, ls_rounds=2, ls_cand=501)


def _lbf_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from jcde import lbf, shards
        from oracle import oracle as O

        O.build()
        spec = _lbf_spec()
        lay, eng = lbf.setup(O.OracleBackend, spec)
        r, w, _ = shards.dist_env()
        log = lbf.run_host(lay, eng, spec, ranks=(r, w))
        out.put((r, log.placements, log.removals, log.free_counts))
    finally:
        dist.destroy_process_group()


def test_cost_key_order():
    from jcde import lbf

    f = np.float32
    one_up = np.nextafter(f(1.0), f(2.0))
    assert lbf.cost_key(f(1.0), 5) < lbf.cost_key(f(1.0), 6) < lbf.cost_key(one_up, 0)
    assert lbf.cost_key(f(-2.0), 9) < lbf.cost_key(f(-1.0), 0) < lbf.cost_key(f(0.0), 0)
    assert lbf.cost_key(f(-0.0), 3) == lbf.cost_key(f(0.0), 3)   # equal costs: the index decides
    assert lbf.cost_key(f(3.4e38), 2**32 - 1) < lbf.NO_KEY
    rng = np.random.default_rng(7)
    costs = rng.choice(rng.uniform(-1e4, 1e4, 64).astype(np.float32), 4096)   # many ties
    keys = [lbf.cost_key(c, i) for i, c in enumerate(costs)]
    assert int(np.argmin(keys)) == int(np.argmin(costs))   # least cost, first on ties


def test_lbf_rank_slices_without_a_process_group(oracle_mod):
    """ranks = (0, 1) with no process group: the slice is the whole round and the build is the
    one-process build."""
    from jcde import lbf

    spec = _lbf_spec()
    spec.steps = 40
    lay, eng = lbf.setup(oracle_mod.OracleBackend, spec)
    a = lbf.run_host(lay, eng, spec)
    lay, eng = lbf.setup(oracle_mod.OracleBackend, spec)
    b = lbf.run_host(lay, eng, spec, ranks=(0, 1))
    assert a.same_as(b) and len(a.placements) == 40


def test_two_rank_lbf_build(oracle_mod):
    """Two gloo ranks build the layout together; each returns the log of the one-process build
    (placements, removals and per-step counts)."""
    from jcde import lbf

    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_lbf_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in ps:
        p.start()
    got = dict((r, (pl, rm, fc)) for r, pl, rm, fc in (out.get(timeout=600) for _ in range(2)))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    spec = _lbf_spec()
    lay, eng = lbf.setup(oracle_mod.OracleBackend, spec)
    ref = lbf.run_host(lay, eng, spec)
    assert len(ref.placements) > 100 and len(ref.removals) == 2
    assert (ref.placements[:, 2] >> 24).max() >= 2   # some choices came from the local-search rounds
    for r in range(2):
        pl, rm, fc = got[r]
        assert lbf.LbfLog(pl, rm, fc).same_as(ref), r
