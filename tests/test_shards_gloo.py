"""The multi-rank query path on CPU: two gloo ranks, each answering its own shard against its own
replica of the layout (verdicts from the oracle), then the step-time reduction and the gather.
The gathered verdicts equal one process answering both shards."""
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
