"""Query shards over ranks: one process per GPU, weak scaling.

Queries are independent and a layout is read-only while a batch runs (cd_engine.rs queries take
&self), so every rank answers its own batch against its own replica of the layout and no data
moves between ranks on the query path.  The exchanges are the step-time reduction (the slowest
rank sets the time of a step) and, where a caller wants every verdict in one place, a gather.

An LBF-style build (lbf/src/opt/search.rs:41-66) has one real exchange per round: every rank
judges its slice of the round's candidates, and the choice is the least (cost, index) key over
the ranks (`min_u64_over_ranks`; `lbf.run_host(..., ranks=...)`).  Every rank then registers the
same winner in its own replica, so the replicas stay equal with no further transfer.
"""
from __future__ import annotations

import os

import numpy as np

from . import workload as W


def dist_env() -> tuple:
    """(rank, world size, local rank) from the launcher's environment."""
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def rank_queries(lay, n: int, seed: int, rank: int) -> np.ndarray:
    """Rank r's batch: n uniform queries from its own stream (seed, 3 + r); rank 0's is the 1-GPU batch."""
    return W.queries_for(lay, n, seed, sid=3 + rank)


def _dist():
    import torch.distributed as dist

    return dist if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1 else None


def _device():
    import torch

    dist = _dist()
    return torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")


def max_over_ranks(x: float) -> float:
    """The largest of every rank's x (the step time of a weak-scaling run)."""
    dist = _dist()
    if dist is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_verdicts(v: np.ndarray) -> np.ndarray:
    """Every rank's verdict array (equal lengths), concatenated in rank order."""
    dist = _dist()
    if dist is None:
        return np.asarray(v)
    import torch

    t = torch.from_numpy(np.ascontiguousarray(v, dtype=np.uint8)).to(_device())
    parts = [torch.empty_like(t) for _ in range(dist.get_world_size())]
    dist.all_gather(parts, t)
    return np.concatenate([p.cpu().numpy() for p in parts])


def min_u64_over_ranks(key: int) -> int:
    """The least of every rank's unsigned 64-bit key.  Carried as int64 with the top bit flipped,
    which keeps the unsigned order (a < b unsigned iff a ^ 2^63 < b ^ 2^63 signed)."""
    dist = _dist()
    if dist is None:
        return int(key)
    import torch

    t = torch.tensor([int(key) - (1 << 63)], dtype=torch.int64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MIN)
    return int(t.item()) + (1 << 63)


def sum_over_ranks(x: int) -> int:
    """The sum of every rank's count."""
    dist = _dist()
    if dist is None:
        return int(x)
    import torch

    t = torch.tensor([int(x)], dtype=torch.int64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return int(t.item())
