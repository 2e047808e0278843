"""Replica sharding of a batch of binaries over ranks (one process per GPU).

Binaries are independent (the reference's batch axis, eob/seobnrv4phm.py:1922-1964
packs them column-wise and nothing couples the columns), so a multi-GPU run
splits the batch by binary and concatenates the per-binary lnL afterwards.
There is no collective on the data path: the only exchange is the final
gather of lnL values (and the max of the per-rank step times for reporting).
"""
from __future__ import annotations

import numpy as np


def shard_range(n: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous balanced range [lo, hi) of n items for `rank` of `world`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of {world}")
    q, r = divmod(n, world)
    lo = rank * q + min(rank, r)
    return lo, lo + q + (1 if rank < r else 0)


def shard_by_cost(cost: np.ndarray, world: int) -> list[np.ndarray]:
    """Split binaries over ranks so that every rank gets a similar longest
    binary and a similar total: binaries in decreasing cost are dealt to the
    rank with the smallest load so far (greedy longest-processing-time).  The
    integrator's time is set by the longest binary of a batch, so dealing the
    long ones first spreads the critical path.  Each rank's indices come back
    in decreasing cost (the order the integrator's work queue wants)."""
    cost = np.asarray(cost, dtype=np.float64)
    order = np.argsort(-cost, kind="stable")
    load = np.zeros(world)
    out = [[] for _ in range(world)]
    for i in order:
        r = int(np.argmin(load))
        out[r].append(int(i))
        load[r] += cost[i]
    return [np.asarray(o, dtype=np.int64) for o in out]


def gather_lnl(local_lnl, local_idx, n_total: int):
    """All-gather per-binary lnL from every rank into one array of n_total
    values indexed by global binary index (torch.distributed must be
    initialised; works with gloo on CPU tensors and with nccl on CUDA ones).
    Binaries no rank computed stay NaN."""
    import torch
    import torch.distributed as dist
    lnl = torch.as_tensor(local_lnl, dtype=torch.float64)
    idx = torch.as_tensor(local_idx, dtype=torch.int64, device=lnl.device)
    world = dist.get_world_size()
    cnt = torch.tensor([lnl.numel()], dtype=torch.int64, device=lnl.device)
    cnts = [torch.zeros_like(cnt) for _ in range(world)]
    dist.all_gather(cnts, cnt)
    m = int(max(int(c.item()) for c in cnts))
    pad_v = torch.full((m,), float("nan"), dtype=torch.float64, device=lnl.device)
    pad_i = torch.full((m,), -1, dtype=torch.int64, device=lnl.device)
    pad_v[:lnl.numel()] = lnl
    pad_i[:idx.numel()] = idx
    all_v = [torch.empty_like(pad_v) for _ in range(world)]
    all_i = [torch.empty_like(pad_i) for _ in range(world)]
    dist.all_gather(all_v, pad_v)
    dist.all_gather(all_i, pad_i)
    out = torch.full((n_total,), float("nan"), dtype=torch.float64, device=lnl.device)
    for v, i in zip(all_v, all_i):
        keep = i >= 0
        out[i[keep]] = v[keep]
    return out


def max_over_ranks(x: float, device=None) -> float:
    """Max of a host scalar over all ranks (identity without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
