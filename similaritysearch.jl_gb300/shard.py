"""Database sharding across ranks and the one exchange step it needs.

The exhaustive path shards by contiguous id ranges: rank r holds objects
``lo_r+1 .. hi_r`` (1-based), answers every query on its shard, and the
per-rank top-k lists are merged by the ``(distance, id)`` key -- what
``ParallelExhaustiveSearch``'s per-batch queues merged in batch order amount
to (src/exact/parallel-exhaustive.jl:64-102, src/pqueue/knnsorted.jl:140-168).

The exchange is one ``all_gather`` of ``m x k`` ids and distances per rank
(8 B per entry), over whatever process group the caller initialised: on an
NCCL group the lists travel as tensors on the rank's current GPU, on gloo as
host tensors.  Replicas -- independent ranks answering independent
query streams -- need only ``max_over_ranks`` for timing.
"""
from __future__ import annotations

import numpy as np


def shard_bounds(n: int, world: int, rank: int) -> tuple[int, int]:
    """0-based half-open row range of ``rank``'s shard: contiguous ranges of
    near-equal size, the larger ones first (the partition of
    src/parallel.jl:612-614)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank out of range")
    base, extra = divmod(int(n), int(world))
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def merge_topk(ids_parts, dists_parts, k: int):
    """Merges per-shard result rows (each ``(m, k_r)``, 1-based global ids,
    0 / +Inf for empty slots) into the ``(m, k)`` global result: the k
    smallest entries of each row under ``(distance, id)``, empty slots last."""
    ids = np.concatenate([np.asarray(p, dtype=np.uint32) for p in ids_parts], axis=1)
    dists = np.concatenate([np.asarray(p, dtype=np.float32) for p in dists_parts], axis=1)
    m = ids.shape[0]
    out_i = np.zeros((m, k), dtype=np.uint32)
    out_d = np.full((m, k), np.inf, dtype=np.float32)
    for j in range(m):
        valid = ids[j] != 0
        cand_i, cand_d = ids[j][valid], dists[j][valid]
        order = np.lexsort((cand_i, cand_d))[:k]
        out_i[j, :order.size] = cand_i[order]
        out_d[j, :order.size] = cand_d[order]
    return out_i, out_d


def sharded_searchbatch(local_search, Q, k: int, n: int, group=None):
    """One sharded ``searchbatch``: ``local_search(Q, k)`` answers on this
    rank's shard with 1-based *local* ids; they are shifted to global ids,
    all-gathered and merged.  Every rank returns the same ``(m, k)`` result.
    Collective: every rank of the group must call it with the same Q and k."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    lo, _ = shard_bounds(n, world, rank)
    li, ld = local_search(Q, k)
    li = np.asarray(li, dtype=np.uint32)
    gi = np.where(li != 0, li + np.uint32(lo), 0).astype(np.uint32)
    # NCCL moves device tensors only: gather on this rank's GPU there, on the
    # host for gloo
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend(group) == "nccl" else None
    ti = torch.from_numpy(gi.astype(np.int64))
    td = torch.from_numpy(np.asarray(ld, dtype=np.float32).copy())
    if dev is not None:
        ti, td = ti.to(dev), td.to(dev)
    all_i = [torch.empty_like(ti) for _ in range(world)]
    all_d = [torch.empty_like(td) for _ in range(world)]
    dist.all_gather(all_i, ti, group=group)
    dist.all_gather(all_d, td, group=group)
    return merge_topk([t.cpu().numpy().astype(np.uint32) for t in all_i], [t.cpu().numpy() for t in all_d], k)


def max_over_ranks(value: float, group=None, device=None) -> float:
    """The largest ``value`` over the ranks (the slowest rank's time); the
    value itself when no process group is initialised."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size(group) == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
