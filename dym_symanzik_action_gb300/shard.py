"""Sharding an ensemble of independent chains over ranks (one GPU per rank).

Chains never exchange data, so an ensemble (a batch of chains, or a stream
of LLR windows) shards by chain: every rank runs its own share through its own
Batch or Server and only the per-chain results travel, once, to rank 0.  The
reference runs one process per chain or window (evermore.sh, jobs2run); this
is the same split with one process per GPU.

* partition(): longest-processing-time greedy over the chains' work
  (links x sweeps), ties broken by chain index so every rank computes the same
  split without communicating; the heaviest rank carries at most the mean plus
  the largest single chain.
* gather(): rank 0 receives every rank's {chain index: result} (torch.distributed
  all_gather_object on the default process group: gloo on CPU, nccl on GPUs).
* run_sharded(): the driver -- this rank's share by partition(), run by the
  caller's compute (one Batch or one Server on the rank's GPU: ensemble.py;
  the oracle in the CPU tests), gathered to rank 0.
"""
from __future__ import annotations

import heapq
from typing import Any, Callable, Dict, List, Sequence


def partition(work: Sequence[float], world: int) -> List[List[int]]:
    """Indices of the chains each of `world` ranks runs, balanced by `work`."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(work)), key=lambda i: (-float(work[i]), i))
    heap = [(0.0, r) for r in range(world)]
    shards: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        shards[r].append(i)
        heapq.heappush(heap, (load + float(work[i]), r))
    for s in shards:
        s.sort()
    return shards


def chain_work(links: Sequence[int], sweeps: Sequence[int] | int) -> List[float]:
    """Work of each chain: links x sweeps."""
    if isinstance(sweeps, int):
        sweeps = [sweeps] * len(links)
    return [float(l) * float(s) for l, s in zip(links, sweeps)]


def gather(results: Dict[int, Any], rank: int, world: int) -> Dict[int, Any] | None:
    """All ranks' {chain index: result}, merged on rank 0 (None elsewhere)."""
    if world == 1:
        return dict(results)
    import torch.distributed as dist
    parts: List[Any] = [None] * world
    dist.all_gather_object(parts, results)
    if rank != 0:
        return None
    merged: Dict[int, Any] = {}
    for p in parts:
        for k, v in p.items():
            if k in merged:
                raise ValueError(f"chain {k} ran on two ranks")
            merged[k] = v
    return merged


def run_sharded(work: Sequence[float], compute: Callable[[List[int]], Dict[int, Any]], rank: int,
                world: int) -> Dict[int, Any] | None:
    """Run this rank's share of the items (partition() by `work`) through
    compute(indices) -> {index: result} and merge every rank's results on
    rank 0 (None on the other ranks).  Nothing crosses ranks but that final
    gather: the chains or requests of one share never meet another's."""
    mine = partition(work, world)[rank]
    return gather(compute(mine), rank, world)
