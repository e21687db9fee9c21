"""Per-rank compute of the sharded ensemble forms (shard.run_sharded).

The reference runs one process per chain or per LLR window (evermore.sh,
jobs2run, scripts/llr2d_parallel.sh); here one process per GPU runs its share
of the chains as one Batch, or its share of the request stream through one
Server, and only per-chain results travel (shard.gather).

* batch_compute(): the chains of a share (ChainSpec, workloads.ensemble) as one
  Batch on the rank's GPU, `sweeps` sweeps; per chain (hits, accepts, SHA-1 of
  the final configuration), identical to the chain run alone.
* stream_compute(): the requests of a share (workloads.llr_requests) served
  by one Server at their arrival times (serve.serve_stream); per request its
  status, a, sweeps and latency.
"""
from __future__ import annotations

import hashlib
import time
from typing import Dict, List, Sequence

import numpy as np


def links_digest(links: np.ndarray) -> str:
    return hashlib.sha1(np.ascontiguousarray(links, np.uint16).tobytes()).hexdigest()


def batch_compute(specs: Sequence, sweeps: int, nhit: int, device: int, autotune: bool = True,
                  timing: dict | None = None):
    """compute(indices) for shard.run_sharded: the chains specs[i] of the share
    as one Batch on `device`.  `timing` (if given) receives the share's link
    count, the batched sweep's wall and device seconds and the tuning."""
    def compute(indices: List[int]) -> Dict[int, list]:
        from . import tables
        from .batch import Batch
        from .metro import Lattice, load_group
        if not indices:
            if timing is not None:
                timing.update(links=0, wall_s=0.0, device_s=0.0, chains=0)
            return {}
        groups, lats = {}, []
        for i in indices:
            s = specs[i]
            if s.group not in groups:
                groups[s.group] = load_group(tables.ensure_table(s.group))
            lats.append(Lattice(groups[s.group], 4, s.Nt, s.Nx, *s.beta, s.seed, start=s.start, device=device))
        b = Batch(device)
        for lat in lats:
            b.add(lat)
        tune = b.autotune(nhit=nhit, nsweeps_per_trial=1) if autotune else None
        t0 = time.perf_counter()
        st = b.update(sweeps, nhit)
        wall = time.perf_counter() - t0
        out = {}
        for k, (i, lat) in enumerate(zip(indices, lats)):
            h, a = b.chain_counters(k)
            out[i] = [int(h), int(a), links_digest(lat.links)]
        if timing is not None:
            timing.update(links=int(sum(l.V * l.D for l in lats)), wall_s=wall, device_s=st.device_ms * 1e-3,
                          chains=len(lats), hits=int(st.hits),
                          tuning=None if tune is None else dict(tile=tune.tile, threads=tune.threads,
                                                                grid_per_sm=tune.grid_per_sm,
                                                                cuda_graph=tune.use_graph))
        b.close()
        for lat in lats:
            lat.close()
        return out
    return compute


def stream_compute(requests: Sequence, device: int, nhit: int = 20, step_sweeps: int = 5, max_chains: int = 512,
                   hbm_budget: int = 8 << 30, timing: dict | None = None):
    """compute(indices) for shard.run_sharded: the requests of the share
    served by one Server on `device` as they arrive (arrival times relative
    to the start of the call)."""
    def compute(indices: List[int]) -> Dict[int, list]:
        from . import tables
        from .metro import load_group
        from .serve import Server, serve_stream
        share = [requests[i] for i in indices]
        if not share:
            if timing is not None:
                timing.update(wall_s=0.0, link_hits=0, requests=0)
            return {}
        g = load_group(tables.ensure_table("S1080"))
        srv = Server(g, max_chains=max_chains, hbm_budget=hbm_budget, nhit=nhit, device=device)
        res, wall = serve_stream(srv, share, step_sweeps)
        if timing is not None:
            timing.update(wall_s=wall, link_hits=int(srv.status()["link_hits"]), requests=len(share))
        srv.close()
        g.close()
        return {r.rid: res[r.rid] for r in share}
    return compute
