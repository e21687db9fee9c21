"""Ensemble sharding over ranks, on CPU: the partition covers every chain once
and is balanced, and two gloo ranks that each run their share through
shard.run_sharded (the driver bench.py runs on GPUs, here with the oracle as
the per-rank compute, one small chain at a time) and gather the results to
rank 0 give exactly the per-chain results of a single process running all
chains."""
import hashlib
import json
import os
import socket

import numpy as np
import pytest

from dym_symanzik_action_gb300 import shard, tables
from dym_symanzik_action_gb300.schedule import schedule
from dym_symanzik_action_gb300.workloads import ensemble

CHAINS = [("S1080", 2, 4, (0.0, 1.5, 0.1), 11), ("BI", 2, 4, (0.0, 2.0, -0.1), 12), ("S1080", 4, 4, (0.0, 3.0, 0.0), 13),
          ("BT", 2, 6, (0.3, 1.0, 0.2), 14), ("BI", 4, 4, (0.0, 1.0, 0.3), 15), ("S1080", 2, 6, (0.0, 2.5, -0.2), 16)]
SWEEPS, NHIT = 2, 3


@pytest.mark.parametrize("world", [1, 2, 4, 8])
def test_partition_of_the_256_chain_ensemble(world):
    specs = ensemble()
    work = shard.chain_work([4 * s.Nt * s.Nx ** 3 for s in specs], 1000)
    parts = shard.partition(work, world)
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(specs)))
    loads = [sum(work[i] for i in p) for p in parts]
    assert max(loads) <= sum(work) / world + max(work)
    assert parts == shard.partition(work, world)  # every rank computes the same split


def run_chain(k):
    from oracle.oracle import OracleGroup, OracleLattice
    gname, Nt, Nx, beta, seed = CHAINS[k]
    L = OracleLattice(OracleGroup(tables.ensure_table(gname)), 4, Nt, Nx)
    L.hot_start(seed)
    h, a = L.sweep(schedule(4, Nt, Nx), beta, seed, 0, SWEEPS, NHIT)
    return [int(h), int(a), hashlib.sha1(np.ascontiguousarray(L.links).tobytes()).hexdigest()]


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        work = shard.chain_work([4 * c[1] * c[2] ** 3 for c in CHAINS], SWEEPS)
        # the same driver bench.py runs on GPUs, with the oracle as the per-rank compute
        merged = shard.run_sharded(work, lambda idx: {k: run_chain(k) for k in idx}, rank, world)
        if rank == 0:
            with open(out_path, "w") as f:
                json.dump({str(k): v for k, v in merged.items()}, f)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_match_one_process(tmp_path):
    import torch.multiprocessing as mp
    out = tmp_path / "merged.json"
    mp.start_processes(_rank_main, args=(2, _free_port(), str(out)), nprocs=2, join=True, start_method="spawn")
    merged = {int(k): v for k, v in json.load(open(out)).items()}
    assert merged == {k: run_chain(k) for k in range(len(CHAINS))}
