#!/usr/bin/env python
"""Benchmark of the discrete-group Symanzik Metropolis engine.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one GPU): a single S(1080) chain on a 32^3 x 8 lattice
(262,144 sites, 1,048,576 uint16 links), cold start, couplings
(beta0, beta1, beta2) = (0, 3.0, -0.15), 10 hits per link.  One step is one
full sweep (every link visited once in the race-free colour phases).  The
metric is link-hits/s = links * hits * sweeps / time.  Synthetic: the group
table is generated (trace-isomorphic to the reference's mys1080-v4).

Timing: W untimed sweeps, then K sweeps each timed with CUDA events on the
chain's stream; a 256 MB buffer (> 129 MB L2) is written between sweeps so
every step starts with the lattice and table out of L2.  `e2e` times the same
sweep through the C ABI (dym_sweep_host) with the configuration copied in
from and out to pinned host memory every step.

--impl reference times the unmodified reference executable (dym-mod-metro
built from the staged sources with its Makefile's flags and NHIT 10, all host
cores) on the same workload and its own mys1080-v4 table: W untimed sweeps
(its Ntherm), then the K steps as one block timed by its TM_END update line.
The engine is not loaded on that arm.
Under torchrun (N > 1) every rank runs its own replica of the chain
(replicas only: a single chain is not sharded); value = total link-hits / the
slowest rank's time.  The forms that do shard -- the 256-chain ensemble and
the served LLR stream -- then also run sharded by work over the ranks
(shard.run_sharded: one Batch / one Server per GPU, per-chain results
gathered to rank 0, no collective on the data path): the `sharded` block.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(group="S1080", D=4, Nt=8, Nx=32, beta=(0.0, 3.0, -0.15), start="cold", nhit=10, seed=20261203)
WORKLOAD_NAME = "single chain S(1080) 32^3x8 cold, beta=(0,3.0,-0.15), 10 hits/link, pool=nearest"


def gathers_per_link_hit(nhit: int) -> float:
    """Algorithmic mult-table gathers per link-hit of the reference algorithm:
    108 per link visit (84 staple products + 24 initial traces) + 25 per hit."""
    return 25.0 + 108.0 / nhit


# L2 work per link visit in 4D, in random 2-byte gathers (one 32-byte sector
# each) from the L2-resident Cayley table.  Mixed-precision kernels (mixed,
# value table): the 87 products of the u_j = s_j * b tree (staples.cuh
# build_u_tree); the hits run from shared memory.  FP64 shared-table kernel:
# 84 staple products + 24 u_j products.  Direct kernel (fp64): those 108 plus
# 25 per hit.  Per launch every block also stages its shared tables from L2.
# dram__bytes_read.sum + dram__bytes_write.sum per sweep launch of this
# workload in the bench's own regime: the mean over the 16 launches of one
# timed step (after the 256 MB flush), from an ncu capture with
# --cache-control none (profiles/sweep_vt_s1080_32x32x32x8_ncu.md: the first
# launch of the step 3.7 MB -- the table and lattice from DRAM and write-backs
# of the flush buffer's dirty lines -- the others 0.6-0.8 MB).  The FP64
# kernel's figure is its capture after ncu's own per-launch flush.  The mixed
# kernel runs this workload only on a chain's first call (the cold chain
# accepts nothing, so later calls use the value table) and has no capture of
# it; None leaves its roofline unreported.
DRAM_BYTES_PER_LAUNCH = {"k_sweep_vt": 899424, "k_sweep_mixed": None, "k_sweep_sub": 2563584}
# smsp__inst_executed.sum (warp instructions) and lts__t_sectors_srcunit_tex.sum
# (L2 sectors requested by the SMs) of one sweep launch of this workload: the
# mean over the 16 launches of a timed step in the same capture (the four
# directions differ by 3% in instructions).  Both are fixed for the workload:
# the cold chain accepts no proposal, so every sweep runs the same
# instructions.
INST_PER_LAUNCH = {"k_sweep_vt": 6107522, "k_sweep_mixed": None, "k_sweep_sub": None}
L2_SECTORS_PER_LAUNCH = {"k_sweep_vt": 492695, "k_sweep_mixed": None, "k_sweep_sub": None}
# Warp instructions an SM can issue per cycle (four schedulers, one each).
ISSUE_PER_SM_CYCLE = 4

PRECISION_DTYPE = {"mixed": "u16/i32+f32 (f64 rechecks)", "shared": "u16/f64", "fp64": "u16/f64"}
PRECISION_TEXT = {
    "mixed": "mixed: exact int32 fixed-point dS, FP32 threshold test, FP64 re-evaluation within the error bound "
             "(decisions identical to FP64)",
    "shared": "fp64 decisions, hit loop from the shared sub-table",
    "fp64": "fp64 decisions, direct table gathers (reference arithmetic)"}


def kernel_model(kernel: int, P: int, npool: int, nhit: int, links_per_launch: int, sms: int):
    """(kernel name, table gathers per link visit, blocks, staged bytes per block) of the
    sweep kernel dym_sweep reported (DYM_KERNEL_*)."""
    # one-wave launches of chunks of max(ceil(links / SMs), 128) links (sweep_launch.cuh phase_shape)
    blocks = -(-links_per_launch // max(-(-links_per_launch // sms), 128))
    if kernel == 4:  # value table (sweep_vt.cu, vt_smem_bytes); accepted moves add 25 gathers each
        return ("k_sweep_vt", 87, blocks, -(-(npool * P * 2) // 16) * 16 + P * 8 + P * 2 + P * 2 + npool * 2 + 16)
    if kernel == 3:  # sweep_mixed.cu, mixed_smem_bytes
        return ("k_sweep_mixed", 87, blocks, P * 8 + 32 * 4 + P * 2 + npool * P * 2 + P + 16)
    if kernel == 2:  # sweep.cu sub_smem_bytes; one wave of 256-thread blocks
        return ("k_sweep_sub", 108, min(sms, -(-links_per_launch // 256)), P * 8 + P * 2 + npool * P * 2 + 16)
    return ("k_sweep_direct", 108 + 25 * nhit, -(-links_per_launch // 256), P * 8 + P * 2 + npool * 2 + 16)


class Clocks:
    """nvidia-smi clock/throttle samples every 200 ms while running."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reference_table_path():
    """The reference's own S(1080) table file (mys1080-v4) from the staged
    reference (baseline/_ref, or $REF_DIR), or None."""
    from oracle.oracle import ref_dir
    r = ref_dir()
    return os.path.join(r, "groups", "mys1080-v4") if r else None


def ensure_reference_build():
    """The unmodified reference executables in oracle/_ref/, built for this
    machine from the staged sources by oracle/build_ref.sh if missing."""
    from oracle import oracle
    exe = os.path.join(oracle.REF_BIN, "dym-mod-metro-nhit10")
    if not os.path.exists(exe):
        ref = oracle.ref_dir()
        if ref is None:
            raise FileNotFoundError("reference sources not staged (oracle/stage_ref.sh) and REF_DIR unset")
        subprocess.run(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True,
                       env=dict(os.environ, REF_DIR=ref), stdout=subprocess.DEVNULL)
    return exe


def reference_binary_run(nsweeps: int, ntherm: int, threads: int):
    """The unmodified reference (dym-mod-metro.cpp built with its Makefile's
    flags, NHIT 10) on the workload: cold 32^3 x 8 chain on its own
    mys1080-v4, beta = (0, 3.0, -0.15), Ntherm untimed sweeps, then one block
    of nsweeps sweeps timed by its own timer (TM_END update,
    dym-mod-metro.cpp:273-278), then its one measurement (untimed).  Returns
    (link-hits, seconds)."""
    from oracle.oracle import run_reference_metro
    w = WORKLOAD
    _, blocks = run_reference_metro(reference_table_path(), w["D"], w["Nt"], w["Nx"], w["beta"], w["seed"],
                                    K=nsweeps, N=1, Ntherm=ntherm, start=w["start"], nhit10=True, threads=threads)
    if len(blocks) != 1:
        raise RuntimeError(f"reference printed {len(blocks)} TM_END update lines, expected 1")
    V = w["Nt"] * w["Nx"] ** (w["D"] - 1)
    return V * w["D"] * w["nhit"] * nsweeps, blocks[0]


def cpu_oracle_run(nsweeps: int, nthreads: int):
    """The oracle port of the reference algorithm on the same workload and the
    reference's own table file, colour phases from oracle.colour_schedule
    (the engine is not loaded): returns (link-hits, seconds)."""
    from oracle.oracle import OracleGroup, OracleLattice, colour_schedule
    w = WORKLOAD
    og = OracleGroup(reference_table_path())
    L = OracleLattice(og, w["D"], w["Nt"], w["Nx"])  # cold start: every link the identity
    sched = colour_schedule(w["D"], w["Nt"], w["Nx"])
    L.sweep(sched, w["beta"], w["seed"], 0, 1, w["nhit"], nthreads=nthreads)  # warm-up sweep
    t0 = time.perf_counter()
    L.sweep(sched, w["beta"], w["seed"], 1, nsweeps, w["nhit"], nthreads=nthreads)
    dt = time.perf_counter() - t0
    return L.V * w["D"] * w["nhit"] * nsweeps, dt


def cpu_baseline(budget_s: float = 15.0):
    """The reference's own OpenMP build timed on this host's cores (all of
    them), with the oracle port beside it as a second, labelled figure."""
    from oracle import oracle
    oracle.build()
    n = os.cpu_count() or 1
    out = {}
    try:
        ensure_reference_build()
        hits1, dt1 = reference_binary_run(2, 0, n)
        ns = max(2, min(200, int(budget_s / max(dt1 / 2, 1e-3))))
        hits, dt = reference_binary_run(ns, 1, n)
        out = {"value": hits / dt, "unit": "link-hits/s", "cores": n, "kind": "reference",
               "sample": f"unmodified reference dym-mod-metro (its Makefile flags, NHIT 10, OMP_NUM_THREADS={n}) "
                         f"on its own mys1080-v4: 1 untimed sweep, then {ns} sweeps of the cold 32^3x8 chain timed "
                         f"by its TM_END update line ({hits:.3e} link-hits, {dt:.2f} s)"}
    except Exception as e:  # reported, not hidden: the line then carries the port only
        out = {"reference_error": f"{type(e).__name__}: {e}"[:300]}
    try:
        h1, d1 = cpu_oracle_run(1, n)
        nsp = max(1, min(200, int(budget_s / max(d1, 1e-3))))
        hp, dp = cpu_oracle_run(nsp, n)
        port = {"value": hp / dp, "unit": "link-hits/s", "cores": n, "kind": "port",
                "sample": f"{nsp} sweeps of the same chain by the oracle restatement of the reference algorithm "
                          f"(reference data layout, OpenMP over a colour phase, {n} threads)"}
    except Exception as e:
        port = {"error": f"{type(e).__name__}: {e}"[:300]}
    if "value" not in out:
        out.update({k: port.get(k) for k in ("value", "unit", "cores", "kind", "sample")})
    out["port"] = port
    return out


def run_reference(args):
    """--impl reference: the unmodified reference executable on this host's
    cores (rank 0 only): W untimed sweeps, then the K timed steps as one
    block of its own update timer."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    n = os.cpu_count() or 1
    try:
        from oracle import oracle
        oracle.build()
        ensure_reference_build()
        hits, dt = reference_binary_run(args.steps, args.warmup, n)
    except Exception as e:
        print(json.dumps({"impl": "reference", "unavailable": f"{type(e).__name__}: {e}"[:300]}), flush=True)
        return
    v = hits / dt
    line = {"impl": "reference", "metric": "link-hits/s", "value": v, "unit": "link-hits/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": bench_config(args.gpus),
            "cpu_baseline": {"value": v, "unit": "link-hits/s", "cores": n, "kind": "reference",
                             "sample": f"unmodified reference dym-mod-metro (Makefile flags, NHIT 10, "
                                       f"OMP_NUM_THREADS={n}) on its own mys1080-v4: {args.warmup} untimed sweeps "
                                       f"(its Ntherm), then {args.steps} sweeps timed by its TM_END update line"},
            "e2e": {"value": v, "unit": "link-hits/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def bench_config(world: int) -> dict:
    """The workload keys shared by both arms' lines."""
    w = WORKLOAD
    V = w["Nt"] * w["Nx"] ** (w["D"] - 1)
    return {"workload": WORKLOAD_NAME, "links": V * w["D"], "nhit": w["nhit"], "sweeps_per_step": 1,
            "l2": "GPU arm: a 256 MB buffer written between steps, also between the e2e steps (L2 flushed); CPU "
                  "arm: the reference's own update timer", "parallelism": f"replicas x{world}"}


def ensemble_bench(dym, device: int, sweeps: int = 5, nhit: int = 10) -> dict:
    """Batched ensemble: 256 chains of uneven size, 200 on S(1080) and 56 on BI, hot
    starts, (beta1, beta2) on a 16x16 grid.  The single-chain GPU path runs
    each chain's sweep with its own dym_sweep call, one chain after another;
    the batched path updates all chains with one kernel per colour-phase slot
    replayed as a CUDA graph, after autotuning.  Both are timed by the wall
    clock around synchronised calls (and by device events)."""
    from dym_symanzik_action_gb300 import tables
    from dym_symanzik_action_gb300.batch import Batch
    from dym_symanzik_action_gb300.workloads import ensemble
    specs = ensemble()
    groups = {n: dym.load_group(tables.ensure_table(n)) for n in ("S1080", "BI")}
    chains = [dym.Lattice(groups[c.group], 4, c.Nt, c.Nx, *c.beta, c.seed, start="hot", device=device)
              for c in specs]
    links = sum(c.links for c in specs)
    for lat in chains:
        lat.update(1, nhit)  # warm-up
    t0 = time.perf_counter()
    single_dev_ms = 0.0
    for _ in range(max(1, sweeps // 2)):
        for lat in chains:
            single_dev_ms += lat.update(1, nhit).device_ms
    single_wall = time.perf_counter() - t0
    single_sweeps = max(1, sweeps // 2)
    b = Batch(device)
    for lat in chains:
        b.add(lat)
    tuning = b.autotune(nhit=nhit, nsweeps_per_trial=1)
    b.update(1, nhit)  # warm-up (graph already captured by the autotuner's last trial)
    t0 = time.perf_counter()
    st = b.update(sweeps, nhit)
    batch_wall = time.perf_counter() - t0
    n, nlinks, nslots = b.size
    hits_single = links * nhit * single_sweeps
    hits_batch = links * nhit * sweeps
    assert st.hits == hits_batch
    out = {"workload": "256 chains: Nx in {8..24}, Nt in {2,4,6,8}, 200 S(1080) + 56 BI, hot, 10 hits/link",
           "chains": n, "links": nlinks, "colour_phase_slots": nslots, "sweeps_timed": sweeps,
           "batched_link_hits_per_s": hits_batch / batch_wall,
           "batched_device_link_hits_per_s": hits_batch / (st.device_ms * 1e-3),
           "single_chain_link_hits_per_s": hits_single / single_wall,
           "single_chain_device_link_hits_per_s": hits_single / (single_dev_ms * 1e-3),
           "speedup_batched_vs_single": (hits_batch / batch_wall) / (hits_single / single_wall),
           "tuning": {"tile": tuning.tile, "threads": tuning.threads, "grid_per_sm": tuning.grid_per_sm,
                      "cuda_graph": tuning.use_graph, "hit_unroll": tuning.hit_unroll}}
    b.close()
    for lat in chains:
        lat.close()
    return out


def serving_bench(dym, device: int, n_requests: int, nhit: int = 20, step_sweeps: int = 5,
                  max_chains: int = 512, max_links: int = 0) -> dict:
    """Served LLR stream: windows arriving as a Poisson stream (200/s) on S(1080)
    lattices Nx in {6,8,12,16}, Nt in {2,4}, beta2 in {0,-0.1}; each request one
    window of 0.5% of the plaquette-energy range, 20 Robbins-Monro iterations of
    50 sweeps.  Requests are submitted when their arrival time has passed (wall
    clock), the server admits them by resident-chain count and device memory,
    and latency is completion minus arrival (serve.serve_stream)."""
    import numpy as np
    from dym_symanzik_action_gb300 import tables
    from dym_symanzik_action_gb300.serve import Server, serve_stream
    from dym_symanzik_action_gb300.workloads import llr_requests
    reqs = llr_requests(n=2000)[:n_requests]
    g = dym.load_group(tables.ensure_table("S1080"))
    srv = Server(g, max_chains=max_chains, hbm_budget=8 << 30, nhit=nhit, device=device, max_links=max_links)
    res, wall = serve_stream(srv, reqs, step_sweeps)
    hits = srv.status()["link_hits"]
    srv.close()
    L = np.array([v[3] for v in res.values()])
    which = "all 2000" if len(reqs) == 2000 else f"first {len(reqs)} of 2000"
    return {"workload": f"{which} LLR window requests, Poisson 200/s, S(1080), Nx in {{6,8,12,16}}, "
                        f"Nt in {{2,4}}, 20 RM x 50 sweeps, {nhit} hits/link, at most {max_chains} resident",
            "requests": len(reqs), "wall_s": wall, "link_hits_per_s": hits / wall,
            "latency_p50_s": float(np.percentile(L, 50)), "latency_p99_s": float(np.percentile(L, 99)),
            "unreached": sum(1 for v in res.values() if v[0] != "done"), "max_resident_chains": max_chains,
            "max_resident_links": max_links or None}  # 0 = no cap


def sharded_bench(local: int, rank: int, world: int, n_requests: int, sweeps: int = 5, nhit: int = 10) -> dict:
    """The forms that shard: every rank runs its share of the 256-chain
    ensemble as one Batch and its share of the LLR request stream through one
    Server (shard.run_sharded; partition by work, no data-path collective),
    results gathered to rank 0.  Value = all ranks' link-hits /
    the slowest rank's wall time (total work fixed: strong scaling)."""
    import numpy as np
    import torch.distributed as dist
    from dym_symanzik_action_gb300 import ensemble, shard
    from dym_symanzik_action_gb300.workloads import ensemble as ens_specs
    from dym_symanzik_action_gb300.workloads import llr_requests

    def all_timings(t):
        parts = [None] * world
        if world > 1:
            dist.all_gather_object(parts, t)
        else:
            parts = [t]
        return parts

    out = {}
    specs = ens_specs()
    work = shard.chain_work([s.links for s in specs], sweeps)
    t = {}
    merged = shard.run_sharded(work, ensemble.batch_compute(specs, sweeps, nhit, local, timing=t), rank, world)
    ts = all_timings(t)
    if rank == 0:
        wall = max(x["wall_s"] for x in ts)
        hits = sum(x.get("hits", 0) for x in ts)
        out["ensemble"] = {"workload": "the 256-chain ensemble, 5 sweeps, 10 hits/link, sharded by work",
                           "ranks": world, "chains_per_rank": [x["chains"] for x in ts],
                           "links_per_rank": [x["links"] for x in ts], "chains_gathered": len(merged),
                           "link_hits_per_s": hits / wall, "slowest_rank_wall_s": wall, "scaling": "strong"}
    if n_requests > 0:
        reqs = llr_requests(n=2000)[:n_requests]
        rwork = [float(r.nplaq * r.K * r.NRM) for r in reqs]
        t = {}
        merged = shard.run_sharded(rwork, ensemble.stream_compute(reqs, local, timing=t), rank, world)
        ts = all_timings(t)
        if rank == 0:
            wall = max(x["wall_s"] for x in ts)
            L = np.array([v[3] for v in merged.values()])
            out["serving"] = {"workload": f"first {len(reqs)} requests of the LLR request stream, sharded by work",
                              "ranks": world, "requests_per_rank": [x["requests"] for x in ts],
                              "link_hits_per_s": sum(x["link_hits"] for x in ts) / wall,
                              "latency_p50_s": float(np.percentile(L, 50)),
                              "latency_p99_s": float(np.percentile(L, 99)),
                              "unreached": sum(1 for v in merged.values() if v[0] != "done"), "scaling": "strong"}
    return out


def chain_rate(dym, group, start: str, device: int, steps: int, warmup: int, flush, beta=None, Nt=None, Nx=None):
    """Device link-hits/s of one chain of the workload's shape (or Nt x Nx^3)
    on `group`, each step one sweep after an L2 flush, as the headline."""
    import torch
    w = WORKLOAD
    Nt, Nx = Nt or w["Nt"], Nx or w["Nx"]
    lat = dym.Lattice(group, w["D"], Nt, Nx, *(beta or w["beta"]), w["seed"], start=start, precision="mixed",
                      device=device)
    for _ in range(warmup):
        lat.update(1, w["nhit"])
    ms, hits, acc, kernels = 0.0, 0, 0, set()
    for k in range(steps):
        flush.fill_(k & 0xFF)
        torch.cuda.synchronize()
        st = lat.update(1, w["nhit"])
        ms += st.device_ms
        hits += st.hits
        acc += st.accepts
        kernels.add(int(st.kernel))
    lat.close()
    names = {2: "k_sweep_sub", 3: "k_sweep_mixed", 4: "k_sweep_vt", 1: "k_sweep_direct"}
    return {"link_hits_per_s": hits / (ms * 1e-3), "ms_per_sweep": ms / steps, "acceptance": acc / hits,
            "kernels": sorted(names.get(k, str(k)) for k in kernels), "sweeps_timed": steps}


def reference_table_bench(dym, device: int, steps: int, warmup: int, flush) -> dict:
    """The headline workload on the reference's own mys1080-v4 file (ReTr with
    rounding noise inside a class), beside the same on the generated table."""
    path = reference_table_path()
    if path is None:
        return {"unavailable": "reference not staged (oracle/stage_ref.sh)"}
    g = dym.load_group(path)
    out = {"table": "the reference's groups/mys1080-v4", "fast_path": bool(g.fast_path),
           "classes_exact": bool(g.classes_exact), "class_spread": g.class_spread}
    out.update(chain_rate(dym, g, "cold", device, steps, warmup, flush))
    g.close()
    return out


def mixed_precision_scan(dym, device: int, sweeps: int = 300, nhit: int = 10) -> dict:
    """S(1080) 48^3 x 12 (5,308,416 links), hot start, beta1 in {2.0, 2.5, 3.0},
    beta2 = -0.1: the mixed kernel against the all-FP64 shared-table kernel from
    the same start, configuration compared every 50 sweeps; recheck fraction
    and largest |dS_fast - dS_fp64| seen at a recheck."""
    import numpy as np
    from dym_symanzik_action_gb300 import tables
    g = dym.load_group(tables.ensure_table("S1080"))
    out = []
    for b1 in (2.0, 2.5, 3.0):
        lm = dym.Lattice(g, 4, 12, 48, 0.0, b1, -0.1, 4848, start="hot", precision="mixed", device=device)
        lf = dym.Lattice(g, 4, 12, 48, 0.0, b1, -0.1, 4848, start="hot", precision="shared", device=device)
        same, hits, acc, rechecks, max_err, ms_m, ms_f = True, 0, 0, 0, 0.0, 0.0, 0.0
        for _ in range(sweeps // 50):
            sm = lm.update(50, nhit)
            sf = lf.update(50, nhit)
            hits += sm.hits
            acc += sm.accepts
            rechecks += sm.rechecks
            max_err = max(max_err, sm.max_ds_err)
            ms_m += sm.device_ms
            ms_f += sf.device_ms
            same = same and sm.accepts == sf.accepts and bool(np.array_equal(lm.links, lf.links))
        out.append({"beta1": b1, "beta2": -0.1, "sweeps": sweeps, "identical_to_fp64": same,
                    "acceptance": acc / hits, "recheck_fraction": rechecks / hits, "max_ds_err": max_err,
                    "mixed_link_hits_per_s": hits / (ms_m * 1e-3), "fp64_link_hits_per_s": hits / (ms_f * 1e-3)})
        lm.close()
        lf.close()
    return {"workload": "S(1080) 48^3x12 hot, beta2=-0.1, 10 hits/link; mixed vs all-FP64 shared-table kernel",
            "scan": out}


def run_ours(args):
    import numpy as np
    import torch

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from dym_symanzik_action_gb300 import build as b
    b.build()
    import dym_symanzik_action_gb300 as dym
    from dym_symanzik_action_gb300 import _lib, tables
    from dym_symanzik_action_gb300._lib import check, lib, ptr

    w = WORKLOAD
    g = dym.load_group(tables.ensure_table(w["group"]))
    lat = dym.Lattice(g, w["D"], w["Nt"], w["Nx"], *w["beta"], w["seed"] + rank, start=w["start"],
                      precision=args.precision, device=local)
    links_per_sweep = lat.V * w["D"]
    hits_per_step = links_per_sweep * w["nhit"]
    nphase = len(lat.schedule()[0])

    # L2 random-gather peak (roofline denominator), measured live.
    sps = C.c_double()
    check(lib().dym_probe_l2_gather(local, 1080 * 1080 * 2, C.byref(sps)))

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        lat.update(1, w["nhit"])
    barrier()
    dev_ms = 0.0
    launches = 0
    acc = 0
    rechecks = 0
    with Clocks(local) as clk:
        t_wall0 = time.perf_counter()
        for k in range(args.steps):
            flush.fill_(k & 0xFF)
            torch.cuda.synchronize()
            st = lat.update(1, w["nhit"])
            kernel_used = st.kernel
            dev_ms += st.device_ms
            launches += st.launches
            acc += st.accepts
            rechecks += st.rechecks
        barrier()
        t_wall = time.perf_counter() - t_wall0
    clocks = clk.summary()

    # e2e: the configuration in from and out to pinned host memory every step,
    # through the C ABI's host-resident sweep (dym_sweep_host: upload and
    # check, the sweep, read-back, one synchronisation).
    n = links_per_sweep
    host_in = torch.empty(n, dtype=torch.uint16, pin_memory=True).numpy()
    host_out = torch.empty(n, dtype=torch.uint16, pin_memory=True).numpy()
    host_in[:] = lat.links.ravel()
    stt = _lib.Stats()
    # The C-ABI function, the chain handle and the two buffers' pointers are
    # looked up once, as a C caller holds them; the timed region is the call.
    sweep_host = lib().dym_sweep_host
    p_in, p_out, p_st = ptr(host_in, C.c_uint16), ptr(host_out, C.c_uint16), C.byref(stt)
    for _ in range(2):
        check(sweep_host(lat._h, p_in, p_out, 1, w["nhit"], p_st))
    barrier()
    e2e_s = 0.0
    for k in range(args.steps):
        flush.fill_(k & 0xFF)  # every step starts with L2 flushed, as the device-timed steps
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc = sweep_host(lat._h, p_in, p_out, 1, w["nhit"], p_st)
        e2e_s += time.perf_counter() - t0
        check(rc)
        p_in, p_out = p_out, p_in  # this step's output is the next step's input
    barrier()

    times = torch.tensor([dev_ms, e2e_s], dtype=torch.float64, device=f"cuda:{local}")
    if world > 1:
        torch.distributed.all_reduce(times, op=torch.distributed.ReduceOp.MAX)
    dev_ms_max, e2e_max = times.tolist()
    total_hits = hits_per_step * args.steps * world
    value = total_hits / (dev_ms_max * 1e-3)
    e2e_value = total_hits / e2e_max

    G_ref = gathers_per_link_hit(w["nhit"])
    avg_launch_s = dev_ms * 1e-3 / max(launches, 1)
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    links_per_launch = links_per_sweep / nphase
    kname, gathers, blocks, block_bytes = kernel_model(kernel_used, g.P, len(g.smallgroup), w["nhit"],
                                                       int(links_per_launch), sms)
    stage_bytes = blocks * block_bytes
    alg_bytes_per_launch = links_per_launch * gathers * 32 + stage_bytes
    hbm_bytes = links_per_sweep * 2 * 2  # every link read and written once per sweep
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    traffic = DRAM_BYTES_PER_LAUNCH.get(kname)
    # Issue roofline: the kernel's warp instructions per launch (ncu) over the
    # live launch time, against SMs x 4 schedulers x the SM clock sampled
    # during the timed region.
    sm_hz = (clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0) * 1e6
    issue_peak = sms * ISSUE_PER_SM_CYCLE * sm_hz
    inst = INST_PER_LAUNCH.get(kname)
    issue_achieved = inst / avg_launch_s if inst else None
    # L2-gather roofline of the reference algorithm: the measured random-gather
    # sector rate over its 25 + 108/NHIT gathers per link-hit.
    l2_roof = sps.value / G_ref
    l2_sectors = L2_SECTORS_PER_LAUNCH.get(kname)

    if rank == 0:
        line = {
            "metric": "link-hits/s", "value": value, "unit": "link-hits/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": PRECISION_DTYPE[args.precision],
            "data": "synthetic",
            "config": bench_config(world),
            "method": {"colour_phases": nphase, "precision": PRECISION_TEXT[args.precision], "kernel": kname,
                       "table": "generated S(1080) (trace-isomorphic to the reference's mys1080-v4)"},
            "roofline": {"bound": "issue", "achieved": issue_achieved, "peak": issue_peak, "unit": "warp-inst/s",
                         "frac": issue_achieved / issue_peak if issue_achieved else None, "traffic": traffic,
                         "peak_source": (f"{sms} SMs x {ISSUE_PER_SM_CYCLE} warp instructions per cycle x "
                                         f"{sm_hz / 1e6:.0f} MHz (median SM clock sampled in the timed region)"),
                         "algorithmic": (f"{kname}: {inst} warp instructions per launch (ncu smsp__inst_executed.sum "
                                         f"of this workload) / CUDA-event launch time; {links_per_launch:.0f} "
                                         f"links x {w['nhit']} hits per launch"),
                         "l2_gather": {
                             "peak_sectors_per_s": sps.value,
                             "peak_source": "measured live: random 2-byte L2 gathers (dym_probe_l2_gather)",
                             "reference_gathers_per_link_hit": G_ref,
                             "roofline_link_hits_per_s": l2_roof, "frac": value / l2_roof,
                             "kernel_gathers_per_link_hit": gathers / w["nhit"],
                             "kernel_alg_bytes_per_launch": alg_bytes_per_launch,
                             "kernel_l2_sectors_per_launch": l2_sectors,
                             "kernel_l2_frac": (l2_sectors / avg_launch_s / sps.value) if l2_sectors else None,
                             "note": ("frac > 1: the hits read shared memory, not L2, and half of the staple "
                                      "gathers hit L1; kernel_l2_frac is the L2 sector rate the kernel drew "
                                      "(ncu) against the gather peak")},
                         "hbm": {"achieved": hbm_bytes / (dev_ms * 1e-3 / args.steps) / 1e9, "peak": hbm_peak,
                                 "unit": "GB/s", "note": "compulsory link streaming, 4 B/link/sweep, of measured"}},
            "e2e": {"value": e2e_value, "unit": "link-hits/s", "h2d_bytes_per_step": n * 2,
                    "d2h_bytes_per_step": n * 2 + 6 * 8, "call": "dym_sweep_host"},
            "gpu_launches": launches,
            "acceptance": acc / (hits_per_step * args.steps), "recheck_fraction": rechecks / (hits_per_step * args.steps),
            "clocks": clocks,
            "wall_s_timed_region": t_wall,
        }
    if rank == 0 and world == 1:
        # Single-GPU extras.  A moving (hot-start) chain of the same shape and
        # couplings, beside the frozen cold one, and the headline on the
        # reference's own table file.
        line["moving_chain"] = dict(workload="single chain S(1080) 32^3x8 HOT, beta=(0,3.0,-0.15), 10 hits/link",
                                    **chain_rate(dym, g, "hot", local, args.steps, args.warmup, flush))
        line["reference_table"] = reference_table_bench(dym, local, args.steps, args.warmup, flush)
        if not args.no_ensemble:
            line["batched"] = ensemble_bench(dym, local)
        if args.serve_requests > 0:
            line["serving"] = serving_bench(dym, local, args.serve_requests)
        if not args.no_mixed_scan:
            line["mixed_precision"] = mixed_precision_scan(dym, local)
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline()
    if world > 1:
        # every rank takes part: each runs its share of the ensemble and the stream
        sh = sharded_bench(local, rank, world, min(args.serve_requests, 400))
        if rank == 0:
            line["sharded"] = sh
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precision", choices=["mixed", "shared", "fp64"], default="mixed",
                    help="single-chain kernel: mixed (default), shared (FP64 shared-table), fp64 (direct)")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the batched 256-chain ensemble")
    ap.add_argument("--no-mixed-scan", action="store_true", help="skip the 48^3x12 mixed-vs-FP64 scan")
    ap.add_argument("--serve-requests", type=int, default=2000,
                    help="requests of the served LLR stream to run (2000 = the whole stream; 0 = skip)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
