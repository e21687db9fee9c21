"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run where the reference sources exist: REF_DIR, or else baseline/_ref (the
unmodified files oracle/stage_ref.sh places there):

    python tests/golden/make_golden.py

It builds oracle/_ref/ (oracle/build_ref.sh) and writes:

* tables_iso.npz -- for each generated table (S1080, BI, BT, BO): an explicit
  trace-preserving isomorphism pi onto the reference's own file
  (mys1080-v4, myBI, myBT, myBO), the SHA-256 of the reference's Cayley table and of
  ours, and the largest trace difference.  Tests rebuild the reference table
  from ours through pi and compare hashes, so the reference file itself is
  not needed at test time.
* sweeps.npz -- configurations after every sweep, hit/accept counts and
  observables, from the reference's get_staples/get_rect_loops/plaquette/
  wilson/getpoly (compiled from its sources) driven by the Philox colour-phase
  hit loop, for several groups, shapes, couplings and proposal pools.
* ref_tables.npz -- the reference's own mys1080-v4 and myBI traces, and
  configurations after every sweep on those files (reference staples, Philox
  hit loop): the pin for the fast kernels on tables with trace noise.
* staples.npz -- every staple of every link of a random S(1080) 4^4 field, by
  the reference's get_staples and get_rect_loops.
* chains_1sigma.npz -- GMES/RMES series of the unmodified reference
  executable (its own table, NHIT 20, one thread) at the 4^4 couplings
  (0, 1.5, 0.1) for 24 seeds: the statistical oracle at the reference's
  compiled NHIT.
* chains_4x4x4x4_hot.npz, chains_4x4x4x4_hot_eq.npz, chains_32x32x32x8_hot.npz
  -- per-run measurement series of the unmodified reference executable (NHIT
  10 build, its own mys1080-v4, hot starts) at the benchmark workloads: the
  4^4 lattice at beta = (0, 1.5, 0.1) with Ntherm 100, the same after 3,000
  thermalisation sweeps, and the 32^3 x 8 lattice (make_chains_workloads).
* llr_ref.npz -- the ANE table (window centre, mean a_n, sd, samples) of the
  unmodified reference llr executable (its own S(1080) table, one thread) on a
  four-window ladder of S1 (plaquette) windows on a 4^3x2 lattice with R = 20
  repeats of the hot-down and cold-up passes: the statistical oracle for the
  device LLR.
* llr_ref_s2.npz -- the same for two S2 (rectangle) windows on a 4^4 lattice
  (axis 2; every extent >= 3 so that no 1x2 rectangle wraps), R = 20.

* llr2d_ref.npz -- the ANE2 table (cell centres, mean a1 and a2, sds, samples)
  of the unmodified reference llr2d executable (full mode, its own S(1080)
  table, one thread) on three cells of a 4^4 lattice along the S2 ridge that
  one-dimensional windows at beta2 = 0 hold, with R = 20 repeats of its cold
  and hot passes.

    python tests/golden/make_golden.py --only llr     # one fixture only
"""
from __future__ import annotations

import hashlib
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from dym_symanzik_action_gb300 import tables  # noqa: E402
from dym_symanzik_action_gb300.schedule import schedule  # noqa: E402
from oracle.oracle import OracleGroup, OracleLattice, RefHarness, ref_dir  # noqa: E402

REF_DIR = ref_dir()
if REF_DIR is None:
    sys.exit("make_golden.py: set REF_DIR to a reference checkout, or stage one with oracle/stage_ref.sh")
REF_TABLES = {"S1080": "mys1080-v4", "BI": "myBI", "BT": "myBT", "BO": "myBO"}

# name: (group, D, Nt, Nx, (beta0, beta1, beta2), start, seed, nhit, pool_all, nsweeps, wl_nx, wl_nt)
SWEEP_CASES = {
    "s1080_4444_hot": ("S1080", 4, 4, 4, (0.0, 1.5, 0.1), "hot", 20261203, 10, False, 4, 4, 4),
    "s1080_4444_hot_poolall": ("S1080", 4, 4, 4, (0.0, 1.5, 0.1), "hot", 7, 10, True, 3, 2, 2),
    "s1080_4444_cold_b3": ("S1080", 4, 4, 4, (0.0, 3.0, -0.15), "cold", 11, 10, False, 3, 4, 4),
    "s1080_2444_hot": ("S1080", 4, 2, 4, (0.0, 2.0, -0.1), "hot", 99, 10, False, 3, 4, 2),
    "bi_4444_hot": ("BI", 4, 4, 4, (0.0, 2.0, 0.0), "hot", 5, 20, False, 3, 4, 4),
    "bt_6666_hot": ("BT", 4, 6, 6, (0.3, 1.0, 0.2), "hot", 3, 5, False, 3, 3, 3),
    "s1080_d3_844_hot": ("S1080", 3, 8, 4, (0.0, 2.5, -0.2), "hot", 13, 10, False, 3, 4, 8),
    "bi_d2_88_hot": ("BI", 2, 8, 8, (0.0, 1.0, 0.5), "hot", 17, 20, False, 3, 8, 8),
    "su4_bixbo_4448_hot": ("BIxBO", 4, 4, 8, (0.0, 2.0, -0.1), "hot", 2880, 10, False, 3, 4, 4),
}


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, np.int32).tobytes()).hexdigest()


def load_text_table(path):
    toks = open(path).read().split()
    P = int(toks[0])
    re_ = np.array(toks[1:1 + P], float)
    im_ = np.array(toks[1 + P:1 + 2 * P], float)
    m = np.array(toks[1 + 2 * P:1 + 2 * P + P * P], np.int64).reshape(P, P)
    return P, re_, im_, m


def find_isomorphism(mm, rm, rem, imm, rer, imr, seed=1):
    """pi with rm[pi[x], pi[y]] == pi[mm[x, y]] and matching traces, or None."""
    P = mm.shape[0]
    ar = np.arange(P)

    def ident(m):
        return next(n for n in range(P) if (m[n] == ar).all() and (m[:, n] == ar).all())

    def orders(m, e):
        o = np.ones(P, int)
        cur = ar.copy()
        while True:
            done = cur == e
            if done.all():
                return o
            cur = np.where(done, cur, m[cur, ar])
            o = np.where(done, o, o + 1)

    em, er = ident(mm), ident(rm)
    om, orr = orders(mm, em), orders(rm, er)
    invr = np.argmax(rm == er, axis=1)
    rng = np.random.default_rng(seed)

    def gen_size(gs):
        seen = {em}
        q = [em]
        for y in q:
            for g in gs:
                x = int(mm[g, y])
                if x not in seen:
                    seen.add(x)
                    q.append(x)
        return len(seen)

    while True:
        g0, g1 = (int(v) for v in rng.integers(0, P, 2))
        if gen_size([g0, g1]) == P:
            break

    def key(re_, im_, o):
        return (round(float(re_), 8), round(float(im_), 8), int(o))

    kr = [key(rer[i], imr[i], orr[i]) for i in range(P)]
    cand0 = [i for i in range(P) if kr[i] == key(rem[g0], imm[g0], om[g0])]
    cand1 = [i for i in range(P) if kr[i] == key(rem[g1], imm[g1], om[g1])]
    reps, covered = [], set()
    for c in cand0:  # images of g0 up to conjugation in the reference group
        if c in covered:
            continue
        reps.append(c)
        covered.update(rm[rm[:, c], invr].tolist())
    for c0 in reps:
        for c1 in cand1:
            pi = -np.ones(P, int)
            pi[em] = er
            used = np.zeros(P, bool)
            used[er] = True
            q = [em]
            ok = True
            for y in q:
                for g, gi in ((g0, c0), (g1, c1)):
                    x = int(mm[g, y])
                    px = int(rm[gi, pi[y]])
                    if pi[x] < 0:
                        if used[px] or abs(rem[x] - rer[px]) > 1e-9 or abs(imm[x] - imr[px]) > 1e-9:
                            ok = False
                            break
                        pi[x] = px
                        used[px] = True
                        q.append(x)
                    elif pi[x] != px:
                        ok = False
                        break
                if not ok:
                    break
            if ok and (pi >= 0).all() and (rm[pi[:, None], pi[None, :]] == pi[mm]).all():
                return pi
    return None


def make_iso(tabdir):
    out = {}
    for mine, ref in REF_TABLES.items():
        g = tables.generate(mine)
        P, rer, imr, rm = load_text_table(os.path.join(REF_DIR, "groups", ref))
        pi = find_isomorphism(g.mult.astype(np.int64), rm, g.retr, g.imtr, rer, imr)
        assert pi is not None, mine
        out[f"{mine}_pi"] = pi.astype(np.uint16)
        out[f"{mine}_ref_sha"] = np.array(sha(rm))
        out[f"{mine}_our_sha"] = np.array(sha(g.mult))
        out[f"{mine}_max_dtrace"] = np.array(max(np.abs(g.retr - rer[pi]).max(), np.abs(g.imtr - imr[pi]).max()))
        print(f"{mine}: isomorphic to {ref}, max trace difference {float(out[f'{mine}_max_dtrace']):.2e}")
    np.savez_compressed(os.path.join(HERE, "tables_iso.npz"), **out)


def make_sweeps(tabdir):
    ref = RefHarness()
    out = {}
    for name, (gname, D, Nt, Nx, beta, start, seed, nhit, pool_all, nsw, wx, wt) in SWEEP_CASES.items():
        path = tables.ensure_table(gname, tabdir)
        og = OracleGroup(path)
        ol = OracleLattice(og, D, Nt, Nx)
        if start == "hot":
            ol.hot_start(seed)
        sched = schedule(D, Nt, Nx)
        ref.init(path, D, Nt, Nx)
        ref.set_links(ol.links)
        links = [ref.get_links()]
        counts = []
        obs = []
        for s in range(nsw):
            counts.append(ref.sweep(sched, beta, seed, s, 1, nhit, pool_all))
            links.append(ref.get_links())
            obs.append(ref.measure(wx, wt))
        out[name + "_links"] = np.stack(links)
        out[name + "_counts"] = np.array(counts, np.uint64)
        out[name + "_obs"] = np.stack(obs)
        out[name + "_sched_dir"] = sched[0]
        out[name + "_sched_len"] = sched[1]
        out[name + "_sched_sites"] = sched[2]
        acc = np.array(counts)[:, 1].sum() / max(np.array(counts)[:, 0].sum(), 1)
        print(f"{name}: {nsw} sweeps, acceptance {acc:.3f}")
    out["cases"] = np.array(repr(SWEEP_CASES))
    np.savez_compressed(os.path.join(HERE, "sweeps.npz"), **out)


def make_staples(tabdir):
    ref = RefHarness()
    path = tables.ensure_table("S1080", tabdir)
    og = OracleGroup(path)
    ol = OracleLattice(og, 4, 4, 4)
    ol.hot_start(424242)
    ref.init(path, 4, 4, 4)
    ref.set_links(ol.links)
    st = np.zeros((4, ol.V, 24), np.uint16)
    for d in range(4):
        for i in range(ol.V):
            a, b = ref.staples(i, d)
            st[d, i] = np.concatenate([a, b])
    np.savez_compressed(os.path.join(HERE, "staples.npz"), links=ol.links, staples=st, seed=np.array(424242))
    print("staples: 4^4 S1080, 1024 links x 24 staples")


# Cases run on the reference's own table files (traces with ~1e-16 of noise
# inside a class), in the reference's element numbering:
# name: (file, D, Nt, Nx, (beta0, beta1, beta2), start, seed, nhit, nsweeps)
REF_TABLE_CASES = {
    "mys1080_4444_hot": ("mys1080-v4", 4, 4, 4, (0.0, 1.5, 0.1), "hot", 20261203, 10, 4),
    "mys1080_4448_hot_b25": ("mys1080-v4", 4, 8, 4, (0.0, 2.5, -0.1), "hot", 31, 10, 3),
    "mys1080_4444_cold_b3": ("mys1080-v4", 4, 4, 4, (0.0, 3.0, -0.15), "cold", 11, 10, 3),
    "mybi_4444_hot": ("myBI", 4, 4, 4, (0.0, 2.0, 0.0), "hot", 5, 20, 3),
}


def make_reftables():
    """ref_tables.npz: the ReTr/ImTr rows of the reference's mys1080-v4 and
    myBI (its numbering; with tables_iso.npz's pi and the generated Cayley
    table they rebuild the reference file's content exactly), and
    configurations/counts after every sweep of REF_TABLE_CASES by the
    reference's own staples on those files."""
    ref = RefHarness()
    out = {}
    for mine, name in (("S1080", "mys1080-v4"), ("BI", "myBI")):
        P, rer, imr, rm = load_text_table(os.path.join(REF_DIR, "groups", name))
        out[f"{mine}_retr"] = rer
        out[f"{mine}_imtr"] = imr
    for case, (fname, D, Nt, Nx, beta, start, seed, nhit, nsw) in REF_TABLE_CASES.items():
        path = os.path.join(REF_DIR, "groups", fname)
        og = OracleGroup(path)
        ol = OracleLattice(og, D, Nt, Nx)
        if start == "hot":
            ol.hot_start(seed)
        sched = schedule(D, Nt, Nx)
        ref.init(path, D, Nt, Nx)
        ref.set_links(ol.links)
        links = [ref.get_links()]
        counts = []
        for k in range(nsw):
            counts.append(ref.sweep(sched, beta, seed, k, 1, nhit, False))
            links.append(ref.get_links())
        out[case + "_links"] = np.stack(links)
        out[case + "_counts"] = np.array(counts, np.uint64)
        acc = np.array(counts)[:, 1].sum() / max(np.array(counts)[:, 0].sum(), 1)
        print(f"{case}: {nsw} sweeps on the reference's {fname}, acceptance {acc:.3f}")
    out["cases"] = np.array(repr(REF_TABLE_CASES))
    np.savez_compressed(os.path.join(HERE, "ref_tables.npz"), **out)


def parse_log(text):
    gmes = [list(map(float, l.split()[1:])) for l in text.splitlines() if l.startswith("GMES:")]
    rmes = [list(map(float, l.split()[1:])) for l in text.splitlines() if l.startswith("RMES:")]
    acc = [float(l.split()[1]) for l in text.splitlines() if l.startswith("ACC:")]
    return np.array(gmes), np.array(rmes), np.array(acc)


def _ref_chain20(seed):
    """One run of the unmodified reference executable (NHIT 20, its compiled
    default), 4^4 at (0, 1.5, 0.1), K 10, N 100, Ntherm 100, hot, one thread."""
    exe = os.path.join(ROOT, "oracle", "_ref", "dym-mod-metro")
    table = os.path.join(REF_DIR, "groups", "mys1080-v4")
    with tempfile.TemporaryDirectory() as td:  # the -pg build writes gmon.out into its cwd
        r = subprocess.run([exe, table, "4", "4", "4", "0", "1.5", "0.1", str(seed), "10", "100", "100"], cwd=td,
                           env=dict(os.environ, OMP_NUM_THREADS="1"), stdout=subprocess.PIPE,
                           stderr=subprocess.STDOUT, text=True, check=True)
    return seed, parse_log(r.stdout)


def make_chains():
    from concurrent.futures import ProcessPoolExecutor
    seeds = list(range(101, 125))
    out = {}
    with ProcessPoolExecutor(max(1, int(os.environ.get("GOLDEN_WORKERS", os.cpu_count() or 1)))) as ex:
        for s, (g, rm, acc) in ex.map(_ref_chain20, seeds):
            out[f"gmes_{s}"] = g
            out[f"rmes_{s}"] = rm
            out[f"acc_{s}"] = acc
            print(f"reference chain seed {s}: {len(g)} measurements, <plaq> {g[:, 3].mean():.4f}, "
                  f"acceptance {acc[-1]:.3f}")
    out["params"] = np.array("mys1080-v4 D=4 Nt=4 Nx=4 beta=(0,1.5,0.1) K=10 N=100 Ntherm=100 NHIT=20 hot")
    out["seeds"] = np.array(seeds)
    np.savez_compressed(os.path.join(HERE, "chains_1sigma.npz"), **out)


def _ref_chain(job):
    """One run of the unmodified reference (NHIT 10 build) in a scratch
    directory; returns (seed, GMES rows, RMES rows, final ACC)."""
    table, D, Nt, Nx, beta, seed, K, N, Ntherm, threads = job
    from oracle.oracle import run_reference_metro
    out, _ = run_reference_metro(table, D, Nt, Nx, beta, seed, K, N, Ntherm, start="hot", nhit10=True,
                                 threads=threads, timeout=7200)
    g, rm, acc = parse_log(out)
    return seed, g, rm, acc[-1]


# The benchmark workloads as statistical fixtures: the 4^4 run as stated (hot,
# beta = (0, 1.5, 0.1), NHIT 10, Ntherm 100, K 10, N 100, the reference's
# nearest-element pool), and the 32^3 x 8 lattice of the single-chain benchmark with Polyakov
# loop and the 8 x 8 Wilson grid, from a hot start in the disordered phase,
# beta = (0, 1.0, 0.1), where the plaquette settles within a few sweeps (at
# the benchmark's own couplings (0, 3.0, -0.15) a cold chain is frozen, and a hot one -- like one
# at the 4^4 run's couplings, which order 4^4 -- relaxes through a
# first-order transition far longer than a fixture run, so that the
# reference's racing updates and the engine's colour phases would be compared
# out of equilibrium), Ntherm 20, K 4, N 2.
CHAINS_4444 = dict(D=4, Nt=4, Nx=4, beta=(0.0, 1.5, 0.1), K=10, N=100, Ntherm=100, seeds=list(range(3001, 3025)),
                      threads=1)
# The 4^4 couplings in equilibrium: the stated protocol (Ntherm 100) ends
# while the hot start is still relaxing (the plaquette falls from -1.6 to
# -2.91 over its 1,100 sweeps, most of it in the first 300), so its run means
# compare two update orders' relaxation; with Ntherm 3000 both sit on the
# plateau (-2.915) and the runs sample the stationary distribution.
CHAINS_4444_EQ = dict(D=4, Nt=4, Nx=4, beta=(0.0, 1.5, 0.1), K=10, N=100, Ntherm=3000,
                         seeds=list(range(3101, 3133)), threads=1)
CHAINS_32C8 = dict(D=4, Nt=8, Nx=32, beta=(0.0, 1.0, 0.1), K=4, N=2, Ntherm=20, seeds=list(range(4001, 4013)),
                      threads=os.cpu_count() or 1, wl=8)


def make_chains_workloads(which=("chains_4x4x4x4_hot.npz", "chains_4x4x4x4_hot_eq.npz", "chains_32x32x32x8_hot.npz")):
    """chains_4x4x4x4_hot.npz, chains_4x4x4x4_hot_eq.npz and
    chains_32x32x32x8_hot.npz: per-run GMES/RMES of the unmodified reference
    (its Makefile flags, NHIT 10, its own mys1080-v4): the 4^4 runs (as stated
    and in equilibrium) one thread per run (runs in parallel), the 32^3 x 8
    lattice with all cores per run.  Stored per run: the measurement series of ReP, ImP,
    plaq, rect and the Wilson grid (32^3 x 8: its first 8 x 8)."""
    from concurrent.futures import ProcessPoolExecutor
    table = os.path.join(REF_DIR, "groups", "mys1080-v4")
    for name, C in (("chains_4x4x4x4_hot.npz", CHAINS_4444), ("chains_4x4x4x4_hot_eq.npz", CHAINS_4444_EQ),
                    ("chains_32x32x32x8_hot.npz", CHAINS_32C8)):
        if name not in which:
            continue
        jobs = [(table, C["D"], C["Nt"], C["Nx"], C["beta"], s, C["K"], C["N"], C["Ntherm"], C["threads"])
                for s in C["seeds"]]
        workers = max(1, int(os.environ.get("GOLDEN_WORKERS", (os.cpu_count() or 1) // C["threads"])))
        with ProcessPoolExecutor(workers) as ex:
            res = list(ex.map(_ref_chain, jobs))
        out = {}
        for seed, g, rm, acc in res:
            wl = C.get("wl")
            grid = g[:, 4:].reshape(len(g), C["Nx"], C["Nt"])
            if wl:
                grid = grid[:, :wl, :wl]
            out[f"series_{seed}"] = np.concatenate([g[:, 1:4], rm[:, 1:2], grid.reshape(len(g), -1)], 1)
            out[f"acc_{seed}"] = np.array(acc)
            print(f"{name} seed {seed}: {len(g)} measurements, <plaq> {g[:, 3].mean():.5f}, acceptance {acc:.3f}")
        out["columns"] = np.array("ReP ImP plaq rect W[k][l] (k spatial outer, l temporal inner)")
        out["params"] = np.array(repr({k: v for k, v in C.items() if k != "threads"}) +
                                 " table=mys1080-v4 NHIT=10 start=hot pool=nearest")
        out["seeds"] = np.array(C["seeds"])
        np.savez_compressed(os.path.join(HERE, name), **out)


# The LLR ladder of llr_ref.npz, in the reference llr's argument order
# (group D Nt Nx axis bg Etop Ebot step hw a0 seed K NRM R).  With
# NPLAQ = 768: window centres -0.6..-1.2 NPLAQ in steps of 0.2 NPLAQ, width
# 0.0225 NPLAQ (0.5% of the S(1080) plaquette-energy range).
LLR_LADDER = dict(D=4, Nt=2, Nx=4, axis=1, bg=0.0, Etop=-460.8, Ebot=-921.6, step=153.6, hw=8.64, a0=1.5,
                  seed=20261203, K=50, NRM=80, R=20)
# S2 windows (NRECT 3072 on 4^4): centres -0.15 and -0.30 NRECT, width 0.0225 NRECT, beta1 = 0; a0 near the
# solution, so that Robbins-Monro converges within NRM on these wide windows.
LLR_LADDER_S2 = dict(D=4, Nt=4, Nx=4, axis=2, bg=0.0, Etop=-460.8, Ebot=-921.6, step=460.8, hw=34.56, a0=0.5,
                     seed=20261203, K=50, NRM=80, R=20)


def make_llr(L=LLR_LADDER, name="llr_ref.npz"):
    exe = os.path.join(ROOT, "oracle", "_ref", "llr")
    table = os.path.join(REF_DIR, "groups", "mys1080-v4")
    args = [L[k] for k in ("D", "Nt", "Nx", "axis", "bg", "Etop", "Ebot", "step", "hw", "a0", "seed", "K", "NRM",
                           "R")]
    with tempfile.TemporaryDirectory() as td:  # the -pg build writes gmon.out into its cwd
        r = subprocess.run([exe, table, *map(str, args)], cwd=td, env=dict(os.environ, OMP_NUM_THREADS="1"),
                           stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, check=True)
    rows = [l.split()[1:] for l in r.stdout.splitlines() if l.startswith("ANE:")]
    if any(len(x) != 4 for x in rows):
        raise RuntimeError("reference llr left a window unreached:\n" + r.stdout)
    ane = np.array(rows, float)
    print(r.stdout)
    np.savez_compressed(os.path.join(HERE, name), ewin=ane[:, 0], mean=ane[:, 1], sd=ane[:, 2],
                        nrep=ane[:, 3].astype(np.int64),
                        args=np.array(" ".join(f"{k}={v}" for k, v in L.items())),
                        table=np.array("mys1080-v4"))


# The two-dimensional cells of llr2d_ref.npz, in the reference llr2d's argument
# order (group D Nt Nx E1top E1bot step1 hw1 c0 c1 c2 step2 hw2 nperp a0 seed
# K NRM R).  4^4 lattice (NPLAQ 1536, NRECT 3072); cells E1 = -0.6, -0.8, -1.0
# NPLAQ, half-widths 0.0225/2 of NPLAQ and NRECT; the ridge E2(E1) is the
# quadratic through the mean S2 of the one-dimensional S1 windows at these
# centres (beta2 = 0), so each cell lies inside the configurations' support.
LLR2D_GRID = dict(D=4, Nt=4, Nx=4, E1top=-921.6, E1bot=-1536.0, step1=307.2, hw1=17.28, c0=80.333, c1=0.143764,
                  c2=-0.000374147, step2=69.12, hw2=34.56, nperp=0, a0=1.0, seed=11, K=40, NRM=70, R=20)


def make_llr2d():
    exe = os.path.join(ROOT, "oracle", "_ref", "llr2d")
    table = os.path.join(REF_DIR, "groups", "mys1080-v4")
    G = LLR2D_GRID
    args = [G[k] for k in ("D", "Nt", "Nx", "E1top", "E1bot", "step1", "hw1", "c0", "c1", "c2", "step2", "hw2",
                           "nperp", "a0", "seed", "K", "NRM", "R")]
    with tempfile.TemporaryDirectory() as td:  # the -pg build writes gmon.out into its cwd
        r = subprocess.run([exe, table, *map(str, args)], cwd=td, env=dict(os.environ, OMP_NUM_THREADS="1"),
                           stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, check=True)
    rows = [l.split()[1:] for l in r.stdout.splitlines() if l.startswith("ANE2:")]
    n1 = int((G["E1top"] - G["E1bot"]) / G["step1"] + 0.5) + 1
    if len(rows) != n1 * (2 * G["nperp"] + 1):
        raise RuntimeError("reference llr2d left a cell unreached:\n" + r.stdout)
    ane = np.array(rows, float)
    print(r.stdout)
    np.savez_compressed(os.path.join(HERE, "llr2d_ref.npz"), e1=ane[:, 0], e2=ane[:, 1], a1=ane[:, 2], a2=ane[:, 3],
                        sd1=ane[:, 4], sd2=ane[:, 5], nrep=ane[:, 6].astype(np.int64),
                        args=np.array(" ".join(f"{k}={v}" for k, v in LLR2D_GRID.items())),
                        table=np.array("mys1080-v4"))


def main():
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", choices=["iso", "staples", "sweeps", "reftables", "chains", "chains_workloads",
                                       "chains_4444", "chains_4444_eq", "chains_32c8", "llr", "llr_s2",
                                       "llr2d"])
    ap.add_argument("--skip-build", action="store_true", help="use oracle/_ref as built (parallel invocations)")
    args = ap.parse_args()
    only = args.only
    if not args.skip_build:
        subprocess.run(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True,
                       env=dict(os.environ, REF_DIR=REF_DIR), stdout=subprocess.DEVNULL)
    with tempfile.TemporaryDirectory() as tabdir:
        if only in (None, "iso"):
            make_iso(tabdir)
        if only in (None, "staples"):
            make_staples(tabdir)
        if only in (None, "sweeps"):
            make_sweeps(tabdir)
    if only in (None, "reftables"):
        make_reftables()
    if only in (None, "chains"):
        make_chains()
    if only in (None, "chains_workloads"):
        make_chains_workloads()
    if only in ("chains_4444", "chains_4444_eq", "chains_32c8"):
        make_chains_workloads(({"chains_4444": "chains_4x4x4x4_hot", "chains_4444_eq": "chains_4x4x4x4_hot_eq",
                                "chains_32c8": "chains_32x32x32x8_hot"}[only] + ".npz",))
    if only in (None, "llr"):
        make_llr()
    if only in (None, "llr_s2"):
        make_llr(LLR_LADDER_S2, "llr_ref_s2.npz")
    if only in (None, "llr2d"):
        make_llr2d()


if __name__ == "__main__":
    main()
