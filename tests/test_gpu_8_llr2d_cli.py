"""dym-llr2d (the drop-in for the reference's llr2d executable) against the same
cell walk driven through the oracle's two-dimensional LLR: the full mode's
ANE2 table and ridge counts, the seed mode's manifest and saved configurations
(reference format: int32 element ids, site-major) and the solve mode's table,
digit for digit."""
import os
import subprocess

import numpy as np
import pytest
from scipy.stats import chi2

from dym_symanzik_action_gb300 import build, tables
from dym_symanzik_action_gb300.schedule import schedule
from oracle.oracle import OracleGroup, OracleLattice

pytestmark = pytest.mark.gpu

Nt, Nx = 4, 4
V = Nt * Nx ** 3
N1P = V * 6  # plaquettes
N2R = 2 * N1P  # rectangles
ARGS = dict(E1top=-0.8 * N1P, E1bot=-1.2 * N1P, step1=0.2 * N1P, hw1=0.0225 * N1P / 2, c0=0.3 * N2R, c1=2.0, c2=0.0,
            step2=0.02 * N2R, hw2=0.0225 * N2R / 2, nperp=1, a0=1.5, seed=7)
K, NRM, NHIT, CAP = 4, 5, 20, 4000


def cell_key(pass_seed, i, j):
    return pass_seed + ((i + 1) << 41) + ((j + 1) << 52)


def grid():
    a = ARGS
    N1 = int((a["E1top"] - a["E1bot"]) / a["step1"] + 0.5) + 1
    cells = {}
    for i in range(N1):
        E1 = a["E1top"] - i * a["step1"]
        for j in range(2 * a["nperp"] + 1):
            cells[i, j] = (E1, a["c0"] + a["c1"] * E1 + a["c2"] * E1 * E1 + (j - a["nperp"]) * a["step2"])
    return N1, cells


def start(og, direction, seed):
    L = OracleLattice(og, 4, Nt, Nx)
    if direction > 0:
        L.hot_start(seed)
    else:
        L.links = np.full(4 * V, og.id, np.uint16)
    return L


def oracle_full(og, sched):
    a = ARGS
    N1, cells = grid()
    np_ = a["nperp"]
    res = {k: [] for k in cells}
    reach = {}
    base = a["seed"]
    for direction, pseed in ((-1, base | (1 << 40)), (1, base)):
        L = start(og, direction, pseed)
        sweeps, count = 0, 0
        for s in range(N1):
            i = s if direction > 0 else N1 - 1 - s
            E1, E2 = cells[i, np_]
            r = L.llr2d_run(sched, E1, a["hw1"], E2, a["hw2"], a["a0"], a["a0"], K=K, NRM=NRM, nhit=NHIT,
                            drive_cap=CAP, seed=pseed, first_sweep=sweeps)
            sweeps += r["sweeps"]
            if r["status"] != "done":
                continue
            count += 1
            res[i, np_].append((r["a1"], r["a2"]))
            ridge = L.links.copy()
            for side in (-1, 1):
                for t in range(1, np_ + 1):
                    j = np_ + side * t
                    Lt = OracleLattice(og, 4, Nt, Nx)
                    Lt.links = ridge
                    E1t, E2t = cells[i, j]
                    rt = Lt.llr2d_run(sched, E1t, a["hw1"], E2t, a["hw2"], r["a1"], r["a2"], K=K, NRM=NRM,
                                      nhit=NHIT, drive_cap=CAP, seed=cell_key(pseed, i, j))
                    if rt["status"] != "done":
                        break
                    res[i, j].append((rt["a1"], rt["a2"]))
            L.links = ridge
        reach[direction] = count
    return N1, cells, res, reach


def ane2(E1, E2, samples):
    x = np.array(samples)
    m = x.mean(axis=0)
    sd = np.sqrt(((x - m) ** 2).sum(axis=0) / (len(x) - 1)) if len(x) > 1 else np.zeros(2)
    return "ANE2: %9.2f %9.2f %10.6f %10.6f %9.5f %9.5f %d" % (E1, E2, m[0], m[1], sd[0], sd[1], len(x))


def argv(path):
    a = ARGS
    return [str(v) for v in (path, 4, Nt, Nx, a["E1top"], a["E1bot"], a["step1"], a["hw1"], a["c0"], a["c1"],
                             a["c2"], a["step2"], a["hw2"], a["nperp"], a["a0"], a["seed"])]


def test_full_mode_matches_oracle(engine):
    path = tables.ensure_table("S1080")
    out = subprocess.run([build.LLR2D_CLI, *argv(path), str(K), str(NRM), "1"], capture_output=True, text=True,
                         timeout=900)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.splitlines()
    og = OracleGroup(path)
    N1, cells, res, reach = oracle_full(og, schedule(4, Nt, Nx))
    assert f"NPLAQ: {N1P}" in lines and f"NRECT: {N2R}" in lines
    assert f"repeat 0: cold ridge {reach[-1]}/{N1}, hot ridge {reach[1]}/{N1}" in lines
    want = [ane2(*cells[k], res[k]) for k in sorted(cells) if res[k]]
    assert [l for l in lines if l.startswith("ANE2:")] == want
    assert f"reached {len(want)}/{len(cells)} cells" in lines
    assert reach[-1] + reach[1] > 0


def test_seed_and_solve_modes_match_oracle(engine, tmp_path):
    path = tables.ensure_table("S1080")
    a = ARGS
    seed = subprocess.run([build.LLR2D_CLI, "seed", *argv(path), str(tmp_path)], capture_output=True, text=True,
                          timeout=900)
    assert seed.returncode == 0, seed.stderr
    manifest = [l for l in seed.stdout.splitlines() if l.startswith("CELL:")]
    assert manifest
    # the oracle's seeding walk: one lattice per pass, transverse cells from the ridge configuration
    og = OracleGroup(path)
    sched = schedule(4, Nt, Nx)
    N1, cells = grid()
    np_ = a["nperp"]
    want, saved = [], set()
    base = a["seed"]
    for direction, pseed in ((-1, base | (1 << 40)), (1, base)):
        L = start(og, direction, pseed)
        sweeps = 0

        def drive(i, j):
            nonlocal sweeps
            E1, E2 = cells[i, j]
            r = L.llr2d_run(sched, E1, a["hw1"], E2, a["hw2"], a["a0"], a["a0"], K=1, NRM=0, nhit=NHIT,
                            drive_cap=CAP, seed=pseed, first_sweep=sweeps)
            sweeps += r["sweeps"]
            if r["status"] == "done" and (i, j) not in saved:
                saved.add((i, j))
                want.append((i, j, L.links.copy()))
            return r["status"] == "done"

        for s in range(N1):
            i = s if direction > 0 else N1 - 1 - s
            if not drive(i, np_):
                continue
            ridge = L.links.copy()
            for side in (-1, 1):
                for t in range(1, np_ + 1):
                    L.links = ridge
                    if not drive(i, np_ + side * t):
                        break
            L.links = ridge
    assert [tuple(map(int, l.split()[2:4])) for l in manifest] == [(i, j) for i, j, _ in want]
    for line, (i, j, links) in zip(manifest, want):
        cfg = np.fromfile(line.split()[8], np.int32)
        assert (cfg.reshape(V, 4).T.ravel() == links).all(), (i, j)
    mf = tmp_path / "manifest.txt"
    mf.write_text(seed.stdout)
    solve = subprocess.run([build.LLR2D_CLI, "solve", path, "4", str(Nt), str(Nx), str(mf), "0", str(len(manifest)),
                            str(a["a0"]), str(K), str(NRM), str(a["seed"])], capture_output=True, text=True,
                           timeout=900)
    assert solve.returncode == 0, solve.stderr
    got = [l for l in solve.stdout.splitlines() if l.startswith("ANE2:")]
    exp = []
    for line, (i, j, links) in zip(manifest, want):
        E1, E2, hw1, hw2 = map(float, line.split()[4:8])  # the manifest's %.2f values, as solve reads them
        Ls = OracleLattice(og, 4, Nt, Nx)
        Ls.links = links
        r = Ls.llr2d_run(sched, E1, hw1, E2, hw2, a["a0"], a["a0"], K=K, NRM=NRM, nhit=NHIT, drive_cap=CAP,
                         seed=cell_key(a["seed"], i, j))
        if r["status"] == "done":
            exp.append("ANE2: %9.2f %9.2f %10.6f %10.6f %9.5f %9.5f %d" % (E1, E2, r["a1"], r["a2"], 0.0, 0.0, 1))
    assert got == exp


def test_dym_llr2d_matches_unmodified_reference():
    """Full mode of dym-llr2d against the unmodified reference llr2d executable
    (tests/golden/llr2d_ref.npz: its own S(1080) table, R = 20 repeats of the
    cold and hot ridge passes on each side, K = 40, NRM = 70) on three cells
    of a 4^4 lattice along the S2 ridge.  Bars, for a1 and a2 each: every
    cell's |z| < 3.5 against the reference's mean (combined standard error),
    and the sum of z^2 over the cells below the 99th percentile of chi^2 with
    one degree of freedom per cell."""
    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", "llr2d_ref.npz"))
    kv = dict(x.split("=") for x in str(ref["args"]).split())
    keys = ("D", "Nt", "Nx", "E1top", "E1bot", "step1", "hw1", "c0", "c1", "c2", "step2", "hw2", "nperp", "a0",
            "seed", "K", "NRM", "R")
    out = subprocess.run([build.LLR2D_CLI, tables.ensure_table("S1080"), *[kv[k] for k in keys]],
                         capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr
    rows = [l.split()[1:] for l in out.stdout.splitlines() if l.startswith("ANE2:")]
    assert len(rows) == len(ref["e1"]), out.stdout
    got = np.array(rows, float)
    np.testing.assert_allclose(got[:, 0], ref["e1"], atol=1e-9)
    np.testing.assert_allclose(got[:, 1], ref["e2"], atol=0.006)
    assert (got[:, 6] == ref["nrep"]).all()
    for col, sdc, name in ((2, 4, "a1"), (3, 5, "a2")):
        se = np.sqrt(got[:, sdc] ** 2 / got[:, 6] + ref["sd" + name[1]] ** 2 / ref["nrep"])
        z = (got[:, col] - ref[name]) / se
        print(f"{name}: z = {np.round(z, 2).tolist()}")
        assert np.all(np.abs(z) < 3.5), (name, got[:, col], ref[name], z)
        assert (z ** 2).sum() < chi2.ppf(0.99, len(z)), (name, got[:, col], ref[name], z)
