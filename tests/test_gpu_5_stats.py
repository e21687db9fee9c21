"""Statistical parity with the unmodified reference, and the drop-in CLI.

tests/golden/chains_1sigma.npz holds GMES/RMES series of the unmodified
reference executable at its compiled NHIT = 20 (its own mys1080-v4 table, hot
start, 4^4, beta = (0, 1.5, 0.1), K 10, N 100, Ntherm 100) for 24 seeds.  The
engine runs the same protocol on the generated, trace-isomorphic S(1080)
table with 24 independent seeds.  Runs from different seeds are independent;
the error of each side's mean is the spread of its per-run means /
sqrt(runs).  Bars, as for the NHIT 10 workloads (test_gpu_14): every one of
the 20 observables within 2 combined standard errors, and Hotelling's T^2 on
(ReP, ImP, plaquette, W[1][1], W[3][3]) above p = 0.01; the fraction within
1 is printed (the observables are strongly correlated, so it is not a count
of independent trials)."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import golden, hotelling_p
from dym_symanzik_action_gb300 import tables

pytestmark = pytest.mark.gpu


def per_run_means(gmes, rmes):
    # GMES: 999, ReP, ImP, plaq, W[0][0..3], ..., W[3][0..3]; RMES: plaq, rect
    return np.concatenate([gmes[:, 1:].mean(0), rmes[:, 1:].mean(0)])


def test_observables_agree_with_reference_chains(engine):
    ref = golden("chains_1sigma.npz")
    ref_runs = np.array([per_run_means(ref[f"gmes_{s}"], ref[f"rmes_{s}"]) for s in ref["seeds"]])
    g = engine.load_group(tables.ensure_table("S1080"))
    our_runs = []
    for s in range(24):
        lat = engine.Lattice(g, 4, 4, 4, 0.0, 1.5, 0.1, 900 + s, start="hot", pool="nearest")
        lat.update(100, 20)
        gm, rm = [], []
        for n in range(100):
            lat.update(10, 20)
            m = lat.measure()
            gm.append([999.0, m.poly_re, m.poly_im, m.plaq, *m.wloop.ravel()])
            rm.append([m.plaq, m.rect])
        our_runs.append(per_run_means(np.array(gm), np.array(rm)))
    our_runs = np.array(our_runs)
    mr, mo = ref_runs.mean(0), our_runs.mean(0)
    se = np.sqrt(ref_runs.var(0, ddof=1) / len(ref_runs) + our_runs.var(0, ddof=1) / len(our_runs))
    z = (mo - mr) / np.where(se > 0, se, 1)
    p = hotelling_p(ref_runs, our_runs, (0, 1, 2, 8, 18))  # ReP, ImP, plaquette, W[1][1], W[3][3]
    print("z-scores (ours - reference) / combined error:", np.round(z, 2).tolist(),
          f"within 1: {np.mean(np.abs(z) < 1):.2f}; Hotelling T^2 p = {p:.3f}")
    assert np.all(np.abs(z) < 2.0), z
    assert p > 0.01, p


def test_cli_matches_python_api(engine):
    from dym_symanzik_action_gb300.build import CLI
    path = tables.ensure_table("S1080")
    r = subprocess.run([CLI, path, "4", "4", "4", "0", "1.5", "0.1", "7", "2", "3", "5"], stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    out = r.stdout.splitlines()
    assert out[0].startswith("PARAMS(grp,D,Nt,Nx,beta0,beta1,beta2,seed): ")
    assert out[1] == "RUN(K,N,Ntherm,NHIT): 2 3 5 20"
    assert "small group size: 72" in out and "START: hot" in out and "thermo done" in out
    gmes = [l for l in out if l.startswith("GMES:")]
    rmes = [l for l in out if l.startswith("RMES:")]
    accl = [l for l in out if l.startswith("ACC:")]
    assert len(gmes) == 3 and len(rmes) == 3 and len(accl) == 3
    assert len(gmes[0].split()) == 1 + 4 + 16
    assert sum(1 for l in out if re.match(r"TM_END:   update {15}", l)) == 3
    g = engine.load_group(path)
    lat = engine.Lattice(g, 4, 4, 4, 0.0, 1.5, 0.1, 7, start="hot")
    lat.update(5, 20)
    for n in range(3):
        lat.update(2, 20)
        m = lat.measure()
        assert m.gmes_line() == gmes[n]
        assert m.rmes_line() == rmes[n]
        assert accl[n] == "ACC: %f" % (lat.acc / lat.hit)


def test_cli_cold_start_and_wilson_restriction(engine):
    from dym_symanzik_action_gb300.build import CLI
    path = tables.ensure_table("S1080")
    env = dict(os.environ, DYM_WLOOP_MAX="2x2", DYM_NHIT="10", DYM_PRECISION="fp64")
    r = subprocess.run([CLI, path, "4", "4", "4", "0", "3.0", "-0.15", "3", "1", "2", "0", "cold"],
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=120, env=env)
    assert r.returncode == 0, r.stderr
    gm = [l for l in r.stdout.splitlines() if l.startswith("GMES:")]
    assert "START: cold" in r.stdout and "RUN(K,N,Ntherm,NHIT): 1 2 0 10" in r.stdout
    assert len(gm) == 2 and len(gm[0].split()) == 1 + 4 + 4


def test_cli_checkpoint_resume(engine, tmp_path):
    """DYM_CHECKPOINT: a run of 2 measurement blocks, resumed for 2 more (no
    thermalisation), prints the GMES and RMES lines of one run of 4 blocks.
    ACC is each run's own running ratio, as in the reference."""
    from dym_symanzik_action_gb300.build import CLI
    path = tables.ensure_table("S1080")
    args = [CLI, path, "4", "4", "4", "0", "1.5", "0.1", "7", "2"]

    def run(extra, env=None):
        r = subprocess.run(args + extra, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=120,
                           env=env)
        assert r.returncode == 0, r.stderr
        return r

    def tagged(r, tag):
        return [l for l in r.stdout.splitlines() if l.startswith(tag)]

    straight = run(["4", "3"])
    ck = tmp_path / "chain.ckpt"
    env = dict(os.environ, DYM_CHECKPOINT=str(ck))
    first = run(["2", "3"], env)
    assert ck.exists() and "resumed" not in first.stderr
    second = run(["2", "0"], env)
    assert "resumed from" in second.stderr and "after 7 sweeps" in second.stderr
    for tag in ("GMES:", "RMES:"):
        assert tagged(first, tag) + tagged(second, tag) == tagged(straight, tag)
    assert engine.checkpoint_info(ck)["sweep"] == 11
