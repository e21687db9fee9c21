"""dym-llr (the drop-in for the reference's llr executable) against the same
window ladder driven through the oracle's LLR: hot pass down from Etop, cold
pass up from Ebot, each window seeded from the previous one's configuration
and a_n; the ANE table, the reach counts and the header lines must match the
reference's format and the oracle's values digit for digit."""
import os
import subprocess

import numpy as np
import pytest
from scipy.stats import chi2

from dym_symanzik_action_gb300 import build, tables
from dym_symanzik_action_gb300.schedule import schedule
from oracle.oracle import OracleGroup, OracleLattice

pytestmark = pytest.mark.gpu


def oracle_ladder(path, D, Nt, Nx, axis, bg, Etop, Ebot, step, hw, a0, seed, K, NRM, R, nhit=20):
    og = OracleGroup(path)
    sched = schedule(D, Nt, Nx)
    M = int((Etop - Ebot) / step + 0.5) + 1
    an = [[] for _ in range(M)]
    reached = []
    for r in range(R):
        base = (seed & 0xFFFFFFFF) + 1000003 * r
        for direction, pseed in ((1, base), (-1, base | (1 << 40))):
            L = OracleLattice(og, D, Nt, Nx)
            if direction > 0:
                L.hot_start(pseed)
            else:
                L.links = np.full(L.V * D, og.id, np.uint16)
            a_prev, sweeps, count = a0, 0, 0
            for k in range(M):
                n = k if direction > 0 else M - 1 - k
                res = L.llr_run(sched, Etop - n * step, hw, a_prev, axis=axis, bg=bg, K=K, NRM=NRM, nhit=nhit,
                                drive_cap=20000, seed=pseed, first_sweep=sweeps)
                sweeps += res["sweeps"]
                if res["status"] != "done":
                    break
                an[n].append(res["a"])
                a_prev = res["a"]
                count += 1
            reached.append(count)
    return M, an, reached


def test_dym_llr_matches_oracle_ladder(engine):
    path = tables.ensure_table("S1080")
    D, Nt, Nx, axis, bg = 4, 4, 4, 1, 0.0
    nplaq = Nt * Nx ** 3 * 6
    Etop, Ebot, step, hw = -0.6 * nplaq, -1.2 * nplaq, 0.2 * nplaq, 0.0225 * nplaq / 2
    a0, seed, K, NRM, R = 1.5, 7, 5, 4, 1
    args = [path, D, Nt, Nx, axis, bg, Etop, Ebot, step, hw, a0, seed, K, NRM, R]
    out = subprocess.run([build.LLR_CLI, *map(str, args)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.splitlines()
    M, an, reached = oracle_ladder(*args)
    assert lines[0].startswith("LLR(grp,D,Nt,Nx,axis,bg): ") and lines[0].endswith(f"| {M} windows")
    assert f"NPLAQ: {nplaq}" in lines and f"NRECT: {2 * nplaq}" in lines and f"AXIS: {axis}" in lines
    assert f"repeat 0: down reached {reached[0]}/{M}, up reached {reached[1]}/{M}" in lines
    want = []
    for n in range(M):
        Ewin = Etop - n * step
        if not an[n]:
            want.append("ANE: %8.2f   --(unreached)" % Ewin)
            continue
        x = np.array(an[n])
        sd = float(np.sqrt(((x - x.mean()) ** 2).sum() / (len(x) - 1))) if len(x) > 1 else 0.0
        want.append("ANE: %8.2f  %9.5f  %9.5f  %d" % (Ewin, x.mean(), sd, len(x)))
    got = [l for l in lines if l.startswith("ANE:")]
    assert got == want
    assert sum(reached) > 0


@pytest.mark.parametrize("fixture", ["llr_ref.npz", "llr_ref_s2.npz"])
def test_dym_llr_matches_unmodified_reference(fixture):
    """The a_n ladder of dym-llr against the unmodified reference llr
    executable (its own S(1080) table, K = 50, NRM = 80, R = 20 repeats of the
    hot-down and cold-up passes on each side): llr_ref.npz, S1 windows on a
    4^3x2 lattice whose 32-link colour classes move the energy by about the
    window width; llr_ref_s2.npz, S2 (rectangle) windows on 4^4.  With 20
    samples a side the combined standard error is sd / 3.2, so a bias of one
    per-run sd in a window gives z ~ 3.2.  Bars: every window's |z| < 3.5, and
    the sum of z^2 over the windows below the 99th percentile of chi^2 with
    one degree of freedom per window (a shift of one sd shared by all windows
    fails it)."""
    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", fixture))
    kv = dict(x.split("=") for x in str(ref["args"]).split())
    keys = ("D", "Nt", "Nx", "axis", "bg", "Etop", "Ebot", "step", "hw", "a0", "seed", "K", "NRM", "R")
    args = [tables.ensure_table("S1080"), *[kv[k] for k in keys]]
    out = subprocess.run([build.LLR_CLI, *args], capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr
    rows = [l.split()[1:] for l in out.stdout.splitlines() if l.startswith("ANE:")]
    assert len(rows) == len(ref["ewin"]) and all(len(r) == 4 for r in rows), out.stdout
    got = np.array(rows, float)
    np.testing.assert_allclose(got[:, 0], ref["ewin"], atol=1e-9)
    assert (got[:, 3] == ref["nrep"]).all()
    se = np.sqrt(got[:, 2] ** 2 / got[:, 3] + ref["sd"] ** 2 / ref["nrep"])
    z = (got[:, 1] - ref["mean"]) / se
    print(f"{fixture}: z = {np.round(z, 2).tolist()}")
    assert np.all(np.abs(z) < 3.5), (got[:, 1], ref["mean"], z)
    assert (z ** 2).sum() < chi2.ppf(0.99, len(z)), (got[:, 1], ref["mean"], z)
