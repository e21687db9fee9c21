"""The reference's own dym-mod-metro driver with its sweeps on the engine.

oracle/_ref/dym-mod-metro-gpu is built by oracle/build_ref.sh from the staged
reference sources: its two sweep loops call dym_sweep_refarray (through
oracle/ref_gpu_driver.cpp) on its own int32 link array, and everything else --
arguments, table loading, its hot or cold start, its measurements, output
lines and timer -- is the reference's code.

* The output keeps the reference's lines.
* Statistics: 24 runs at the 4^4 couplings (0, 1.5, 0.1) after 3,000
  thermalisation sweeps, K 10, N 100, against the 32 runs of the unmodified
  reference in chains_4x4x4x4_hot_eq.npz: every one of the 20 observables
  within 2 combined standard errors, and Hotelling's T^2 on (ReP, ImP,
  plaquette, W[1][1], W[3][3]) above p = 0.01.  The fixture's runs are the
  reference's serial update order with NHIT 10, these its compiled NHIT 20 on
  the engine's colour phases: both sample the same stationary distribution,
  which is what equilibrium run means compare (with the stated 100
  thermalisation sweeps the hot start is still relaxing, at a rate that
  depends on the update order).
* One block of 20 sweeps of the cold 32^3 x 8 chain at (0, 3.0, -0.15) timed
  by its own TM_END update line (printed as link-hits/s).
Skipped where the reference is not staged."""
import os
import subprocess
import tempfile
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from conftest import golden, hotelling_p
from oracle.oracle import _TM_UPDATE, REF_BIN, ref_dir

pytestmark = pytest.mark.gpu

EXE = os.path.join(REF_BIN, "dym-mod-metro-gpu")


def run(args, timeout=600):
    with tempfile.TemporaryDirectory() as td:  # its timer objects are built with -pg (gmon.out in the cwd)
        r = subprocess.run([EXE, *map(str, args)], cwd=td, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                           text=True, timeout=timeout, env=dict(os.environ, OMP_NUM_THREADS="4"))
    assert r.returncode == 0, r.stdout[-2000:]
    return r.stdout


def parse(out):
    """Per-measurement rows [ReP, ImP, plaq, rect, W[0][0..3], ..., W[3][0..3]]
    from the GMES (999, ReP, ImP, plaq, W...) and RMES (plaq, rect) lines."""
    g = np.array([list(map(float, l.split()[1:])) for l in out.splitlines() if l.startswith("GMES:")])
    rm = np.array([list(map(float, l.split()[1:])) for l in out.splitlines() if l.startswith("RMES:")])
    return np.concatenate([g[:, 1:4], rm[:, 1:2], g[:, 4:]], axis=1)


@pytest.fixture(scope="module")
def table():
    r = ref_dir()
    if r is None or not os.path.exists(EXE):
        pytest.skip("reference not staged (oracle/stage_ref.sh) or dym-mod-metro-gpu not built")
    return os.path.join(r, "groups", "mys1080-v4")


def test_reference_driver_output_lines(engine, table):
    out = run([table, 4, 4, 4, 0.0, 1.5, 0.1, 7, 2, 3, 5])
    lines = out.splitlines()
    assert "PARAMS(grp,D,Nt,Nx,beta0,beta1,beta2,seed): " in lines[0]
    assert lines[1] == "RUN(K,N,Ntherm,NHIT): 2 3 5 20"
    assert parse(out).shape == (3, 4 + 16)
    acc = [float(l.split()[1]) for l in lines if l.startswith("ACC:")]
    assert len(acc) == 3 and all(0.0 < x < 1.0 for x in acc)
    assert len(_TM_UPDATE.findall(out)) == 3


def test_reference_driver_statistics(engine, table):
    fix = golden("chains_4x4x4x4_hot_eq.npz")
    ref = np.array([fix[f"series_{s}"].mean(0) for s in fix["seeds"]])
    with ThreadPoolExecutor(6) as ex:
        outs = list(ex.map(lambda s: run([table, 4, 4, 4, 0.0, 1.5, 0.1, s, 10, 100, 3000]), range(7001, 7025)))
    ours = np.array([parse(o).mean(0) for o in outs])
    se = np.sqrt(ref.var(0, ddof=1) / len(ref) + ours.var(0, ddof=1) / len(ours))
    z = (ours.mean(0) - ref.mean(0)) / np.where(se > 0, se, 1)
    p = hotelling_p(ref, ours, (0, 1, 2, 9, 19))
    print("reference driver on the engine: z =", np.round(z, 2).tolist(),
          f"within 1: {np.mean(np.abs(z) < 1):.2f}; Hotelling T^2 p = {p:.3f}")
    assert ours.shape[1] == ref.shape[1] == 4 + 16
    assert np.all(np.abs(z) < 2.0), z
    assert p > 0.01, p


def test_reference_driver_timing(engine, table):
    out = run([table, 4, 8, 32, 0.0, 3.0, -0.15, 20261203, 20, 1, 1, "cold"])
    t = [float(x) for x in _TM_UPDATE.findall(out)]
    assert len(t) == 1
    rate = 32 ** 3 * 8 * 4 * 20 * 20 / t[0]
    print(f"reference driver on the engine, 32^3x8 cold, 20 sweeps in one call: {t[0]:.4f} s, {rate:.3e} link-hits/s")
