"""Statistical parity with the unmodified reference at the benchmark workloads.

The fixtures hold measurement series of the reference's own executable (its
Makefile flags, NHIT 10, its own mys1080-v4, nearest-element pool, hot
starts; tests/golden/make_golden.py):

* chains_4x4x4x4_hot.npz -- the 4^4 run as stated: beta = (0, 1.5, 0.1), Ntherm
  100, K 10, N 100, the full 4 x 4 Wilson grid; 24 runs, one thread each (so
  each run is the reference's serial update order).
* chains_4x4x4x4_hot_eq.npz -- the same couplings after 3,000 thermalisation
  sweeps; 32 runs.  As stated, the 4^4 run ends while the hot start is still
  relaxing: the plaquette falls from -1.6 to -2.91 over the 1,100 sweeps (to
  -2.91 only at the end), so its run means compare two update orders' approach
  to equilibrium (the reference's serial order, the engine's colour phases:
  both valid, not equally fast per sweep) as well as the distribution; with
  3,000 sweeps first both sample the plateau (-2.915), the stationary
  distribution the two must share.
* chains_32x32x32x8_hot.npz -- the single-chain benchmark's lattice, 32^3 x 8, with the Polyakov loop
  and the 8 x 8 Wilson grid, in the disordered phase (beta = (0, 1.0, 0.1);
  Ntherm 20, K 4, N 2); 12 runs with all cores (the reference's OpenMP build).

The engine runs the same protocols on the same table (rebuilt from the
fixtures) with independent seeds, all chains of a protocol as one Batch.
Errors are binned by run: runs from different seeds are independent, so the
error of each side's mean is the spread of its per-run means over
sqrt(runs), whatever the autocorrelation inside a run.  z = (engine -
reference) / combined error, per observable.

The observables of one run are strongly correlated (the Wilson loops of an
ordered 4^4 lattice move together; plaquette and rectangle have correlation
1.0 across runs), so the fraction of |z| below 1 is not a count of
independent trials: it is printed beside the 68% expected, and the joint
test is Hotelling's two-sample T^2 on a well-conditioned subset (ReP, ImP,
plaquette, W[1][1], W[3][3]).

Bars.  The 4^4 runs (20 observables), as stated and in equilibrium: every
|z| < 2 and the T^2 test's p-value above 0.01.  The 32^3 x 8 lattice (68
observables, most of them large Wilson loops that are zero within noise):
with that many comparisons a few beyond 2 are expected by chance
(P(all 68 < 2) ~ 4% for independent ones), so every |z| < 3.5 (a 3%
family-wise rate), at least 85% within 2 and at least half within 1."""
import numpy as np
import pytest

from conftest import golden, hotelling_p

pytestmark = pytest.mark.gpu


def run_engine(engine, ref_table, C, seeds, wl):
    from dym_symanzik_action_gb300.batch import Batch
    g = engine.load_group(ref_table("mys1080-v4"))
    lats = [engine.Lattice(g, C["D"], C["Nt"], C["Nx"], *C["beta"], s, start="hot", pool="nearest",
                           precision="mixed") for s in seeds]
    b = Batch(0)
    for lat in lats:
        b.add(lat)
    b.update(C["Ntherm"], 10)
    series = [[] for _ in lats]
    for n in range(C["N"]):
        b.update(C["K"], 10)
        for k, lat in enumerate(lats):
            m = lat.measure(wl, C["Nt"] if wl == 0 else wl)
            series[k].append([m.poly_re, m.poly_im, m.plaq, m.rect, *m.wloop.ravel()])
    b.close()
    for lat in lats:
        lat.close()
    return np.array([np.mean(s, 0) for s in series])


def zscores(ref, ours):
    se = np.sqrt(ref.var(0, ddof=1) / len(ref) + ours.var(0, ddof=1) / len(ours))
    return (ours.mean(0) - ref.mean(0)) / np.where(se > 0, se, 1)


def params(fix):
    import ast
    return ast.literal_eval(str(fix["params"]).split(" table=")[0])


@pytest.mark.parametrize("fixture,seeds", [("chains_4x4x4x4_hot.npz", range(5001, 5025)),
                                           ("chains_4x4x4x4_hot_eq.npz", range(5101, 5133))],
                         ids=["as-stated", "equilibrium"])
def test_4x4x4x4_within_two_sigma_of_reference(engine, ref_table, fixture, seeds):
    fix = golden(fixture)
    C = params(fix)
    ref = np.array([fix[f"series_{s}"].mean(0) for s in fix["seeds"]])
    ours = run_engine(engine, ref_table, C, seeds, 0)
    z = zscores(ref, ours)
    p = hotelling_p(ref, ours, (0, 1, 2, 9, 19))  # ReP, ImP, plaquette, W[1][1], W[3][3]
    print(f"{fixture}: z = {np.round(z, 2).tolist()}; within 1 sigma {np.mean(np.abs(z) < 1):.2f} "
          f"(68% expected for independent observables); Hotelling T^2 p = {p:.3f}")
    assert ours.shape[1] == ref.shape[1] == 4 + 16
    assert np.all(np.abs(z) < 2.0), z
    assert p > 0.01, p


def test_32x32x32x8_lattice_agrees_with_reference(engine, ref_table):
    fix = golden("chains_32x32x32x8_hot.npz")
    C = params(fix)
    ref = np.array([fix[f"series_{s}"].mean(0) for s in fix["seeds"]])
    ours = run_engine(engine, ref_table, C, range(6001, 6013), C["wl"])
    z = zscores(ref, ours)
    f1, f2 = np.mean(np.abs(z) < 1), np.mean(np.abs(z) < 2)
    print(f"32^3x8: z = {np.round(z, 2).tolist()}; within 1 sigma {f1:.2f}, within 2 sigma {f2:.2f}")
    assert ours.shape[1] == ref.shape[1] == 4 + 64
    assert np.all(np.abs(z) < 3.5), z
    assert f2 >= 0.85 and f1 >= 0.5
