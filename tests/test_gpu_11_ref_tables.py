"""The engine on the reference's own table files.

The reference's shipped tables carry rounding noise in their traces: ReTr is
constant on a conjugacy class only to ~1e-16 (44 distinct doubles for the 11
classes of mys1080-v4).  The mixed kernels take their fast decisions from
class values, with the spread inside their error bound, and re-evaluate the
hits near the threshold on the reference's own elements b s_j, so they must
run on these files (fast_path) and give the reference's configurations bit for
bit.

* mys1080-v4 and myBI are rebuilt from the fixtures (generated table, the
  isomorphism pi, the file's own trace rows) and every sweep is compared with
  the reference's staples and hit loop run on the files themselves
  (ref_tables.npz); once as run, once with DYM_RECHECK_ALL=1, which sends
  every hit through the FP64 re-evaluation; and both again with the
  value-table kernel on every call after the first (DYM_VT_MAX_ACCEPT=1) and
  two lanes per link (DYM_LANES_PER_LINK=2).
* Every shipped table staged in baseline/_ref (or $REF_DIR) -- S(1080), BI,
  BT, BO, S648 (identity at id 4), S108, the SU(4) tables siii_360x4,
  svii_120x4, sviii_120x4 and si_60x4 -- is run by the engine and by the
  reference's own functions compiled from its sources (oracle/_ref), sweep by
  sweep; skipped where the reference is not staged.
* The LLR on the rebuilt mys1080-v4 equals the oracle bit for bit.
"""
import os

import numpy as np
import pytest

from conftest import golden, ref_table_cases, staged_reference
from dym_symanzik_action_gb300.schedule import schedule
from oracle.oracle import REF_LIB, OracleGroup, OracleLattice

pytestmark = pytest.mark.gpu

KERNEL_MIXED, KERNEL_MIXED_VALUES = 3, 4


@pytest.mark.parametrize("lanes", [1, 2], ids=["1lane", "2lanes-vt"])
@pytest.mark.parametrize("recheck_all", [False, True], ids=["fast", "recheck-all"])
@pytest.mark.parametrize("name", list(ref_table_cases().keys()))
def test_fast_kernels_on_reference_files(engine, ref_table, monkeypatch, name, recheck_all, lanes):
    fname, D, Nt, Nx, beta, start, seed, nhit, nsw = ref_table_cases()[name]
    gold = golden("ref_tables.npz")
    if recheck_all:
        monkeypatch.setenv("DYM_RECHECK_ALL", "1")
    if lanes == 2:
        monkeypatch.setenv("DYM_LANES_PER_LINK", "2")
        monkeypatch.setenv("DYM_VT_MAX_ACCEPT", "1.0")
    g = engine.load_group(ref_table(fname))
    assert not g.classes_exact and g.class_spread > 0
    assert g.fast_path
    lat = engine.Lattice(g, D, Nt, Nx, *beta, seed, start=start, precision="mixed")
    assert (lat.links.ravel() == gold[name + "_links"][0]).all()
    kernels = set()
    for s in range(nsw):
        st = lat.update(1, nhit)
        kernels.add(st.kernel)
        assert (st.hits, st.accepts) == tuple(int(x) for x in gold[name + "_counts"][s])
        assert (lat.links.ravel() == gold[name + "_links"][s + 1]).all(), f"sweep {s}"
        if recheck_all:
            assert st.rechecks == st.hits
    assert kernels <= {KERNEL_MIXED, KERNEL_MIXED_VALUES}
    if lanes == 2 and nsw > 1:
        assert KERNEL_MIXED_VALUES in kernels


STAGED = ["mys1080-v4", "myBI", "myBT", "myBO", "S648", "S108", "siii_360x4", "svii_120x4", "sviii_120x4",
          "si_60x4"]


@pytest.mark.parametrize("fname", STAGED)
def test_staged_reference_tables_match_reference_code(engine, fname):
    ref = staged_reference()
    if ref is None or not os.path.exists(REF_LIB):
        pytest.skip("reference not staged (oracle/stage_ref.sh) or oracle/_ref not built")
    from oracle.oracle import RefHarness
    path = os.path.join(ref, "groups", fname)
    g = engine.load_group(path)
    # couplings with a few tenths acceptance for each group's trace range
    b1 = 1.5 if g.min_retr > -3.5 else 1.0
    beta, seed, nhit, nsw = (0.0, b1, 0.1), 4040 + g.P, 10, 3
    h = RefHarness()
    for precision in ("mixed", "fp64"):
        lat = engine.Lattice(g, 4, 4, 4, *beta, seed, start="hot", precision=precision)
        h.init(path, 4, 4, 4)
        h.set_links(lat.links.ravel())
        sched = lat.schedule()
        for s in range(nsw):
            st = lat.update(1, nhit)
            hh, ha = h.sweep(sched, beta, seed, s, 1, nhit)
            assert (st.hits, st.accepts) == (hh, ha), (fname, precision, s)
            assert (lat.links.ravel() == h.get_links()).all(), (fname, precision, s)
        if precision == "mixed" and g.fast_path:
            assert st.kernel in (KERNEL_MIXED, KERNEL_MIXED_VALUES)
        lat.close()


def test_llr_on_reference_file_matches_oracle(engine, ref_table):
    path = ref_table("mys1080-v4")
    D, Nt, Nx, seed = 4, 4, 4, 3
    og = OracleGroup(path)
    L = OracleLattice(og, D, Nt, Nx)
    L.hot_start(seed)
    n = Nt * Nx ** 3 * 6
    kw = dict(ewin=-0.8 * n, hw=0.0225 * n / 2, a0=1.5, axis=1, bg=0.1, K=5, NRM=6, nhit=10, drive_cap=200)
    r = L.llr_run(schedule(D, Nt, Nx), seed=seed, **kw)
    lat = engine.Lattice(engine.load_group(path), D, Nt, Nx, 0.0, 0.0, 0.0, seed, start="hot")
    res = lat.llr_run(**kw)
    assert res.status == r["status"] == "done"
    assert (res.a_hist == r["a_hist"]).all()
    assert (res.hits, res.accepts) == (r["hits"], r["accepts"])
    assert (lat.links.ravel() == L.links).all()
