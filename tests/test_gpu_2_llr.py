"""Device LLR (dym_llr_run) against the oracle's LLR restatement, bit for bit:
every a_n, the final energies, the configuration and all counters."""
import numpy as np
import pytest

from dym_symanzik_action_gb300 import tables
from test_llr import CASES, nplaq, run_oracle

@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_gpu_llr_matches_oracle(engine, case):
    name, gname, D, Nt, Nx, start, seed, axis, bg, cen, a0, K, NRM, nhit, cap = case
    L, r = run_oracle(case)
    g = engine.load_group(tables.ensure_table(gname))
    lat = engine.Lattice(g, D, Nt, Nx, 0.0, 0.0, 0.0, seed, start=start)
    n = nplaq(D, Nt, Nx) * (1 if axis == 1 else 2)
    res = lat.llr_run(ewin=cen * n, hw=0.0225 * n / 2, a0=a0, axis=axis, bg=bg, K=K, NRM=NRM, nhit=nhit,
                      drive_cap=cap)
    np.testing.assert_allclose(res.a_hist, r["a_hist"], rtol=1e-6, atol=0)
    assert (res.a_hist == r["a_hist"]).all()  # in fact identical
    assert res.status == r["status"]
    assert (res.drive_sweeps, res.sweeps) == (r["drive_sweeps"], r["sweeps"])
    assert (res.hits, res.accepts) == (r["hits"], r["accepts"])
    assert (res.phase_accepts, res.phase_rejects) == (r["phase_accepts"], r["phase_rejects"])
    assert res.S1 == r["S1"] and res.S2 == r["S2"]
    assert (lat.links.ravel() == L.links).all()
    # The tracked energies are fixed-point class sums (class values rounded to
    # 2^-32): within half a unit per term of the FP64 recount.
    s1, s2 = lat.llr_energy()
    n1 = nplaq(D, Nt, Nx)
    assert abs(s1 - res.S1) <= n1 * 2.0 ** -33 and abs(s2 - res.S2) <= 2 * n1 * 2.0 ** -33


CASES_2D = [
    # name, group, Nt, Nx, start, seed, S1 centre / NPLAQ, S2 centre / NRECT, a1, a2, K, NRM, nhit, cap
    ("s1080_4444_2d_cold", "S1080", 4, 4, "cold", 8, -2.5, -2.2, 3.0, 0.5, 4, 5, 10, 300),
    ("bi_4444_2d_hot", "BI", 4, 4, "hot", 5, -0.6, -0.4, 1.0, 0.5, 4, 5, 10, 300),
    ("s1080_3444_2d_hot", "S1080", 3, 4, "hot", 11, -1.0, -0.7, 2.0, 0.0, 4, 5, 10, 300),
]


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES_2D, ids=[c[0] for c in CASES_2D])
def test_gpu_llr2d_matches_oracle(engine, case):
    from dym_symanzik_action_gb300.schedule import schedule
    from oracle.oracle import OracleGroup, OracleLattice
    name, gname, Nt, Nx, start, seed, c1, c2, a1, a2, K, NRM, nhit, cap = case
    og = OracleGroup(tables.ensure_table(gname))
    L = OracleLattice(og, 4, Nt, Nx)
    if start == "hot":
        L.hot_start(seed)
    else:
        L.links = np.full(4 * L.V, og.id, np.uint16)
    n1 = L.V * 6
    cell = (c1 * n1, 0.0225 * n1 / 2, c2 * 2 * n1, 0.0225 * 2 * n1 / 2)
    r = L.llr2d_run(schedule(4, Nt, Nx), *cell, a1, a2, K=K, NRM=NRM, nhit=nhit, drive_cap=cap, seed=seed)
    g = engine.load_group(tables.ensure_table(gname))
    lat = engine.Lattice(g, 4, Nt, Nx, 0.0, 0.0, 0.0, seed, start=start)
    res = lat.llr2d_run(*cell, a1, a2, K=K, NRM=NRM, nhit=nhit, drive_cap=cap)
    assert res.status == r["status"] == "done"
    assert (res.a_hist == r["a_hist"]).all()
    assert (res.a1, res.a2, res.S1, res.S2) == (r["a1"], r["a2"], r["S1"], r["S2"])
    assert (res.drive_sweeps, res.sweeps, res.hits, res.accepts) == (r["drive_sweeps"], r["sweeps"], r["hits"],
                                                                     r["accepts"])
    assert (res.phase_accepts, res.phase_rejects) == (r["phase_accepts"], r["phase_rejects"])
    assert (lat.links.ravel() == L.links).all()
