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
    s1, s2 = lat.llr_energy()
    assert s1 == res.S1 and s2 == res.S2
