"""LLR (interval-restricted sweeps + Robbins-Monro, llr.cpp:178-250).

CPU: the oracle's colour-parallel LLR tracks the energies exactly (its
fixed-point class sums equal the reference's plaquette/rectangle loops to
1e-9), drives into the window, and is deterministic.
GPU: dym_llr_run reproduces the oracle bit for bit -- every a_n, the final
energies, the configuration and all counters."""
import numpy as np
import pytest

from dym_symanzik_action_gb300 import tables
from dym_symanzik_action_gb300.schedule import schedule
from oracle.oracle import OracleGroup, OracleLattice

CASES = [
    # name, group, D, Nt, Nx, start, seed, axis, bg, window centre / NPLAQ, a0, K, NRM, nhit, drive_cap
    ("s1080_4444_drive", "S1080", 4, 4, 4, "hot", 3, 1, 0.1, -0.8, 1.5, 5, 6, 10, 200),
    ("s1080_2444_cold", "S1080", 4, 2, 4, "cold", 8, 1, -0.1, -2.5, 3.0, 4, 5, 10, 200),
    ("bi_4444_axis2", "BI", 4, 4, 4, "hot", 5, 2, 1.0, -0.5, 1.0, 4, 4, 10, 200),
    ("s1080_4444_unreached", "S1080", 4, 4, 4, "hot", 9, 1, 0.0, -2.9, 0.0, 3, 3, 5, 2),
]


def nplaq(D, Nt, Nx):
    return Nt * Nx ** (D - 1) * D * (D - 1) // 2


def run_oracle(case):
    name, gname, D, Nt, Nx, start, seed, axis, bg, cen, a0, K, NRM, nhit, cap = case
    og = OracleGroup(tables.ensure_table(gname))
    L = OracleLattice(og, D, Nt, Nx)
    if start == "hot":
        L.hot_start(seed)
    n = nplaq(D, Nt, Nx) * (1 if axis == 1 else 2)
    r = L.llr_run(schedule(D, Nt, Nx), ewin=cen * n, hw=0.0225 * n / 2, a0=a0, axis=axis, bg=bg, K=K, NRM=NRM,
                  nhit=nhit, drive_cap=cap, seed=seed)
    return L, r


@pytest.mark.parametrize("case", CASES[:3], ids=[c[0] for c in CASES[:3]])
def test_oracle_llr_tracks_energy_exactly(case):
    L, r = run_oracle(case)
    s1, s2 = L.energies()
    assert abs(r["S1"] - s1) < 1e-9 * max(1, abs(s1)) and abs(r["S2"] - s2) < 1e-9 * max(1, abs(s2))
    assert r["status"] == "done"
    assert np.all(np.isfinite(r["a_hist"]))
    L2, r2 = run_oracle(case)
    assert (L2.links == L.links).all() and (r2["a_hist"] == r["a_hist"]).all()


def test_oracle_llr_unreachable_window():
    L, r = run_oracle(CASES[3])
    assert r["status"] == "unreached" and r["drive_sweeps"] == 2
