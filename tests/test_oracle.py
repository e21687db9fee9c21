"""The oracle (oracle/dym_oracle.c) against the reference's own code: every
golden fixture was produced by the reference's get_staples/get_rect_loops/
plaquette/wilson/getpoly compiled from its sources (tests/golden/make_golden.py),
and the oracle must reproduce it -- bit-exact for link configurations and
counts, to 1e-12 for observables (the fixture sums in site order, the oracle
through element histograms)."""
import math

import numpy as np
import pytest

from conftest import golden, sweep_cases
from dym_symanzik_action_gb300 import tables
from oracle.oracle import OracleGroup, OracleLattice, lib


def test_philox_known_answers():
    # Known-answer vectors of Philox4x32-10 published with Random123.
    kats = [
        ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
        ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
        ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
         [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
    ]
    import ctypes as C
    for ctr, key, want in kats:
        c = np.array(ctr, np.uint32)
        k = np.array(key, np.uint32)
        o = np.zeros(4, np.uint32)
        P = C.POINTER(C.c_uint32)
        lib().or_philox(c.ctypes.data_as(P), k.ctypes.data_as(P), o.ctypes.data_as(P))
        assert o.tolist() == want


def test_exp_within_two_ulp_of_libm():
    rng = np.random.default_rng(3)
    xs = np.concatenate([-rng.exponential(3.0, 20000), -rng.uniform(0, 740, 2000), [0.0, -1e-300, -708.5, -745.0]])
    worst = 0
    for x in xs:
        a, b = lib().or_exp(float(x)), math.exp(float(x))
        if b == 0.0:
            assert a < 5e-324 * 4
            continue
        worst = max(worst, abs(a - b) / math.ulp(b))
    assert worst <= 2.0


def test_pick_equals_truncated_product():
    rng = np.random.default_rng(4)
    for r0 in rng.integers(0, 2**32, 5000, dtype=np.uint64):
        for n in (12, 72, 1080, 5040):
            assert lib().or_pick(int(r0), n) == int(n * (float(r0) * 2.0**-32))


def test_staples_match_reference():
    g = golden("staples.npz")
    og = OracleGroup(tables.ensure_table("S1080"))
    L = OracleLattice(og, 4, 4, 4)
    L.links = g["links"]
    for d in range(4):
        for i in range(L.V):
            st, re = L.staples(i, d)
            assert (np.concatenate([st, re]) == g["staples"][d, i]).all(), (d, i)


@pytest.mark.parametrize("name", list(sweep_cases().keys()))
def test_sweeps_match_reference(name, sweeps_golden):
    gname, D, Nt, Nx, beta, start, seed, nhit, pool_all, nsw, wx, wt = sweep_cases()[name]
    gold = sweeps_golden
    sched = (gold[name + "_sched_dir"], gold[name + "_sched_len"], gold[name + "_sched_sites"])
    og = OracleGroup(tables.ensure_table(gname))
    L = OracleLattice(og, D, Nt, Nx)
    if start == "hot":
        L.hot_start(seed)
    assert (L.links == gold[name + "_links"][0]).all()
    for s in range(nsw):
        h, a = L.sweep(sched, beta, seed, s, 1, nhit, pool_all, nthreads=2)
        assert (h, a) == tuple(int(x) for x in gold[name + "_counts"][s])
        assert (L.links == gold[name + "_links"][s + 1]).all(), f"sweep {s}"
        obs = L.measure(wx, wt)
        np.testing.assert_allclose(obs, gold[name + "_obs"][s], rtol=0, atol=1e-12)


def test_oracle_threads_deterministic():
    og = OracleGroup(tables.ensure_table("S1080"))
    from dym_symanzik_action_gb300.schedule import schedule
    sched = schedule(4, 4, 4)
    out = []
    for nt in (1, 4):
        L = OracleLattice(og, 4, 4, 4)
        L.hot_start(5)
        L.sweep(sched, (0, 1.5, 0.1), 5, 0, 2, 10, nthreads=nt)
        out.append(L.links)
    assert (out[0] == out[1]).all()


@pytest.mark.parametrize("name", list(__import__("conftest").ref_table_cases().keys()))
def test_oracle_on_reference_files(name, ref_table):
    """The oracle on the reference's own table files (ReTr with rounding noise
    inside a class), rebuilt from the fixtures, reproduces the reference's
    staples and hit loop run on the files themselves."""
    from conftest import ref_table_cases
    from dym_symanzik_action_gb300.schedule import schedule
    fname, D, Nt, Nx, beta, start, seed, nhit, nsw = ref_table_cases()[name]
    gold = golden("ref_tables.npz")
    og = OracleGroup(ref_table(fname))
    L = OracleLattice(og, D, Nt, Nx)
    if start == "hot":
        L.hot_start(seed)
    assert (L.links == gold[name + "_links"][0]).all()
    sched = schedule(D, Nt, Nx)
    for s in range(nsw):
        h, a = L.sweep(sched, beta, seed, s, 1, nhit, False, nthreads=2)
        assert (h, a) == tuple(int(x) for x in gold[name + "_counts"][s])
        assert (L.links == gold[name + "_links"][s + 1]).all(), f"sweep {s}"
