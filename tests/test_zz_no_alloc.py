"""dym_measure_noalloc (fixed device scratch, no allocation) against dym_measure,
both called through the C ABI.

Both count every loop in exact integer histograms and then take the same FP64
dot products (correctly rounded multiplies and adds, then one division) in
the same order, so the observables must be identical, bit for bit.  Two
calls in a row check that the shared scratch is cleared between calls; a
sweep between calls checks that it follows the configuration.  On a fresh
chain whose first measurement is the no-allocation call, the device's free
memory is unchanged across the calls.  This file is collected last so that
it also runs after the other GPU tests have used the device."""
import ctypes as C

import numpy as np
import pytest

from dym_symanzik_action_gb300 import _lib, tables
from dym_symanzik_action_gb300._lib import check, lib, ptr

pytestmark = pytest.mark.gpu

CASES = {
    # group, D, Nt, Nx, betas, start, seed, (wl_nx, wl_nt)
    "s1080_8x4_full": ("S1080", 4, 4, 8, (0.0, 1.5, 0.1), "hot", 11, (0, 0)),
    "s1080_8x4_2x3": ("S1080", 4, 4, 8, (0.0, 3.0, -0.15), "cold", 12, (2, 3)),
    "s1080_nogrid": ("S1080", 4, 4, 4, (0.0, 1.5, 0.1), "hot", 13, (-1, -1)),
    "bi_6x4_full": ("BI", 4, 4, 6, (0.0, 2.0, -0.1), "hot", 14, (0, 0)),
}


def measure_via(fn_name, lat, wl_nx, wl_nt):
    nx = lat.Nx if wl_nx == 0 else max(wl_nx, 0)
    nt = lat.Nt if wl_nt == 0 else max(wl_nt, 0)
    if wl_nx < 0 or wl_nt < 0:
        nx = nt = 0
    w = np.full(max(nx * nt, 1), np.nan)
    o = _lib.Obs()
    opts = _lib.MeasOpts(wl_nx=wl_nx, wl_nt=wl_nt)
    check(getattr(lib(), fn_name)(lat._h, C.byref(opts), C.byref(o), ptr(w, C.c_double)))
    return np.array([o.plaq, o.rect, o.poly_re, o.poly_im]), (o.wl_nx, o.wl_nt), w[: nx * nt]


def assert_same(a, b):
    (ha, ga, wa), (hb, gb, wb) = a, b
    assert ga == gb
    np.testing.assert_array_equal(ha, hb)
    np.testing.assert_array_equal(wa, wb)


@pytest.mark.parametrize("name", list(CASES))
def test_noalloc_matches_measure(engine, name):
    gname, D, Nt, Nx, beta, start, seed, (wx, wt) = CASES[name]
    g = engine.load_group(tables.ensure_table(gname))
    lat = engine.Lattice(g, D, Nt, Nx, *beta, seed, start=start)
    lat.update(3, 10)
    ref = measure_via("dym_measure", lat, wx, wt)
    first = measure_via("dym_measure_noalloc", lat, wx, wt)
    second = measure_via("dym_measure_noalloc", lat, wx, wt)
    assert_same(first, ref)
    assert_same(second, ref)
    lat.update(2, 10)
    ref2 = measure_via("dym_measure", lat, wx, wt)
    third = measure_via("dym_measure_noalloc", lat, wx, wt)
    assert_same(third, ref2)
    if start == "hot":
        assert not np.array_equal(ref[0], ref2[0])  # the configuration moved
    lat.close()


@pytest.mark.parametrize("grid", [(12, 10), (40, 40)])
def test_noalloc_rejects_oversize(engine, grid):
    g = engine.load_group(tables.ensure_table("S1080"))
    lat = engine.Lattice(g, 4, 4, 4, 0.0, 1.5, 0.1, 5)
    o = _lib.Obs()
    opts = _lib.MeasOpts(wl_nx=grid[0], wl_nt=grid[1])
    w = np.zeros(grid[0] * grid[1])
    rc = lib().dym_measure_noalloc(lat._h, C.byref(opts), C.byref(o), ptr(w, C.c_double))
    assert rc == -8  # DYM_ERANGE
    msg = lib().dym_last_error().decode()
    assert "dym_measure_noalloc" in msg and ("fixed scratch" in msg or "fixed result area" in msg)
    # the chain stays usable
    h, gr, _ = measure_via("dym_measure_noalloc", lat, 2, 2)
    assert gr == (2, 2) and np.isfinite(h).all()
    lat.close()


def test_noalloc_allocates_nothing_on_a_fresh_chain(engine):
    """The first measurement of a new chain through dym_measure_noalloc: the
    device's free memory (cudaMemGetInfo) is the same before and after two
    calls, and the results equal dym_measure's taken afterwards."""
    torch = pytest.importorskip("torch")
    g = engine.load_group(tables.ensure_table("S1080"))
    warm = engine.Lattice(g, 4, 4, 4, 0.0, 1.5, 0.1, 21)
    measure_via("dym_measure_noalloc", warm, 2, 2)  # the device's array is looked up (device code loaded)
    lat = engine.Lattice(g, 4, 4, 8, 0.0, 1.5, 0.1, 22, start="hot")
    lat.update(2, 10)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(0)[0]
    first = measure_via("dym_measure_noalloc", lat, 4, 4)
    second = measure_via("dym_measure_noalloc", lat, 4, 4)
    free1 = torch.cuda.mem_get_info(0)[0]
    assert free1 == free0, (free0, free1)
    ref = measure_via("dym_measure", lat, 4, 4)  # allocates the chain's histogram buffers now
    assert_same(first, ref)
    assert_same(second, ref)
    lat.close()
    warm.close()
