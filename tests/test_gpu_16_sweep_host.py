"""dym_sweep_host: sweeps of a configuration held in host memory in one call
(upload and check, sweeps, read-back, one synchronisation) -- the same
configurations and counters as dym_links_set + dym_sweep + dym_links_get, for
pageable and page-locked buffers, with host_out aliasing host_in, and with
either buffer absent; a refused upload (an id >= the group order) leaves the
chain and its sweep counter as they were.  dym_sweep_refarray: the same on
an array in the reference's own layout (int32, a[i*D + d]), updated in place,
and left untouched when refused."""
import ctypes as C

import numpy as np
import pytest

from dym_symanzik_action_gb300 import _lib, tables
from dym_symanzik_action_gb300._lib import lib, ptr

pytestmark = pytest.mark.gpu


def pinned(n):
    torch = pytest.importorskip("torch")
    return torch.empty(n, dtype=torch.uint16, pin_memory=True).numpy()


def chain(engine, precision, seed=5, start="hot", beta=(0.0, 2.0, -0.1)):
    g = engine.load_group(tables.ensure_table("S1080"))
    return engine.Lattice(g, 4, 4, 8, *beta, seed, start=start, precision=precision)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("buffers", ["pageable", "pinned", "aliased"])
def test_sweep_host_equals_set_sweep_get(engine, precision, buffers):
    ref = chain(engine, precision)
    ours = chain(engine, precision, seed=5)
    n = ref.D * ref.V
    rng = np.random.default_rng(3)
    cfg = rng.integers(0, 1080, n).astype(np.uint16)
    if buffers == "pageable":
        hin, hout = cfg.copy(), np.zeros(n, np.uint16)
    elif buffers == "pinned":
        hin, hout = pinned(n), pinned(n)
        hin[:] = cfg
    else:
        hin = pinned(n)
        hin[:] = cfg
        hout = hin
    for step in range(3):
        ref.links = cfg
        sr = ref.update(2, 10)
        want = ref.links.ravel()
        if buffers == "aliased":
            hin[:] = cfg
        so = ours.update_host(hin, hout, 2, 10)
        assert (so.hits, so.accepts, so.rechecks, so.sweep, so.kernel) == \
            (sr.hits, sr.accepts, sr.rechecks, sr.sweep, sr.kernel), step
        assert np.array_equal(hout, want), step
        assert np.array_equal(ours.links.ravel(), want), step
        cfg = want.copy()
        if buffers != "aliased":
            hin[:] = cfg


def test_sweep_host_without_buffers(engine):
    a = chain(engine, "mixed", seed=9)
    b = chain(engine, "mixed", seed=9)
    a.update(3, 10)
    sb = b.update_host(None, None, 3, 10)
    assert sb.sweep == 3
    assert np.array_equal(a.links, b.links)
    out = np.zeros(a.D * a.V, np.uint16)
    a.update(1, 10)
    b.update_host(None, out, 1, 10)
    assert np.array_equal(out, a.links.ravel())


def test_sweep_host_refused_upload_leaves_chain_unchanged(engine):
    a = chain(engine, "mixed", seed=11)
    b = chain(engine, "mixed", seed=11)
    a.update(1, 10)
    b.update(1, 10)
    before = b.links.ravel().copy()
    bad = before.copy()
    bad[12345 % bad.size] = 1080  # out of range for S(1080)
    out = np.zeros_like(bad)
    st = _lib.Stats()
    rc = lib().dym_sweep_host(b._h, ptr(bad, C.c_uint16), ptr(out, C.c_uint16), 2, 10, C.byref(st))
    assert _lib.ERRORS.get(rc) == "DYM_EINVAL"
    assert b"out of range" in lib().dym_last_error()
    assert np.array_equal(b.links.ravel(), before)
    assert np.array_equal(out, before)
    # the refused call advanced nothing: both chains continue identically
    sa = a.update(2, 10)
    sb = b.update(2, 10)
    assert (sa.sweep, sa.hits, sa.accepts) == (sb.sweep, sb.hits, sb.accepts) and sb.sweep == 3
    assert np.array_equal(a.links, b.links)


def to_ref(links, D):
    """Direction-major [D][V] ids -> the reference's a[i*D + d] (int32)."""
    return np.ascontiguousarray(np.asarray(links).reshape(D, -1).T, np.int32).ravel()


@pytest.mark.parametrize("buffers", ["pageable", "pinned"])
def test_refarray_equals_sweep_host(engine, buffers):
    """dym_sweep_refarray on the reference's own layout (int32, site-major,
    updated in place) gives the configurations and counters of
    dym_sweep_host on the same configuration."""
    a_chain = chain(engine, "mixed", seed=21)
    r_chain = chain(engine, "mixed", seed=21)
    n = a_chain.D * a_chain.V
    cfg = np.random.default_rng(8).integers(0, 1080, n).astype(np.uint16)
    if buffers == "pinned":
        torch = pytest.importorskip("torch")
        ref = torch.empty(n, dtype=torch.int32, pin_memory=True).numpy()
    else:
        ref = np.zeros(n, np.int32)
    ref[:] = to_ref(cfg, a_chain.D)
    out = np.zeros(n, np.uint16)
    for step in range(3):
        sa = a_chain.update_host(cfg, out, 2, 10)
        sr = r_chain.update_refarray(ref, 2, 10)
        assert (sr.hits, sr.accepts, sr.rechecks, sr.sweep, sr.kernel) == \
            (sa.hits, sa.accepts, sa.rechecks, sa.sweep, sa.kernel), step
        assert np.array_equal(ref, to_ref(out, a_chain.D)), step
        cfg = out.copy()


@pytest.mark.parametrize("bad", [1080, -1])
def test_refarray_refused_leaves_array_and_chain(engine, bad):
    a = chain(engine, "mixed", seed=31)
    b = chain(engine, "mixed", seed=31)
    ref = to_ref(b.links.ravel(), b.D)
    ref[777] = bad
    keep = ref.copy()
    st = _lib.Stats()
    rc = lib().dym_sweep_refarray(b._h, ptr(ref, C.c_int32), 2, 10, C.byref(st))
    assert _lib.ERRORS.get(rc) == "DYM_EINVAL"
    assert b"a[777]" in lib().dym_last_error()
    assert np.array_equal(ref, keep)
    sa, sb = a.update(1, 10), b.update(1, 10)
    assert (sa.sweep, sa.hits, sa.accepts) == (sb.sweep, sb.hits, sb.accepts) and sb.sweep == 1
    assert np.array_equal(a.links, b.links)
