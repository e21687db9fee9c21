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


@pytest.mark.parametrize("kernel", ["values", "values-2-lanes", "elements", "fp64-shared", "fp64-direct",
                                    "fp64-direct-3d"])
def test_final_sweep_writes_pinned_output(engine, monkeypatch, kernel):
    """A page-locked host_out (and a page-locked reference array) is written by
    the final sweep itself, every link once: the result equals dym_sweep +
    dym_links_get for each sweep kernel, with host_out aliasing host_in too."""
    torch = pytest.importorskip("torch")
    monkeypatch.setenv("DYM_VT_MAX_ACCEPT", "2.0" if kernel.startswith("values") else "-1")
    monkeypatch.setenv("DYM_LANES_PER_LINK", "2" if kernel == "values-2-lanes" else "1")
    D, precision, want_kernel = 4, "mixed", {"values": 4, "values-2-lanes": 4, "elements": 3}.get(kernel)
    if kernel == "fp64-shared":
        precision, want_kernel = "shared", 2
    if kernel.startswith("fp64-direct"):
        precision, want_kernel = "fp64", 1
        D = 3 if kernel.endswith("3d") else 4
    g = engine.load_group(tables.ensure_table("S1080"))
    mk = lambda: engine.Lattice(g, D, 4, 8, 0.0, 2.0, -0.1, 77, start="hot", precision=precision)  # noqa: E731
    ref, ours, arr = mk(), mk(), mk()
    n = ref.D * ref.V
    buf = pinned(n)
    ref_arr = torch.empty(n, dtype=torch.int32, pin_memory=True).numpy()
    cfg = ref.links.ravel().copy()
    for step in range(3):
        sr = ref.update(2, 10)
        buf[:] = cfg
        so = ours.update_host(buf, buf, 2, 10)
        ref_arr[:] = to_ref(cfg, D)
        sa = arr.update_refarray(ref_arr, 2, 10)
        want = ref.links.ravel()
        assert so.kernel == sa.kernel == sr.kernel == want_kernel, (step, so.kernel, sr.kernel)
        assert (so.hits, so.accepts) == (sa.hits, sa.accepts) == (sr.hits, sr.accepts), step
        assert np.array_equal(buf, want), step
        assert np.array_equal(ref_arr, to_ref(want, D)), step
        cfg = want.copy()


def test_refused_upload_pinned_buffers(engine):
    """With page-locked buffers a refused upload still leaves host_out holding
    the chain's unchanged configuration and the reference array untouched."""
    torch = pytest.importorskip("torch")
    b = chain(engine, "mixed", seed=41)
    b.update(1, 10)
    before = b.links.ravel().copy()
    n = before.size
    hin, hout = pinned(n), pinned(n)
    hin[:] = before
    hin[999] = 1080
    hout[:] = 0
    st = _lib.Stats()
    rc = lib().dym_sweep_host(b._h, ptr(hin, C.c_uint16), ptr(hout, C.c_uint16), 2, 10, C.byref(st))
    assert _lib.ERRORS.get(rc) == "DYM_EINVAL" and b"at 999" in lib().dym_last_error()
    assert np.array_equal(hout, before) and np.array_equal(b.links.ravel(), before)
    ref = torch.empty(n, dtype=torch.int32, pin_memory=True).numpy()
    ref[:] = to_ref(before, b.D)
    ref[5] = -3
    keep = ref.copy()
    rc = lib().dym_sweep_refarray(b._h, ptr(ref, C.c_int32), 2, 10, C.byref(st))
    assert _lib.ERRORS.get(rc) == "DYM_EINVAL" and b"a[5]" in lib().dym_last_error()
    assert np.array_equal(ref, keep) and np.array_equal(b.links.ravel(), before)
    assert b.update(1, 10).sweep == 2
