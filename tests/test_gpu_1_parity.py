"""GPU parity: the CUDA sweep and observables against the reference fixtures
and the oracle.

Bar: link configurations and hit/accept counts bit-exact after every sweep;
observables bit-exact against the oracle's histogram sums and within 1e-12
of the reference's site-order sums.  All three accept paths are covered:
fp64 (direct kernel, every decision as the reference), shared (FP64
decisions with the shared sub-table) and mixed (exact fixed-point dS with an
FP32 threshold test and FP64 re-evaluation near the threshold); all must give
identical configurations."""
import numpy as np
import pytest

from conftest import golden, sweep_cases
from dym_symanzik_action_gb300 import tables
from dym_symanzik_action_gb300.schedule import schedule
from oracle.oracle import OracleGroup, OracleLattice

pytestmark = pytest.mark.gpu

_groups = {}


def group(engine, name):
    if name not in _groups:
        _groups[name] = engine.load_group(tables.ensure_table(name))
    return _groups[name]


def test_staples_match_reference(engine):
    g = golden("staples.npz")
    lat = engine.Lattice(group(engine, "S1080"), 4, 4, 4, 0, 1.5, 0.1, 1)
    lat.links = g["links"].reshape(4, -1)
    for d in range(4):
        st = lat.staples(d, np.arange(lat.V))
        assert (st == g["staples"][d]).all(), d


@pytest.mark.parametrize("precision", ["fp64", "shared", "mixed"])
@pytest.mark.parametrize("name", list(sweep_cases().keys()))
def test_sweeps_match_reference(engine, sweeps_golden, name, precision):
    gname, D, Nt, Nx, beta, start, seed, nhit, pool_all, nsw, wx, wt = sweep_cases()[name]
    gold = sweeps_golden
    lat = engine.Lattice(group(engine, gname), D, Nt, Nx, *beta, seed, start=start,
                         pool="all" if pool_all else "nearest", precision=precision)
    pd, pl, sites = lat.schedule()
    assert (pd == gold[name + "_sched_dir"]).all() and (pl == gold[name + "_sched_len"]).all()
    assert (sites == gold[name + "_sched_sites"]).all()
    assert (lat.links.ravel() == gold[name + "_links"][0]).all()
    og = OracleGroup(tables.ensure_table(gname))
    ol = OracleLattice(og, D, Nt, Nx)
    for s in range(nsw):
        st = lat.update(1, nhit)
        assert (st.hits, st.accepts) == tuple(int(x) for x in gold[name + "_counts"][s])
        assert (lat.links.ravel() == gold[name + "_links"][s + 1]).all(), f"sweep {s}"
        m = lat.measure(wx, wt)
        got = np.concatenate([[m.poly_re, m.poly_im, m.plaq, m.rect], m.wloop.ravel()])
        np.testing.assert_allclose(got, gold[name + "_obs"][s], rtol=0, atol=1e-12)
        ol.links = lat.links.ravel()
        assert (got == ol.measure(wx, wt)).all()


CASES = [
    # group, D, Nt, Nx, beta, start, pool, nhit, sweeps
    ("S1080", 4, 8, 8, (0.0, 1.5, 0.1), "hot", "nearest", 10, 2),
    ("S1080", 4, 8, 8, (0.0, 3.0, -0.15), "cold", "nearest", 10, 3),
    ("S1080", 4, 12, 8, (0.2, 2.0, -0.1), "hot", "all", 7, 2),
    ("BI", 4, 6, 6, (0.0, 3.0, 0.2), "hot", "nearest", 20, 2),
    ("BI", 4, 2, 12, (0.0, 1.0, -0.3), "hot", "nearest", 10, 2),
    ("BT", 3, 5, 5, (0.0, 2.0, 0.5), "hot", "nearest", 10, 2),
]


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-D{c[1]}-{c[2]}x{c[3]}-{c[5]}-{c[6]}" for c in CASES])
def test_random_configs_match_oracle(engine, case):
    gname, D, Nt, Nx, beta, start, pool, nhit, nsw = case
    seed = 1000 + Nt * 7 + Nx
    og = OracleGroup(tables.ensure_table(gname))
    sched = schedule(D, Nt, Nx)
    for precision in ("fp64", "shared", "mixed"):
        lat = engine.Lattice(group(engine, gname), D, Nt, Nx, *beta, seed, start=start, pool=pool,
                             precision=precision)
        ol = OracleLattice(og, D, Nt, Nx)
        ol.links = lat.links.ravel()
        for s in range(nsw):
            st = lat.update(1, nhit)
            h, a = ol.sweep(sched, beta, seed, s, 1, nhit, pool == "all")
            assert (st.hits, st.accepts) == (h, a)
            assert (lat.links.ravel() == ol.links).all(), (precision, s)


def test_full_size_cold_chain_matches_oracle(engine):
    """32^3 x 8 (1,048,576 links), cold start at beta = (0, 3, -0.15), NHIT 10:
    two sweeps bit-exact against the oracle, all three accept paths."""
    D, Nt, Nx, beta, nhit = 4, 8, 32, (0.0, 3.0, -0.15), 10
    og = OracleGroup(tables.ensure_table("S1080"))
    sched = schedule(D, Nt, Nx)
    ol = OracleLattice(og, D, Nt, Nx)
    res = {}
    for precision in ("mixed", "shared", "fp64"):
        lat = engine.Lattice(group(engine, "S1080"), D, Nt, Nx, *beta, 20261203, start="cold", precision=precision)
        st = lat.update(2, nhit)
        assert st.hits == lat.V * D * nhit * 2
        res[precision] = (lat.links.ravel(), st.accepts)
    for p in ("mixed", "shared"):
        assert (res[p][0] == res["fp64"][0]).all() and res[p][1] == res["fp64"][1], p
    h, a = ol.sweep(sched, beta, 20261203, 0, 2, nhit)
    assert a == res["fp64"][1]
    assert (ol.links == res["fp64"][0]).all()


def test_full_size_hot_chain_matches_oracle(engine):
    D, Nt, Nx, beta, nhit = 4, 8, 32, (0.0, 3.0, -0.15), 10
    og = OracleGroup(tables.ensure_table("S1080"))
    lat = engine.Lattice(group(engine, "S1080"), D, Nt, Nx, *beta, 77, start="hot", precision="mixed")
    ol = OracleLattice(og, D, Nt, Nx)
    ol.hot_start(77)
    assert (ol.links == lat.links.ravel()).all()
    st = lat.update(1, nhit)
    h, a = ol.sweep(schedule(D, Nt, Nx), beta, 77, 0, 1, nhit)
    assert (st.hits, st.accepts) == (h, a)
    assert (ol.links == lat.links.ravel()).all()
    m = lat.measure(4, 4)
    ol_obs = ol.measure(4, 4)
    got = np.concatenate([[m.poly_re, m.poly_im, m.plaq, m.rect], m.wloop.ravel()])
    assert (got == ol_obs).all()


def test_shared_table_path_is_selected_for_generated_tables(engine):
    for name in ("S1080", "BI", "BT"):
        assert group(engine, name).fast_path, name


def test_mixed_precision_reports_rechecks(engine):
    """Hot S(1080) 8^4 at beta = (0, 2, -0.1): the mixed kernel re-evaluates a
    small fraction of hits in FP64, reports the largest |dS_fast - dS_fp64|
    seen there (below its bound), and gives the fp64 kernel's configuration."""
    D, Nt, Nx, beta, nhit = 4, 8, 8, (0.0, 2.0, -0.1), 10
    res = {}
    for precision in ("mixed", "fp64"):
        lat = engine.Lattice(group(engine, "S1080"), D, Nt, Nx, *beta, 4242, start="hot", precision=precision)
        st = lat.update(5, nhit)
        res[precision] = (lat.links.ravel(), st)
    (lm, sm), (lf, sf) = res["mixed"], res["fp64"]
    assert (lm == lf).all() and sm.accepts == sf.accepts
    assert sf.rechecks == 0
    assert 0 < sm.rechecks < 1e-3 * sm.hits
    assert 0.0 <= sm.max_ds_err < 1e-3


def test_value_table_kernel_takes_over_when_moves_are_rare(engine):
    """Cold S(1080) 8^4 at beta = (0, 3, -0.15): almost nothing is accepted, so
    after its first call the mixed chain runs the value-table kernel
    (DYM_KERNEL_MIXED_VALUES = 4); every configuration equals the FP64 kernel's.
    A hot chain at beta1 = 1 keeps the element-table kernel (3)."""
    D, Nt, Nx, beta, nhit = 4, 8, 8, (0.0, 3.0, -0.15), 10
    lm = engine.Lattice(group(engine, "S1080"), D, Nt, Nx, *beta, 31, start="cold", precision="mixed")
    lf = engine.Lattice(group(engine, "S1080"), D, Nt, Nx, *beta, 31, start="cold", precision="fp64")
    kernels = []
    for call in range(4):
        sm = lm.update(2, nhit)
        sf = lf.update(2, nhit)
        kernels.append(sm.kernel)
        assert sf.kernel == 1
        assert sm.accepts == sf.accepts and (lm.links == lf.links).all(), call
    assert kernels[0] == 3 and kernels[1:] == [4, 4, 4]
    lh = engine.Lattice(group(engine, "S1080"), D, Nt, Nx, 0.0, 1.0, 0.0, 32, start="hot", precision="mixed")
    assert [lh.update(1, nhit).kernel for _ in range(3)] == [3, 3, 3]


def test_links_set_rejects_out_of_range_ids(engine):
    """dym_links_set refuses an element id >= P, names the first bad index and
    leaves the chain's configuration as it was."""
    from dym_symanzik_action_gb300._lib import DymError
    lat = engine.Lattice(group(engine, "BT"), 4, 4, 4, 0.0, 1.0, 0.0, 3, start="hot")
    before = lat.links.copy()
    bad = before.copy().ravel()
    bad[777] = lat.group.P
    bad[900] = 0xFFFF
    with pytest.raises(DymError, match="at 777$"):
        lat.links = bad
    assert (lat.links == before).all()
    good = np.roll(before.ravel(), 5)
    lat.links = good
    assert (lat.links.ravel() == good).all()


def test_links_transfer_page_locked(engine):
    """A page-locked host buffer is read by the checking kernel itself: the
    same refusal (first bad index, chain unchanged) and the same round trip as
    a pageable buffer."""
    import ctypes as C
    import torch
    from dym_symanzik_action_gb300._lib import DymError, check, lib, ptr
    lat = engine.Lattice(group(engine, "BT"), 4, 4, 4, 0.0, 1.0, 0.0, 3, start="hot")
    before = lat.links.copy().ravel()
    n = before.size
    hin = torch.empty(n, dtype=torch.uint16, pin_memory=True).numpy()
    hout = torch.empty(n, dtype=torch.uint16, pin_memory=True).numpy()
    hin[:] = before
    hin[321] = lat.group.P
    hin[400] = 0xFFFF
    with pytest.raises(DymError, match="at 321$"):
        check(lib().dym_links_set(lat._h, ptr(hin, C.c_uint16)))
    check(lib().dym_links_get(lat._h, ptr(hout, C.c_uint16)))
    assert (hout == before).all()
    hin[:] = np.roll(before, 7)
    check(lib().dym_links_set(lat._h, ptr(hin, C.c_uint16)))
    hout[:] = 0
    check(lib().dym_links_get(lat._h, ptr(hout, C.c_uint16)))
    assert (hout == np.roll(before, 7)).all() and (lat.links.ravel() == hout).all()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_l2_window_leaves_configurations_unchanged(engine, precision):
    """Pinning the Cayley table in L2 (an access-policy window on the chain's
    stream) changes where the table lives, not what the sweep computes: the
    same chain with and without the window, switched on and off between
    calls, gives the same links and counters after every call."""
    g = group(engine, "S1080")
    plain = engine.Lattice(g, 4, 4, 8, 0.0, 2.0, -0.1, 11, start="hot", precision=precision)
    pinned = engine.Lattice(g, 4, 4, 8, 0.0, 2.0, -0.1, 11, start="hot", precision=precision)
    pinned.set_l2_window(True)
    pinned.set_l2_window(True)  # idempotent
    for on in (True, False, True):
        pinned.set_l2_window(on)
        a = plain.update(2, 10)
        b = pinned.update(2, 10)
        assert (a.hits, a.accepts) == (b.hits, b.accepts)
        assert (plain.links == pinned.links).all()
    pinned.close()  # releases the window and the set-aside
    again = engine.Lattice(g, 4, 4, 8, 0.0, 2.0, -0.1, 11, start="hot", precision=precision)
    again.set_l2_window(True)
    again.set_l2_window(False)
    again.close()
    plain.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_checkpoint_resume_is_bit_exact(engine, tmp_path, precision):
    """A chain saved after 3 sweeps and loaded into a fresh chain (created
    with another seed, couplings, start and precision mode) continues exactly
    as the chain that ran 6 sweeps without stopping: the checkpoint carries
    the seed and the sweep counter that key the Philox stream, and the
    couplings.  Refused loads (another lattice, ids out of range) leave the
    chain as it was."""
    from dym_symanzik_action_gb300._lib import DymError
    from test_checkpoint import write_checkpoint
    g = group(engine, "S1080")
    whole = engine.Lattice(g, 4, 4, 8, 0.0, 2.0, -0.1, 21, start="hot", precision=precision)
    whole.update(3, 10)
    b = whole.update(3, 10)
    first = engine.Lattice(g, 4, 4, 8, 0.0, 2.0, -0.1, 21, start="hot", precision=precision)
    first.update(3, 10)
    p = tmp_path / "c.ckpt"
    first.save_checkpoint(p)
    saved = first.links.copy()
    first.close()
    info = engine.checkpoint_info(p)
    assert (info["sweep"], info["seed"], info["beta1"], info["beta2"]) == (3, 21, 2.0, -0.1)
    assert info["table_hash"] == g.table_hash
    other = "shared" if precision == "fp64" else "fp64"
    resumed = engine.Lattice(g, 4, 4, 8, 1.0, 0.5, 0.0, 999, start="cold", precision=other)
    resumed.load_checkpoint(p)
    assert (resumed.links == saved).all() and resumed.seed == 21 and resumed.beta == (0.0, 2.0, -0.1)
    r = resumed.update(3, 10)
    assert (resumed.links == whole.links).all()
    assert (r.hits, r.accepts, r.sweep) == (b.hits, b.accepts, b.sweep) == (b.hits, b.accepts, 6)

    before = resumed.links.copy()
    small = engine.Lattice(g, 4, 4, 6, 0.0, 2.0, -0.1, 21, start="hot")
    with pytest.raises(DymError) as e:
        small.load_checkpoint(p)
    assert e.value.code == -1
    small.close()
    bad = saved.ravel().copy()
    bad[1234] = g.P
    q = tmp_path / "bad.ckpt"
    write_checkpoint(q, 4, 4, 8, g.P, 0, g.table_hash, 5, 77, (0.0, 1.0, 0.0), bad)
    with pytest.raises(DymError, match="at 1234$"):
        resumed.load_checkpoint(q)
    assert (resumed.links == before).all()
    assert resumed.update(1, 10).sweep == 7  # counter untouched by the refused load
    resumed.close()
    whole.close()
