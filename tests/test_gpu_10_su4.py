"""The SU(4) subgroup BI (x) BO of order 2880 -- the order of the reference's
largest shipped SU(4) table, element ids beyond 11 bits -- through every
engine path that takes it, bit for bit against the oracle: Metropolis sweeps
at each precision setting (the mixed kernel with 32-bit packed sub-table
entries, the FP64 shared-table kernel, the FP64 direct kernel), observables,
the batched ensemble next to SU(2) chains (its mixed kernel packs 16-bit
entries, so this batch runs the FP64 shared-table batch kernel), and LLR on
either axis."""
import numpy as np
import pytest

from dym_symanzik_action_gb300 import tables
from dym_symanzik_action_gb300.batch import Batch, Tuning
from dym_symanzik_action_gb300.schedule import schedule
from oracle.oracle import OracleGroup, OracleLattice
from test_llr import nplaq, run_oracle

pytestmark = pytest.mark.gpu

NAME = "BIxBO"
KERNEL_DIRECT, KERNEL_SHARED, KERNEL_MIXED = 1, 2, 3


@pytest.fixture(scope="module")
def su4(engine):
    path = tables.ensure_table(NAME)
    return engine.load_group(path), OracleGroup(path)


def test_group_loads_with_the_shared_table_path(su4):
    g, og = su4
    assert g.P == 2880 and og.P == 2880
    assert g.fast_path


@pytest.mark.parametrize("precision,kernel", [("fp64", KERNEL_DIRECT), ("shared", KERNEL_SHARED),
                                              ("mixed", KERNEL_MIXED)])
def test_sweeps_and_observables_match_oracle(engine, su4, precision, kernel):
    g, og = su4
    D, Nt, Nx, beta, nhit, seed = 4, 4, 8, (0.0, 2.0, -0.1), 10, 2880
    lat = engine.Lattice(g, D, Nt, Nx, *beta, seed, start="hot", precision=precision)
    ol = OracleLattice(og, D, Nt, Nx)
    ol.hot_start(seed)
    assert (ol.links == lat.links.ravel()).all()
    sched = schedule(D, Nt, Nx)
    for s in range(3):
        st = lat.update(1, nhit)
        assert st.kernel == kernel
        h, a = ol.sweep(sched, beta, seed, s, 1, nhit)
        assert (st.hits, st.accepts) == (h, a)
        assert (lat.links.ravel() == ol.links).all(), s
    m = lat.measure(4, 4)
    got = np.concatenate([[m.poly_re, m.poly_im, m.plaq, m.rect], m.wloop.ravel()])
    assert (got == ol.measure(4, 4)).all()


def test_batch_with_su2_chains_matches_single_chains(engine, su4):
    g, _ = su4
    bi = engine.load_group(tables.ensure_table("BI"))
    shapes = [(g, 8, 4, (0.0, 2.0, -0.1)), (bi, 8, 2, (0.0, 2.0, -0.1)), (g, 4, 6, (0.0, 1.0, 0.3)),
              (bi, 12, 4, (0.0, 3.0, 0.0))]

    def chains(precision):
        return [engine.Lattice(grp, 4, Nt, Nx, *beta, 900 + k, start="hot", precision=precision)
                for k, (grp, Nx, Nt, beta) in enumerate(shapes)]

    alone = chains("fp64")
    counts = [lat.update(3, 10) for lat in alone]
    batched = chains("mixed")
    b = Batch()
    for lat in batched:
        b.add(lat)
    b.tuning = Tuning(256, 256, 1, True)
    tot = b.update(3, 10)
    assert tot.hits == sum(c.hits for c in counts) and tot.accepts == sum(c.accepts for c in counts)
    for x, y in zip(alone, batched):
        assert (x.links == y.links).all()


LLR_CASES = [
    # name, group, D, Nt, Nx, start, seed, axis, bg, window centre / NPLAQ, a0, K, NRM, nhit, drive_cap
    ("su4_4444_hot", NAME, 4, 4, 4, "hot", 21, 1, 0.2, -0.6, 1.0, 4, 5, 10, 300),
    ("su4_4444_cold_axis2", NAME, 4, 4, 4, "cold", 22, 2, 0.5, -3.0, 2.0, 4, 5, 10, 300),
]


@pytest.mark.parametrize("case", LLR_CASES, ids=[c[0] for c in LLR_CASES])
def test_llr_matches_oracle(engine, su4, case):
    name, gname, D, Nt, Nx, start, seed, axis, bg, cen, a0, K, NRM, nhit, cap = case
    L, r = run_oracle(case)
    assert r["status"] == "done"
    lat = engine.Lattice(su4[0], D, Nt, Nx, 0.0, 0.0, 0.0, seed, start=start)
    n = nplaq(D, Nt, Nx) * (1 if axis == 1 else 2)
    res = lat.llr_run(ewin=cen * n, hw=0.0225 * n / 2, a0=a0, axis=axis, bg=bg, K=K, NRM=NRM, nhit=nhit,
                      drive_cap=cap)
    assert res.status == r["status"]
    assert (res.a_hist == r["a_hist"]).all()
    assert (res.hits, res.accepts, res.sweeps) == (r["hits"], r["accepts"], r["sweeps"])
    assert res.S1 == r["S1"] and res.S2 == r["S2"]
    assert (lat.links.ravel() == L.links).all()


def test_mixed_kernel_rechecks_and_matches_fp64_at_16x16x16x8(engine, su4):
    """Hot 16^3 x 8 at beta = (0, 2, -0.1), NHIT 10, 5 sweeps: the mixed kernel
    (32-bit entries) re-evaluates a small fraction of the hits in FP64, stays
    within its error bound, and gives the FP64 kernel's configuration; after a
    cold start (moves rare) it keeps the element-table kernel, the value-table
    kernel taking only 16-bit entries."""
    g, _ = su4
    D, Nt, Nx, beta, nhit = 4, 8, 16, (0.0, 2.0, -0.1), 10
    res = {}
    for precision in ("mixed", "fp64"):
        lat = engine.Lattice(g, D, Nt, Nx, *beta, 4242, start="hot", precision=precision)
        st = lat.update(5, nhit)
        res[precision] = (lat.links.ravel(), st)
    (lm, sm), (lf, sf) = res["mixed"], res["fp64"]
    assert sm.kernel == KERNEL_MIXED and sf.kernel == KERNEL_DIRECT
    assert (lm == lf).all() and sm.accepts == sf.accepts
    assert 0 < sm.rechecks < 1e-3 * sm.hits
    assert 0.0 <= sm.max_ds_err < 1e-3
    cold = engine.Lattice(g, D, Nt, Nx, 0.0, 4.0, -0.1, 7, start="cold", precision="mixed")
    ref = engine.Lattice(g, D, Nt, Nx, 0.0, 4.0, -0.1, 7, start="cold", precision="fp64")
    for _ in range(2):
        assert cold.update(1, nhit).kernel == KERNEL_MIXED
        ref.update(1, nhit)
        assert (cold.links == ref.links).all()
