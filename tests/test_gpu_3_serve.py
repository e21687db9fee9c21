"""Served LLR windows: every request's response equals running that request
alone on a fresh chain with dym_llr_run (bit for bit), whether the server
holds one chain at a time or many, with queueing and chain reuse."""
import numpy as np
import pytest

from dym_symanzik_action_gb300 import tables
from dym_symanzik_action_gb300.serve import Server

pytestmark = pytest.mark.gpu

REQS = [  # id, Nt, Nx, centre/NPLAQ, start, bg
    (0, 2, 4, -1.0, "hot", 0.0), (1, 4, 4, -2.0, "cold", -0.1), (2, 2, 6, -0.7, "hot", -0.1),
    (3, 4, 4, -1.2, "hot", 0.0), (4, 2, 4, -2.4, "cold", 0.0), (5, 4, 6, -0.9, "hot", -0.1),
    (6, 2, 4, -1.0, "hot", 0.0), (7, 4, 4, -0.5, "hot", -0.1),
]
K, NRM, NHIT, CAP = 4, 3, 5, 60


def window(Nt, Nx, cen):
    npl = 6 * Nt * Nx ** 3
    return cen * npl, 0.5 * 0.0225 * npl


def run_server(engine, max_chains):
    g = engine.load_group(tables.ensure_table("S1080"))
    s = Server(g, max_chains=max_chains, nhit=NHIT)
    for rid, Nt, Nx, cen, start, bg in REQS:
        ewin, hw = window(Nt, Nx, cen)
        s.submit(rid, Nt, Nx, ewin, hw, a0=2.0, seed=1000 + rid, start=start, bg=bg, K=K, NRM=NRM, drive_cap=CAP)
    out = {}
    for _ in range(10000):
        s.step(2)
        for r in s.poll():
            out[r.id] = r
        if len(out) == len(REQS):
            break
    st = s.status()
    s.close()
    return out, st


def test_served_results_equal_alone(engine):
    g = engine.load_group(tables.ensure_table("S1080"))
    alone = {}
    for rid, Nt, Nx, cen, start, bg in REQS:
        ewin, hw = window(Nt, Nx, cen)
        lat = engine.Lattice(g, 4, Nt, Nx, 0.0, 0.0, 0.0, 1000 + rid, start=start)
        alone[rid] = lat.llr_run(ewin=ewin, hw=hw, a0=2.0, axis=1, bg=bg, K=K, NRM=NRM, nhit=NHIT, drive_cap=CAP)
    for max_chains in (8, 3):
        served, st = run_server(engine, max_chains)
        assert set(served) == set(alone) and st["active"] == 0 and st["queued"] == 0
        for rid, r in served.items():
            a = alone[rid]
            assert r.status == a.status and r.sweeps == a.sweeps and r.hits == a.hits
            assert (r.a_hist == a.a_hist).all() and r.S1 == a.S1 and r.S2 == a.S2


def test_server_cancel_reject_and_budget(engine):
    """Every accepted request gets exactly one response.  A request whose
    chain alone exceeds the device-memory budget is refused at submit
    (DYM_ERANGE); a request with an invalid window is answered "rejected"
    without failing the step or the other requests; a queued or a resident
    request can be withdrawn ("cancelled", the resident one with the sweeps it
    ran), freeing its slot; the rest finish as they would alone."""
    from dym_symanzik_action_gb300._lib import DymError
    g = engine.load_group(tables.ensure_table("S1080"))
    s = Server(g, max_chains=2, hbm_budget=64 << 20, nhit=NHIT)
    with pytest.raises(DymError) as e:
        s.submit(99, 16, 48, *window(16, 48, -1.0), a0=2.0, seed=1, K=K, NRM=NRM, drive_cap=CAP)  # ~100 MB
    assert e.value.code == -8
    for rid, Nt, Nx, cen, start, bg in REQS[:4]:
        ewin, hw = window(Nt, Nx, cen)
        s.submit(rid, Nt, Nx, ewin, hw if rid != 1 else 0.0, a0=2.0, seed=1000 + rid, start=start, bg=bg, K=K,
                 NRM=NRM, drive_cap=CAP)
    s.cancel(3)  # still queued
    got = {r.id: r for r in s.poll()}
    assert set(got) == {3} and got[3].status == "cancelled" and got[3].hits == 0
    s.step(2)  # admits 0 and 2 (1 is rejected on admission)
    got = {r.id: r for r in s.poll()}
    assert set(got) == {1} and got[1].status == "rejected"
    assert s.status()["active"] == 2
    s.cancel(2)  # resident
    got = {r.id: r for r in s.poll()}
    assert set(got) == {2} and got[2].status == "cancelled" and got[2].hits > 0
    st = s.status()
    assert st["active"] == 1 and st["queued"] == 0
    with pytest.raises(DymError) as e:
        s.cancel(2)
    assert e.value.code == -1
    for _ in range(10000):
        s.step(2)
        got.update({r.id: r for r in s.poll()})
        if 0 in got:
            break
    assert got[0].status in ("done", "unreached")
    alone, _ = run_server_subset(engine, [REQS[0]])
    assert got[0].a == alone[0].a and got[0].hits == alone[0].hits and (got[0].a_hist == alone[0].a_hist).all()
    assert s.status()["active"] == 0
    s.close()


def run_server_subset(engine, reqs):
    g = engine.load_group(tables.ensure_table("S1080"))
    s = Server(g, max_chains=1, nhit=NHIT)
    for rid, Nt, Nx, cen, start, bg in reqs:
        ewin, hw = window(Nt, Nx, cen)
        s.submit(rid, Nt, Nx, ewin, hw, a0=2.0, seed=1000 + rid, start=start, bg=bg, K=K, NRM=NRM, drive_cap=CAP)
    out = {}
    for _ in range(10000):
        s.step(2)
        out.update({r.id: r for r in s.poll()})
        if len(out) == len(reqs):
            break
    st = s.status()
    s.close()
    return out, st
