"""Two lanes per link in the value-table kernel (DYM_LANES_PER_LINK=2), and
its hit-unroll variants (DYM_HIT_UNROLL).

The pair splits a link's staples by side (+f / -f of every plane), sums its
partial fixed-point sums with shuffles and takes each decision from the same
integers as the one-lane kernel, with the exact re-evaluation summing the
pair's terms in the reference's order.  So the configurations and the
hit / accept / re-evaluation counts must be the one-lane kernel's after every
sweep: on the cold 32^3 x 8 chain of the benchmark (every proposal rejected),
and on moving chains forced onto the value-table kernel (DYM_VT_MAX_ACCEPT=1)
where accepted moves update the pair's elements and re-evaluations occur.
The one-lane chain is itself checked against the oracle elsewhere; here a
moving 8^4 chain is also compared with the oracle directly."""
import numpy as np
import pytest

from dym_symanzik_action_gb300 import tables
from dym_symanzik_action_gb300.schedule import schedule
from oracle.oracle import OracleGroup, OracleLattice

pytestmark = pytest.mark.gpu

KERNEL_MIXED_VALUES = 4


def run(engine, monkeypatch, lanes, shape, beta, seed, start, sweeps, nhit, group="S1080"):
    monkeypatch.setenv("DYM_LANES_PER_LINK", str(lanes))
    monkeypatch.setenv("DYM_VT_MAX_ACCEPT", "1.0")
    g = engine.load_group(tables.ensure_table(group))
    Nt, Nx = shape
    lat = engine.Lattice(g, 4, Nt, Nx, *beta, seed, start=start, precision="mixed")
    out = []
    for _ in range(sweeps):
        st = lat.update(1, nhit)
        out.append((lat.links.copy(), st.hits, st.accepts, st.rechecks, st.kernel))
    lat.close()
    return out


CASES = {
    "cold_32x8_b3": ((8, 32), (0.0, 3.0, -0.15), 20261203, "cold", 3, 10),
    "hot_8x8_b2": ((8, 8), (0.0, 2.0, -0.1), 4242, "hot", 4, 10),
    "hot_16x8_b1": ((8, 16), (0.0, 1.0, 0.0), 99, "hot", 3, 7),
    "hot_4x6_b25": ((4, 6), (0.3, 2.5, -0.2), 7, "hot", 4, 10),
}


@pytest.mark.parametrize("name", list(CASES))
def test_two_lanes_equal_one_lane(engine, monkeypatch, name):
    shape, beta, seed, start, sweeps, nhit = CASES[name]
    one = run(engine, monkeypatch, 1, shape, beta, seed, start, sweeps, nhit)
    two = run(engine, monkeypatch, 2, shape, beta, seed, start, sweeps, nhit)
    for s, (a, b) in enumerate(zip(one, two)):
        assert a[1:4] == b[1:4], (s, a[1:4], b[1:4])
        assert np.array_equal(a[0], b[0]), f"sweep {s}"
    assert all(x[4] == KERNEL_MIXED_VALUES for x in two[1:])
    if start == "hot":
        assert sum(x[2] for x in two) > 0  # accepted moves exercised


def test_two_lanes_moving_chain_matches_oracle(engine, monkeypatch):
    D, Nt, Nx, beta, seed, nhit = 4, 4, 8, (0.0, 2.0, -0.1), 515, 10
    path = tables.ensure_table("S1080")
    got = run(engine, monkeypatch, 2, (Nt, Nx), beta, seed, "hot", 3, nhit)
    ol = OracleLattice(OracleGroup(path), D, Nt, Nx)
    ol.hot_start(seed)
    sched = schedule(D, Nt, Nx)
    for s in range(3):
        h, a = ol.sweep(sched, beta, seed, s, 1, nhit)
        assert (got[s][1], got[s][2]) == (h, a), s
        assert (got[s][0].ravel() == ol.links).all(), f"sweep {s}"


@pytest.mark.parametrize("name", ["cold_32x8_b3", "hot_8x8_b2", "hot_16x8_b1"])
def test_hit_unroll_variants_equal(engine, monkeypatch, name):
    """The value-table kernel's hits one at a time (DYM_HIT_UNROLL=1), in
    speculative pairs (2, the default: both sums from the current state, the
    second re-formed after an accept) and in groups of draws computed ahead
    (5, 10) take the same decisions."""
    shape, beta, seed, start, sweeps, nhit = CASES[name]
    runs = {}
    for hu in ("1", "2", "5", "10"):
        monkeypatch.setenv("DYM_HIT_UNROLL", hu)
        runs[hu] = run(engine, monkeypatch, 1, shape, beta, seed, start, sweeps, nhit)
    for hu in ("2", "5", "10"):
        for s, (a, b) in enumerate(zip(runs["1"], runs[hu])):
            assert a[1:5] == b[1:5], (hu, s)
            assert np.array_equal(a[0], b[0]), (hu, s)
