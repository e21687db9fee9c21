"""Small, odd and largest extents on the four-dimensional fast kernels:
every neighbour offset wraps (extent 1: onto the site itself; 2: a move of
two returns to the site; 3 and 5: one wrap each way), the colour schedule
needs more than four colours (42 to 60 phases), and 256 is the largest
extent whose coordinates pack into 8 bits.  The element-table and
value-table mixed kernels and the FP64 direct kernel give the oracle's
configurations and counts bit for bit after every sweep, from a hot start.
Beyond 256 a mixed-precision chain runs the FP64 shared-table kernel, with
the same result."""
import pytest

from dym_symanzik_action_gb300 import tables
from dym_symanzik_action_gb300.schedule import schedule
from oracle.oracle import OracleGroup, OracleLattice

pytestmark = pytest.mark.gpu

EXTENTS = [(1, 4), (2, 3), (3, 3), (3, 5), (5, 3), (256, 4)]
KERNELS = {"values": ("mixed", "2.0", 4), "elements": ("mixed", "-1", 3), "fp64": ("fp64", "-1", 1)}


@pytest.mark.parametrize("kernel", list(KERNELS))
@pytest.mark.parametrize("extents", EXTENTS, ids=[f"{a}x{b}" for a, b in EXTENTS])
def test_small_extents_match_oracle(engine, monkeypatch, kernel, extents):
    Nt, Nx = extents
    precision, vt_max, want = KERNELS[kernel]
    monkeypatch.setenv("DYM_VT_MAX_ACCEPT", vt_max)
    D, beta, nhit, seed = 4, (0.0, 2.0, -0.1), 5, 4242 + 10 * Nt + Nx
    path = tables.ensure_table("S1080")
    lat = engine.Lattice(engine.load_group(path), D, Nt, Nx, *beta, seed, start="hot", precision=precision)
    ol = OracleLattice(OracleGroup(path), D, Nt, Nx)
    ol.links = lat.links.ravel()
    sched = schedule(D, Nt, Nx)
    for s in range(3):
        st = lat.update(1, nhit)
        assert st.kernel == want, (s, st.kernel)
        h, a = ol.sweep(sched, beta, seed, s, 1, nhit)
        assert (st.hits, st.accepts) == (h, a), s
        assert (lat.links.ravel() == ol.links).all(), s
    lat.close()


def test_extent_beyond_packing_falls_back(engine, monkeypatch):
    monkeypatch.setenv("DYM_VT_MAX_ACCEPT", "2.0")
    D, Nt, Nx, beta, nhit, seed = 4, 257, 4, (0.0, 2.0, -0.1), 5, 91
    path = tables.ensure_table("S1080")
    lat = engine.Lattice(engine.load_group(path), D, Nt, Nx, *beta, seed, start="hot", precision="mixed")
    ol = OracleLattice(OracleGroup(path), D, Nt, Nx)
    ol.links = lat.links.ravel()
    st = lat.update(2, nhit)
    assert st.kernel == 2
    assert (st.hits, st.accepts) == ol.sweep(schedule(D, Nt, Nx), beta, seed, 0, 2, nhit)
    assert (lat.links.ravel() == ol.links).all()
    lat.close()
