"""The colour schedule is race-free.

The reference's two-parity checkerboard (dym-mod-metro.cpp:152-159) is not:
its rectangle staples read same-parity links of the same direction.  The
engine's schedule is checked twice: by the library's own offset check and,
independently, by the oracle, which enumerates the links each update reads
from the staple formulas of dym-mod-metro.cpp:63-142."""
import numpy as np
import pytest

from dym_symanzik_action_gb300 import tables
from dym_symanzik_action_gb300.schedule import conflicts, schedule
from oracle.oracle import OracleGroup, OracleLattice

SHAPES = [(4, 4, 4), (4, 8, 4), (4, 2, 4), (4, 6, 6), (4, 3, 6), (4, 8, 12), (4, 12, 8), (4, 1, 4), (4, 4, 5),
          (4, 6, 8), (4, 2, 6), (4, 4, 3), (3, 4, 4), (3, 2, 6), (3, 5, 5), (2, 8, 8), (2, 3, 3), (2, 2, 2),
          (4, 2, 2)]


@pytest.fixture(scope="module")
def bt():
    return OracleGroup(tables.ensure_table("BT"))


@pytest.mark.parametrize("D,Nt,Nx", SHAPES)
def test_schedule_is_race_free(bt, D, Nt, Nx):
    pd, pl, sites = schedule(D, Nt, Nx)
    V = Nt * Nx ** (D - 1)
    assert pl.sum() == V * D
    nphase, c = conflicts(D, Nt, Nx)
    assert c == 0 and nphase == len(pd)
    L = OracleLattice(bt, D, Nt, Nx)
    assert L.conflicts((pd, pl, sites)) == 0
    # phases are ordered by direction, sites ascending within a phase
    assert (np.diff(pd) >= 0).all()
    off = 0
    for n in pl:
        assert (np.diff(sites[off:off + n].astype(np.int64)) > 0).all()
        off += n


def test_four_colours_per_direction_when_extents_divisible_by_four():
    for Nt, Nx in [(4, 4), (8, 32), (12, 48), (8, 8), (4, 16)]:
        pd, _, _ = schedule(4, Nt, Nx)
        assert len(pd) == 16


def test_reference_parity_checkerboard_races(bt):
    """The reference's own schedule: one phase per (direction, parity)."""
    D, Nt, Nx = 4, 4, 4
    L = OracleLattice(bt, D, Nt, Nx)
    V = L.V
    coords = np.stack(np.unravel_index(np.arange(V), (Nx, Nx, Nx, Nt))[::-1])  # t fastest
    parity = coords.sum(0) & 1
    pd, pl, sites = [], [], []
    for d in range(D):
        for par in (0, 1):
            s = np.nonzero(parity == par)[0].astype(np.uint32)
            pd.append(d)
            pl.append(len(s))
            sites.append(s)
    bad = L.conflicts((np.array(pd, np.int32), np.array(pl, np.uint32), np.concatenate(sites)))
    assert bad > 0


@pytest.mark.parametrize("shape", [(4, 4, 4), (4, 2, 4), (4, 6, 6), (3, 8, 4), (2, 8, 8), (4, 5, 5), (4, 3, 4),
                                   (4, 2, 12), (4, 6, 8), (4, 4, 6), (4, 8, 16)])
def test_plain_python_schedule_equals_library(shape):
    """The CPU legs of bench.py build their colour phases without the engine
    (oracle.colour_schedule); they must be the library's phases exactly."""
    from oracle.oracle import colour_schedule
    a, b = colour_schedule(*shape), schedule(*shape)
    for x, y in zip(a, b):
        assert x.dtype == y.dtype and x.shape == y.shape and (x == y).all()
