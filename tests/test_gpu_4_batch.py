"""Batched ensemble: chains of uneven size and two groups updated together
give, chain by chain, the configurations and counters of running each chain
alone (bit-exact), with and without the CUDA graph, for every tuning the
autotuner tries, with the mixed-precision batch kernel (chains created
"mixed") and the FP64 shared-table batch kernel (chains created "shared")."""
import numpy as np
import pytest

from dym_symanzik_action_gb300 import tables
from dym_symanzik_action_gb300.batch import Batch, Tuning

pytestmark = pytest.mark.gpu

SHAPES = [("S1080", 8, 4, (0.0, 1.5, 0.1)), ("BI", 8, 2, (0.0, 2.0, -0.1)), ("S1080", 12, 6, (0.0, 3.0, -0.2)),
          ("BI", 12, 8, (0.0, 1.0, 0.3)), ("S1080", 8, 2, (0.0, 2.5, 0.0)), ("S1080", 16, 4, (0.0, 4.0, -0.3))]


def make_chains(engine, seed0=700, precision="mixed"):
    groups = {n: engine.load_group(tables.ensure_table(n)) for n in ("S1080", "BI")}
    return [engine.Lattice(groups[g], 4, Nt, Nx, *beta, seed0 + k, start="hot", precision=precision)
            for k, (g, Nx, Nt, beta) in enumerate(SHAPES)], groups


@pytest.mark.parametrize("tuning", [Tuning(256, 256, 1, True), Tuning(128, 128, 2, False), Tuning(1024, 256, 1, True),
                                    Tuning(512, 256, 1, True, 2), Tuning(256, 128, 2, False, 5)],
                         ids=["graph-256", "nograph-128", "graph-tile1024", "graph-hitunroll2", "nograph-hitunroll5"])
@pytest.mark.parametrize("precision", ["mixed", "shared"])
def test_batch_matches_single_chains(engine, tuning, precision):
    alone, _ = make_chains(engine, precision="fp64")
    counts = [lat.update(3, 10) for lat in alone]
    mixed, _ = make_chains(engine, precision=precision)
    b = Batch()
    for lat in mixed:
        b.add(lat)
    b.tuning = tuning
    tot = b.update(3, 10)
    assert tot.hits == sum(c.hits for c in counts) and tot.accepts == sum(c.accepts for c in counts)
    if precision == "shared":
        assert tot.rechecks == 0
    assert tot.rechecks < 1e-3 * tot.hits and 0.0 <= tot.max_ds_err < 1e-3
    for k, (x, y) in enumerate(zip(alone, mixed)):
        assert (x.links == y.links).all(), k
        assert b.chain_counters(k) == (counts[k].hits, counts[k].accepts)
    # the chains continue identically after the batch (sweep counters advanced)
    for x, y in zip(alone, mixed):
        x.update(1, 10)
        y.update(1, 10)
        assert (x.links == y.links).all()


def test_batch_autotune_restores_state(engine):
    chains, _ = make_chains(engine, seed0=900)
    b = Batch()
    for lat in chains:
        b.add(lat)
    before = [lat.links.copy() for lat in chains]
    best = b.autotune(nhit=10, nsweeps_per_trial=1)
    assert best.tile in (128, 256, 512, 1024) and best.threads in (128, 256, 512) and best.hit_unroll in (1, 2)
    for x, lat in zip(before, chains):
        assert (x == lat.links).all()
    ref, _ = make_chains(engine, seed0=900)
    b.update(2, 10)
    for x, y in zip(ref, chains):
        x.update(2, 10)
        assert (x.links == y.links).all()
