"""Mixed precision at scale: S(1080) 48^3 x 12 (5,308,416 links), hot start,
beta1 in {2.0, 2.5, 3.0}, beta2 = -0.1.  The mixed kernel (exact fixed-point
dS, FP32 threshold test, FP64 re-evaluation within its error bound) must give
the configuration of the all-FP64 path after every block of sweeps, re-check
only a small fraction of hits, and see |dS_fast - dS_fp64| far below its
bound at the re-checks."""
import numpy as np
import pytest

from dym_symanzik_action_gb300 import tables

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("beta1", [2.0, 2.5, 3.0])
def test_mixed_matches_fp64_at_48x12(engine, beta1):
    g = engine.load_group(tables.ensure_table("S1080"))
    lm = engine.Lattice(g, 4, 12, 48, 0.0, beta1, -0.1, 4848, start="hot", precision="mixed")
    lf = engine.Lattice(g, 4, 12, 48, 0.0, beta1, -0.1, 4848, start="hot", precision="shared")
    hits = rechecks = 0
    max_err = 0.0
    for block in range(3):
        sm = lm.update(10, 10)
        sf = lf.update(10, 10)
        assert sm.accepts == sf.accepts, block
        assert np.array_equal(lm.links, lf.links), block
        hits += sm.hits
        rechecks += sm.rechecks
        max_err = max(max_err, sm.max_ds_err)
    assert hits == 30 * 10 * lm.V * 4
    assert rechecks < 1e-3 * hits
    assert max_err < 1e-3
    # a few sweeps of the direct FP64 kernel (reference arithmetic) agree too
    ld = engine.Lattice(g, 4, 12, 48, 0.0, beta1, -0.1, 4848, start="hot", precision="fp64")
    lm2 = engine.Lattice(g, 4, 12, 48, 0.0, beta1, -0.1, 4848, start="hot", precision="mixed")
    ld.update(2, 10)
    lm2.update(2, 10)
    assert np.array_equal(ld.links, lm2.links)
    for lat in (lm, lf, ld, lm2):
        lat.close()
