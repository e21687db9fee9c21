import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _have_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _have_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def engine():
    """Built libdymgpu (compiled in-tree on first use)."""
    from dym_symanzik_action_gb300 import build
    build.build()
    import dym_symanzik_action_gb300 as dym
    return dym


@pytest.fixture(scope="session")
def table():
    from dym_symanzik_action_gb300 import tables
    return tables.ensure_table


def golden(name: str):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


@pytest.fixture(scope="session")
def sweeps_golden():
    return golden("sweeps.npz")


def sweep_cases():
    import ast
    return ast.literal_eval(str(golden("sweeps.npz")["cases"]))


def ref_table_cases():
    import ast
    return ast.literal_eval(str(golden("ref_tables.npz")["cases"]))


# Generated table standing for each reference file whose content the fixtures
# can rebuild (tables_iso.npz: pi; ref_tables.npz: the file's trace rows).
REBUILDABLE = {"mys1080-v4": "S1080", "myBI": "BI"}


def reference_table(fname: str, outdir: str) -> str:
    """Path of a table file with the content of the reference's groups/<fname>
    (its numbering, Cayley table and ReTr/ImTr doubles; the trailing matrices
    left out): rebuilt from the generated table through the isomorphism pi of
    tables_iso.npz, with the file's own trace rows from ref_tables.npz, and
    checked against the SHA-256 of the reference's Cayley table."""
    import hashlib
    from dym_symanzik_action_gb300 import tables
    mine = REBUILDABLE[fname]
    path = os.path.join(outdir, fname)
    if os.path.exists(path):
        return path
    iso, rt = golden("tables_iso.npz"), golden("ref_tables.npz")
    g = tables.generate(mine)
    pi = iso[f"{mine}_pi"].astype(np.int64)
    P = len(pi)
    rm = np.empty((P, P), np.int64)
    rm[pi[:, None], pi[None, :]] = pi[np.asarray(g.mult, np.int64)]
    assert hashlib.sha256(rm.astype(np.int32).tobytes()).hexdigest() == str(iso[f"{mine}_ref_sha"])
    re_, im_ = rt[f"{mine}_retr"], rt[f"{mine}_imtr"]
    with open(path + ".tmp", "w") as f:
        f.write(f"{P}\n")
        f.write(" ".join(repr(float(x)) for x in re_) + "\n")
        f.write(" ".join(repr(float(x)) for x in im_) + "\n")
        for row in rm:
            f.write(" ".join(map(str, row.tolist())) + "\n")
    os.replace(path + ".tmp", path)
    return path


@pytest.fixture(scope="session")
def ref_table(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("reftables"))
    return lambda fname: reference_table(fname, d)


def staged_reference():
    """baseline/_ref (the unmodified reference files staged by
    oracle/stage_ref.sh) or $REF_DIR, if present; else None."""
    from oracle.oracle import ref_dir
    return ref_dir()


def hotelling_p(ref, ours, cols):
    """p-value of Hotelling's two-sample T^2 test of equal means of the per-run
    observables ref, ours ([runs, observables]) on the columns `cols` (a
    subset whose pooled covariance is well conditioned)."""
    from scipy.stats import f as fdist
    a, b = ref[:, list(cols)], ours[:, list(cols)]
    n1, n2, p = len(a), len(b), a.shape[1]
    S = ((n1 - 1) * np.cov(a, rowvar=False) + (n2 - 1) * np.cov(b, rowvar=False)) / (n1 + n2 - 2)
    d = a.mean(0) - b.mean(0)
    t2 = n1 * n2 / (n1 + n2) * d @ np.linalg.solve(S, d)
    return float(fdist.sf((n1 + n2 - p - 1) / (p * (n1 + n2 - 2)) * t2, p, n1 + n2 - p - 1))
