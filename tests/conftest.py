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
