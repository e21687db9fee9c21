"""The C-ABI library: loads, exports every symbol include/dymgpu.h declares,
parses group files like the reference loader and reports errors by code
where the reference aborts (group.c:13-98).  No device needed."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from dym_symanzik_action_gb300 import tables


def declared_functions():
    text = open(os.path.join(ROOT, "include", "dymgpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dym_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(engine):
    from dym_symanzik_action_gb300._lib import LIB_PATH, PROTOTYPES
    out = subprocess.run(["nm", "-D", "--defined-only", LIB_PATH], stdout=subprocess.PIPE, text=True, check=True)
    exported = {l.split()[-1] for l in out.stdout.splitlines()}
    decl = declared_functions()
    assert len(decl) >= 15
    missing = [f for f in decl if f not in exported]
    assert not missing, missing
    assert set(decl) == set(PROTOTYPES), set(decl) ^ set(PROTOTYPES)


def test_group_load_and_info(engine):
    g = engine.load_group(tables.ensure_table("S1080"))
    assert g.P == 1080 and g.id == 0
    assert len(g.smallgroup) == 72
    assert g.n_classes == 11 and g.classes_exact
    assert g.min_retr == -3.0
    t = tables.generate("S1080")
    assert (g.mult == t.mult).all() and (g.ReTr == t.retr).all()
    inv = g.inv
    assert (g.mult[np.arange(1080), inv] == 0).all()


def test_load_reference_style_noisy_traces(engine, tmp_path):
    """Trace values with 1e-16 noise (as in the reference's own files) load,
    with classes_exact false."""
    t = tables.generate("BI")
    t.retr = t.retr + np.where(np.arange(t.P) % 3 == 0, 1e-16, 0.0)
    p = str(tmp_path / "noisy")
    tables.write_table(t, p)
    g = engine.load_group(p)
    assert g.P == 120 and not g.classes_exact and g.n_classes == 9
    assert 0 < g.class_spread < 1e-15


def write_raw(path, P, retr, imtr, mult, extra=""):
    with open(path, "w") as f:
        f.write(f"{P}\n{' '.join(repr(float(x)) for x in retr)}\n{' '.join(repr(float(x)) for x in imtr)}\n")
        f.write(" ".join(str(int(x)) for x in np.asarray(mult).ravel()) + extra)


@pytest.mark.parametrize("case", ["missing", "truncated", "out_of_range", "no_identity", "no_inverse",
                                  "too_large", "bad_token"])
def test_group_load_errors(engine, tmp_path, case):
    from dym_symanzik_action_gb300._lib import DymError
    t = tables.generate("BT")
    p = str(tmp_path / case)
    m = t.mult.copy()
    code = {"missing": -2, "too_large": -8}.get(case, -3)
    if case == "missing":
        p = str(tmp_path / "does_not_exist")
    elif case == "truncated":
        write_raw(p, t.P, t.retr, t.imtr, m.ravel()[:-5])
    elif case == "out_of_range":
        m[3, 4] = 99
        write_raw(p, t.P, t.retr, t.imtr, m)
    elif case == "no_identity":
        m = (m + 1) % t.P
        write_raw(p, t.P, t.retr, t.imtr, m)
    elif case == "no_inverse":
        m[:, :] = 0
        m[0, :] = np.arange(t.P)
        m[:, 0] = np.arange(t.P)
        m[1:, 1:] = 1
        write_raw(p, t.P, t.retr, t.imtr, m)
    elif case == "too_large":
        with open(p, "w") as f:
            f.write("5041\n")
    elif case == "bad_token":
        with open(p, "w") as f:
            f.write("2\n0 0\n0 0\n0 1 1 x\n")
    with pytest.raises(DymError) as e:
        engine.load_group(p)
    assert e.value.code == code


def test_trailing_tokens_ignored(engine, tmp_path):
    t = tables.generate("BT")
    p = str(tmp_path / "trailing")
    write_raw(p, t.P, t.retr, t.imtr, t.mult, extra=" 1.5 2.5 junk\n")
    g = engine.load_group(p)
    assert g.P == 24 and (g.mult == t.mult).all()


def test_chain_without_device_fails_loudly(engine):
    """No CPU fallback: creating a chain needs the GPU."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from dym_symanzik_action_gb300._lib import DymError
    g = engine.load_group(tables.ensure_table("BT"))
    with pytest.raises(DymError) as e:
        engine.Lattice(g, 4, 4, 4, 0, 1, 0, 1)
    assert e.value.code == -5


def test_cli_usage(engine):
    from dym_symanzik_action_gb300.build import CLI
    r = subprocess.run([CLI], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 1
    assert "usage:" in r.stderr and "group D Nt Nx beta0 beta1 beta2 seed [K] [N] [Ntherm]" in r.stderr
