"""Group tables: the generated S(1080), BI, BT and BO tables are groups, have
class-constant traces, and are trace-preserving isomorphic to the reference's
own table files (pinned by tests/golden/tables_iso.npz); the SU(4) table
BI (x) BO (order 2880) is a group of 4x4 special unitary matrices with
class-constant traces."""
import hashlib

import numpy as np
import pytest

from conftest import golden
from dym_symanzik_action_gb300 import tables


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.int32).tobytes()).hexdigest()


@pytest.fixture(scope="module", params=["BT", "BO", "BI", "S1080", "BIxBO"])
def tab(request):
    return tables.generate(request.param)


def test_order_and_identity(tab):
    P = {"BT": 24, "BO": 48, "BI": 120, "S1080": 1080, "BIxBO": 2880}[tab.name]
    assert tab.P == P
    ar = np.arange(P)
    assert (tab.mult[0] == ar).all() and (tab.mult[:, 0] == ar).all()
    # every row and column is a permutation (Latin square)
    assert (np.sort(tab.mult, axis=1) == ar).all()
    assert (np.sort(tab.mult, axis=0) == ar[:, None]).all()


def test_associative(tab):
    m = tab.mult
    P = tab.P
    if P <= 120:
        for a in range(P):
            assert (m[m[a]] == m[a][m]).all()  # (a*b)*c == a*(b*c) for all b, c
    else:
        rng = np.random.default_rng(0)
        a, b, c = rng.integers(0, P, (3, 2_000_000))
        assert (m[m[a, b], c] == m[a, m[b, c]]).all()


def test_traces_are_class_functions(tab):
    m = tab.mult
    inv = np.argmax(m == 0, axis=1)
    for h in range(tab.P):
        conj = m[m[inv[h]], h]  # h^-1 x h for all x
        assert (tab.retr[conj] == tab.retr).all()
        assert (tab.imtr[conj] == tab.imtr).all()


def test_matrices_match_table(tab):
    rng = np.random.default_rng(1)
    a, b = rng.integers(0, tab.P, (2, 500))
    prod = tab.mats[a] @ tab.mats[b]
    assert np.abs(prod - tab.mats[tab.mult[a, b]]).max() < 1e-9
    tr = np.trace(tab.mats, axis1=1, axis2=2)
    assert np.abs(-tr.real - tab.retr).max() < 1e-12
    assert np.abs(-tr.imag - tab.imtr).max() < 1e-12


def test_isomorphic_to_reference_table(tab):
    """pi maps our table onto the reference file's: rebuilding the reference
    Cayley table from ours through pi reproduces its SHA-256."""
    iso = golden("tables_iso.npz")
    name = tab.name
    if f"{name}_pi" not in iso.files:
        pytest.skip(f"the reference ships no table of {name}")
    assert sha(tab.mult) == str(iso[f"{name}_our_sha"])
    pi = iso[f"{name}_pi"].astype(np.int64)
    P = tab.P
    assert sorted(pi.tolist()) == list(range(P))
    ref = np.empty((P, P), np.int64)
    ref[pi[:, None], pi[None, :]] = pi[tab.mult]
    assert sha(ref) == str(iso[f"{name}_ref_sha"])
    assert float(iso[f"{name}_max_dtrace"]) < 1e-14


def test_class_statistics():
    s = tables.generate("S1080")
    assert len(set(s.retr)) == 11 and len(set(zip(s.retr, s.imtr))) == 16
    lo = s.retr.min()
    nn = s.retr[s.retr > lo].min()
    assert lo == -3.0 and abs(nn + (1 + 5 ** 0.5) / 2) < 1e-15
    assert int(((s.retr > lo) & (s.retr < nn + 1e-6)).sum()) == 72


def test_su4_table():
    t = tables.generate("BIxBO")
    n = t.mats.shape[1]
    assert n == 4
    assert np.abs(np.linalg.det(t.mats) - 1).max() < 1e-12
    eye = np.eye(4)
    assert np.abs(t.mats @ np.conj(np.swapaxes(t.mats, 1, 2)) - eye).max() < 1e-12
    assert t.retr[0] == -4.0 and (t.imtr == 0).all()
    lo = t.retr.min()
    nn = t.retr[t.retr > lo].min()
    assert abs(nn + 1 + 5 ** 0.5) < 1e-15  # -Tr g Tr h with Tr g = golden ratio, h = 1
    assert int(((t.retr > lo) & (t.retr < nn + 1e-6)).sum()) == 12
    assert len(set(t.retr)) == 23
    assert sha(t.mult) == sha(tables.generate("BIxBO").mult)  # deterministic


def test_written_file_round_trips(tmp_path):
    from oracle.oracle import OracleGroup
    t = tables.generate("BI")
    p = str(tmp_path / "BI")
    tables.write_table(t, p)
    g = OracleGroup(p)
    mult, inv, re, im = g.tables()
    assert (mult == t.mult).all()
    assert (re == t.retr).all() and (im == t.imtr).all()
    assert g.id == 0 and len(g.pool) == 12
