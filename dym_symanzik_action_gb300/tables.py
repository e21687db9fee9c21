"""Group-table generator for the discrete gauge groups the engine runs on.

Writes Cayley tables in the plain-text group format the reference loader reads
(groups/README.md:7-21 of the reference; parser group.c:13-65):

    P
    ReTr[0] .. ReTr[P-1]        real part of  -Tr(U_n)
    ImTr[0] .. ImTr[P-1]        imag part of  -Tr(U_n)
    mult[0][0] .. mult[P-1][P-1]
    [3x3 groups: the matrix of every element, 18 doubles each: Re, Im of
     U[0][0], U[0][1], ..., U[2][2] -- the layout the reference's
     configuration writer reads after the table (dym-mod-metro-savecfg.cpp:47,
     248-265); loaders ignore these trailing tokens]

The sign convention (minus the trace) follows the reference's generators, so the
identity has the smallest ReTr.

Groups generated here, each as a matrix group closed under multiplication:

* ``S1080``  -- the order-1080 subgroup Sigma(360x3) of SU(3), from the four
  generators published by Fairbairn, Fulton and Klink (J. Math. Phys. 5, 1038,
  1964): the cyclic permutation, diag(1,-1,-1), the golden-ratio matrix and the
  omega-phase matrix.  These are the same mathematical generators the reference
  uses (groups/generators/genS1080.py:29-35); they fix the embedding in SU(3),
  i.e. the character values, which is what the physics depends on.
* ``BI``     -- the binary icosahedral group (order 120) in SU(2): the unit
  quaternions generated by i, j, (1+i+j+k)/2 and (i + j/phi + phi k)/2.
* ``BT``     -- the binary tetrahedral group (order 24) in SU(2).
* ``BO``     -- the binary octahedral group (order 48) in SU(2): BT and the
  quaternion (1 + i)/sqrt2.
* ``BIxBO``  -- an SU(4) subgroup of order 2880: the Kronecker products g (x) h
  of g in BI and h in BO, i.e. (BI x BO)/{(1,1), (-1,-1)} acting on C^2 (x) C^2.
  It has the order of the reference's largest shipped SU(4) table and is the
  case P > 2048 of the engine (element ids beyond 11 bits).  Built from the
  two SU(2) tables (no 4x4 products): Tr(g (x) h) = Tr g Tr h, so
  ReTr = -(Tr g)(Tr h) from the two snapped traces, bit-identical within a
  class and across machines.

Differences from the reference's tables (on purpose):

* element numbering comes from a breadth-first closure, so it differs from the
  reference files; the tables are trace-preserving isomorphic to them (the
  golden-fixture script checks this with an explicit isomorphism);
* every trace is snapped to its closed form (a + b*sqrt5)/4 (real part) and
  sqrt3*(c + d*sqrt5)/4 (imaginary part), evaluated with IEEE double operations
  in a fixed order, so ReTr is bit-identical across all elements of a conjugacy
  class and across machines.  The reference files carry numerical noise of
  ~1e-16 instead (44 distinct ReTr doubles for 11 classes in S(1080)).

The closure is BFS by left multiplication with the generators; row n of the
Cayley table is obtained from its BFS parent's row through the generator's
left-multiplication permutation, so no P^2 matrix products are needed.
"""
from __future__ import annotations

import math
import os
import tempfile
from dataclasses import dataclass

import numpy as np

__all__ = ["GroupTable", "generate", "write_table", "ensure_table", "GROUPS", "PRODUCTS"]


@dataclass
class GroupTable:
    name: str
    P: int
    retr: np.ndarray  # float64 [P]
    imtr: np.ndarray  # float64 [P]
    mult: np.ndarray  # int32 [P, P]
    mats: np.ndarray  # complex128 [P, n, n]


def _s1080_generators():
    w = complex(math.cos(2 * math.pi / 3), math.sin(2 * math.pi / 3))
    up = 0.5 * (-1.0 + math.sqrt(5.0))
    um = 0.5 * (-1.0 - math.sqrt(5.0))
    a = np.array([[0, 1, 0], [0, 0, 1], [1, 0, 0]], complex)
    f = np.diag([1, -1, -1]).astype(complex)
    h = 0.5 * np.array([[-1, um, up], [um, up, -1], [up, -1, um]], complex)
    q = np.array([[-1, 0, 0], [0, 0, -w], [0, -w * w, 0]], complex)
    return [a, f, h, q]


def _quat(a, b, c, d):
    """Unit quaternion a + b i + c j + d k as an SU(2) matrix."""
    return np.array([[a + 1j * d, c + 1j * b], [-c + 1j * b, a - 1j * d]], complex)


def _bi_generators():
    phi = (1 + math.sqrt(5.0)) / 2
    return [_quat(0, 1, 0, 0), _quat(0, 0, 1, 0), _quat(0.5, 0.5, 0.5, 0.5),
            _quat(0.0, 0.5, 0.5 / phi, 0.5 * phi)]


def _bt_generators():
    return [_quat(0, 1, 0, 0), _quat(0, 0, 1, 0), _quat(0.5, 0.5, 0.5, 0.5)]


def _bo_generators():
    r = 1.0 / math.sqrt(2.0)
    return _bt_generators() + [_quat(r, r, 0, 0)]


GROUPS = {"S1080": (_s1080_generators, 1080), "BI": (_bi_generators, 120),
          "BT": (_bt_generators, 24), "BO": (_bo_generators, 48)}
# SU(4) groups built as Kronecker products of two SU(2) groups: (factors, order).
PRODUCTS = {"BIxBO": (("BI", "BO"), 2880)}


def _key(m: np.ndarray) -> bytes:
    return np.round(np.concatenate([m.real.ravel(), m.imag.ravel()]) * 1e6).astype(np.int64).tobytes()


def _snap(x: float, what: str, root: float = 5.0) -> float:
    """Closed form (a + b*sqrt(root))/4 for x, found by bounded integer search."""
    sr = math.sqrt(root)
    for b in range(-8, 9):
        a = round(4 * x - b * sr)
        if abs(a) <= 24 and abs(x - (a + b * sr) / 4.0) < 1e-7:
            return (a + b * sr) / 4.0 + 0.0  # +0.0 turns -0.0 into 0.0
    raise ValueError(f"no closed form for {what} = {x!r}")


def _canonical_traces(mats: np.ndarray, root: float = 5.0):
    s3 = math.sqrt(3.0)
    tr = np.trace(mats, axis1=1, axis2=2)
    retr = np.array([_snap(-t.real, "ReTr", root) for t in tr])
    imtr = np.array([s3 * (_snap(-t.imag / s3, "ImTr/sqrt3", root)) + 0.0 for t in tr])
    return retr, imtr


def _kronecker_product(name: str) -> GroupTable:
    """The group {g (x) h} from the Cayley tables of two SU(2) groups A and B.

    (g, h) and (-g, -h) give the same matrix, so an element is the pair with the
    smaller A index of the two; elements are numbered in (A index, B index)
    order, which puts the identity (0, 0) first."""
    (na, nb), order = PRODUCTS[name]
    A, B = generate(na), generate(nb)
    neg_a = int(np.flatnonzero(np.isclose(A.retr, 2.0))[0])  # -1 in A: ReTr = -Tr = 2
    neg_b = int(np.flatnonzero(np.isclose(B.retr, 2.0))[0])
    negA, negB = A.mult[neg_a], B.mult[neg_b]  # index of -g, -h
    ii, jj = np.meshgrid(np.arange(A.P), np.arange(B.P), indexing="ij")
    keep = ii < negA[ii]  # the representative of {(g, h), (-g, -h)}
    I, J = ii[keep], jj[keep]
    P = I.size
    if P != order:
        raise RuntimeError(f"{name}: {P} elements, expected {order}")
    canon = np.full((A.P, B.P), -1, np.int64)
    canon[I, J] = np.arange(P)
    canon[negA[I], negB[J]] = np.arange(P)
    mult = canon[A.mult[I[:, None], I[None, :]], B.mult[J[:, None], J[None, :]]].astype(np.int32)
    # ReTr = -Tr(g) Tr(h) = -(ReTr_A)(ReTr_B): one IEEE product of two snapped values.
    retr = -(A.retr[I] * B.retr[J]) + 0.0
    imtr = np.zeros(P)
    mats = np.einsum("nab,ncd->nacbd", A.mats[I], B.mats[J]).reshape(P, 4, 4)
    return GroupTable(name, P, retr, imtr, mult, mats)


def generate(name: str) -> GroupTable:
    if name in PRODUCTS:
        return _kronecker_product(name)
    gens_fn, order = GROUPS[name]
    gens = gens_fn()
    n = gens[0].shape[0]
    ident = np.eye(n, dtype=complex)
    elems = [ident]
    index = {_key(ident): 0}
    parent = [-1]
    via = [-1]
    # left[g][j] = index of gens[g] @ elems[j]
    left = [[] for _ in gens]
    j = 0
    while j < len(elems):
        for g, G in enumerate(gens):
            m = G @ elems[j]
            k = _key(m)
            idx = index.get(k)
            if idx is None:
                idx = len(elems)
                index[k] = idx
                elems.append(m)
                parent.append(j)
                via.append(g)
                if idx >= 100000:
                    raise RuntimeError("closure did not terminate")
            left[g].append(idx)
        j += 1
    P = len(elems)
    if P != order:
        raise RuntimeError(f"{name}: closure gave {P} elements, expected {order}")
    left = [np.asarray(l, np.int32) for l in left]
    mult = np.empty((P, P), np.int32)
    mult[0] = np.arange(P, dtype=np.int32)
    for r in range(1, P):  # BFS order: parent row is already filled
        mult[r] = left[via[r]][mult[parent[r]]]
    mats = np.stack(elems)
    retr, imtr = _canonical_traces(mats, root=2.0 if name == "BO" else 5.0)
    return GroupTable(name, P, retr, imtr, mult, mats)


def write_table(tab: GroupTable, path: str) -> None:
    tmp = path + f".tmp{os.getpid()}"
    with open(tmp, "w") as f:
        f.write(f"{tab.P}\n")
        f.write(" ".join(repr(float(x)) for x in tab.retr) + "\n")
        f.write(" ".join(repr(float(x)) for x in tab.imtr) + "\n")
        for row in tab.mult:
            f.write(" ".join(map(str, row.tolist())) + "\n")
        if tab.mats.shape[1] == 3:
            for m in tab.mats:
                f.write(" ".join(repr(float(v)) for z in m.ravel() for v in (z.real, z.imag)) + "\n")
    os.replace(tmp, path)


def default_cache_dir() -> str:
    d = os.environ.get("DYM_TABLE_DIR")
    if d:
        return d
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "_tables")


def ensure_table(name: str, cache_dir: str | None = None) -> str:
    """Path of the generated table file for `name`, generating it on first use."""
    cache_dir = cache_dir or default_cache_dir()
    os.makedirs(cache_dir, exist_ok=True)
    path = os.path.join(cache_dir, "v2", name)  # v2: SU(3) matrices appended
    os.makedirs(os.path.dirname(path), exist_ok=True)
    if not os.path.exists(path):
        write_table(generate(name), path)
    return path


if __name__ == "__main__":
    import sys
    out = sys.argv[2] if len(sys.argv) > 2 else None
    print(ensure_table(sys.argv[1], out))
