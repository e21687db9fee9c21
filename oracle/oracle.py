"""ctypes loader of the oracle (oracle/dym_oracle.c) -- test infrastructure.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, as the checker or the timed CPU baseline; the engine never does.
"""
from __future__ import annotations

import ctypes as C
import os
import re
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "dym_oracle.c")
OUT = os.path.join(HERE, "_build", "liboracle.so")
CORE = os.path.join(os.path.dirname(HERE), "dym_symanzik_action_gb300", "csrc", "dym_core.h")
REF_LIB = os.path.join(HERE, "_ref", "libdymref.so")
REF_BIN = os.path.join(HERE, "_ref")
STAGED_REF = os.path.join(os.path.dirname(HERE), "baseline", "_ref")


def ref_dir():
    """The reference sources to build the checkers from: $REF_DIR, or else
    baseline/_ref (filled by oracle/stage_ref.sh); None when neither holds
    dym-mod-metro.cpp."""
    for cand in (os.environ.get("REF_DIR"), STAGED_REF):
        if cand and os.path.isfile(os.path.join(cand, "dym-mod-metro.cpp")):
            return cand
    return None


def build() -> str:
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if (not os.path.exists(OUT) or os.path.getmtime(OUT) < max(os.path.getmtime(SRC), os.path.getmtime(CORE))):
        cmd = ["gcc", "-O2", "-std=gnu99", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-Wall",
               SRC, "-o", OUT + ".tmp"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode:
            raise RuntimeError("oracle build failed:\n" + r.stdout)
        os.replace(OUT + ".tmp", OUT)
    return OUT


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        l = C.CDLL(build())
        vp, i, u32, u64, d = C.c_void_p, C.c_int, C.c_uint32, C.c_uint64, C.c_double
        P = C.POINTER
        sig = {
            "or_group_load": (i, [C.c_char_p, P(vp)]),
            "or_group_free": (None, [vp]),
            "or_group_order": (i, [vp]),
            "or_group_identity": (i, [vp]),
            "or_group_pool": (i, [vp, P(C.c_int)]),
            "or_group_tables": (None, [vp, P(C.c_int), P(C.c_int), P(d), P(d)]),
            "or_lattice_create": (i, [vp, i, i, i, P(vp)]),
            "or_lattice_free": (None, [vp]),
            "or_lattice_volume": (C.c_uint, [vp]),
            "or_set_links": (None, [vp, P(C.c_uint16)]),
            "or_get_links": (None, [vp, P(C.c_uint16)]),
            "or_hot_start": (None, [vp, u64]),
            "or_staples": (None, [vp, C.c_uint, C.c_uint, P(C.c_int), P(C.c_int)]),
            "or_schedule_conflicts": (u64, [vp, P(C.c_int), P(u32), P(u32), i]),
            "or_sweep": (None, [vp, P(C.c_int), P(u32), P(u32), i, d, d, d, u64, u32, i, i, i, P(u64), i]),
            "or_measure": (None, [vp, i, i, P(d), P(u64)]),
            "or_philox": (None, [P(u32), P(u32), P(u32)]),
            "or_exp": (d, [d]),
            "or_pick": (u32, [u32, u32]),
            "or_llr_run": (i, [vp, P(C.c_int), P(u32), P(u32), i, i, d, d, d, d, i, i, i, i, u64, u32, P(d),
                               P(C.c_int64), P(d)]),
            "or_llr2d_run": (i, [vp, P(C.c_int), P(u32), P(u32), i, d, d, d, d, d, d, i, i, i, i, u64, u32, P(d),
                                 P(C.c_int64), P(d), P(d)]),
            "or_energies": (None, [vp, P(d), P(d)]),
        }
        for name, (res, args) in sig.items():
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


def _p(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


class OracleGroup:
    def __init__(self, path: str):
        h = C.c_void_p()
        rc = lib().or_group_load(path.encode(), C.byref(h))
        if rc:
            raise ValueError(f"oracle: cannot load group {path} (code {rc})")
        self.h = h
        self.P = lib().or_group_order(h)
        self.id = lib().or_group_identity(h)
        pool = np.zeros(self.P, np.int32)
        n = lib().or_group_pool(h, _p(pool, C.c_int))
        self.pool = pool[:n].copy()

    def tables(self):
        P = self.P
        mult = np.zeros((P, P), np.int32)
        inv = np.zeros(P, np.int32)
        re = np.zeros(P)
        im = np.zeros(P)
        lib().or_group_tables(self.h, _p(mult, C.c_int), _p(inv, C.c_int), _p(re, C.c_double), _p(im, C.c_double))
        return mult, inv, re, im

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.or_group_free(self.h)
            self.h = None


class OracleLattice:
    """Reference-layout lattice driven in the engine's colour phases."""

    def __init__(self, group: OracleGroup, D: int, Nt: int, Nx: int):
        h = C.c_void_p()
        if lib().or_lattice_create(group.h, D, Nt, Nx, C.byref(h)):
            raise ValueError("oracle: bad lattice shape")
        self.h, self.group, self.D, self.Nt, self.Nx = h, group, D, Nt, Nx
        self.V = lib().or_lattice_volume(h)
        self.hits = 0
        self.accepts = 0

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.or_lattice_free(self.h)
            self.h = None

    @property
    def links(self) -> np.ndarray:
        out = np.zeros(self.V * self.D, np.uint16)
        lib().or_get_links(self.h, _p(out, C.c_uint16))
        return out

    @links.setter
    def links(self, dm: np.ndarray) -> None:
        dm = np.ascontiguousarray(dm, np.uint16)
        assert dm.size == self.V * self.D
        lib().or_set_links(self.h, _p(dm, C.c_uint16))

    def hot_start(self, seed: int) -> None:
        lib().or_hot_start(self.h, seed)

    def staples(self, i: int, d: int):
        st = np.zeros(2 * (self.D - 1), np.int32)
        re = np.zeros(6 * (self.D - 1), np.int32)
        lib().or_staples(self.h, i, d, _p(st, C.c_int), _p(re, C.c_int))
        return st, re

    def conflicts(self, sched) -> int:
        pd, pl, sites = sched
        return int(lib().or_schedule_conflicts(self.h, _p(pd, C.c_int), _p(pl, C.c_uint32), _p(sites, C.c_uint32),
                                               len(pd)))

    def sweep(self, sched, beta, seed, first_sweep, nsweeps, nhit, pool_all=False, nthreads=0):
        pd, pl, sites = sched
        ctr = np.zeros(2, np.uint64)
        lib().or_sweep(self.h, _p(pd, C.c_int), _p(pl, C.c_uint32), _p(sites, C.c_uint32), len(pd),
                       float(beta[0]), float(beta[1]), float(beta[2]), seed, first_sweep, nsweeps, nhit,
                       1 if pool_all else 0, _p(ctr, C.c_uint64), nthreads)
        self.hits += int(ctr[0])
        self.accepts += int(ctr[1])
        return int(ctr[0]), int(ctr[1])

    def energies(self):
        s1, s2 = C.c_double(), C.c_double()
        lib().or_energies(self.h, C.byref(s1), C.byref(s2))
        return s1.value, s2.value

    def llr_run(self, sched, ewin, hw, a0, axis=1, bg=0.0, K=50, NRM=80, nhit=20, drive_cap=20000, seed=0,
                first_sweep=0):
        pd, pl, sites = sched
        out = np.zeros(4)
        iout = np.zeros(6, np.int64)
        hist = np.zeros(max(NRM, 1))
        rc = lib().or_llr_run(self.h, _p(pd, C.c_int), _p(pl, C.c_uint32), _p(sites, C.c_uint32), len(pd), axis,
                              float(bg), float(ewin), float(hw), float(a0), K, NRM, nhit, drive_cap, seed, first_sweep,
                              _p(out, C.c_double), _p(iout, C.c_int64), _p(hist, C.c_double))
        if rc:
            raise ValueError(f"oracle llr failed ({rc})")
        status = {0: "drive", 1: "settle", 2: "rm", 3: "done", 4: "unreached"}[int(out[3])]
        return dict(a=out[0], S1=out[1], S2=out[2], status=status, drive_sweeps=int(iout[0]), sweeps=int(iout[1]),
                    hits=int(iout[2]), accepts=int(iout[3]), phase_accepts=int(iout[4]),
                    phase_rejects=int(iout[5]), a_hist=hist[:NRM].copy())

    def llr2d_run(self, sched, E1, hw1, E2, hw2, a1, a2, K=40, NRM=70, nhit=20, drive_cap=4000, seed=0,
                  first_sweep=0):
        """Two-dimensional cell with the colour-parallel rule (llr2d.cpp:178-259)."""
        pd, pl, sites = sched
        out = np.zeros(5)
        iout = np.zeros(6, np.int64)
        h1 = np.zeros(max(NRM, 1))
        h2 = np.zeros(max(NRM, 1))
        rc = lib().or_llr2d_run(self.h, _p(pd, C.c_int), _p(pl, C.c_uint32), _p(sites, C.c_uint32), len(pd),
                                float(E1), float(hw1), float(E2), float(hw2), float(a1), float(a2), K, NRM, nhit,
                                drive_cap, seed, first_sweep, _p(out, C.c_double), _p(iout, C.c_int64),
                                _p(h1, C.c_double), _p(h2, C.c_double))
        if rc:
            raise ValueError(f"oracle llr2d failed ({rc})")
        status = {0: "drive", 1: "settle", 2: "rm", 3: "done", 4: "unreached"}[int(out[3])]
        return dict(a1=out[0], a2=out[4], S1=out[1], S2=out[2], status=status, drive_sweeps=int(iout[0]),
                    sweeps=int(iout[1]), hits=int(iout[2]), accepts=int(iout[3]), phase_accepts=int(iout[4]),
                    phase_rejects=int(iout[5]), a_hist=np.stack([h1[:NRM], h2[:NRM]], axis=1))

    def measure(self, wl_nx: int, wl_nt: int, want_hist: bool = False):
        out = np.zeros(4 + max(wl_nx, 0) * max(wl_nt, 0))
        hist = np.zeros((3 + max(wl_nx, 0) * max(wl_nt, 0)) * self.group.P, np.uint64) if want_hist else None
        lib().or_measure(self.h, wl_nx, wl_nt, _p(out, C.c_double), _p(hist, C.c_uint64))
        return (out, hist) if want_hist else out


def _conflict_offsets(D: int, d: int):
    """Same-direction links read by the update of link (x, d) (the staple index
    sets of dym-mod-metro.cpp:63-142): +-e_d, +-e_a, +-2e_a, +-e_d +-e_a."""
    out = []
    for s in (-1, 1):
        v = [0] * D
        v[d] = s
        out.append(v)
    for a in range(D):
        if a == d:
            continue
        for s in (-2, -1, 1, 2):
            v = [0] * D
            v[a] = s
            out.append(v)
        for sd in (-1, 1):
            for sa in (-1, 1):
                v = [0] * D
                v[d], v[a] = sd, sa
                out.append(v)
    return out


def colour_schedule(D: int, Nt: int, Nx: int):
    """The race-free colour-phase schedule, restated in plain Python for the
    CPU legs that must not load the engine: per direction the linear colouring
    colour = (sum_b w_b x_b) mod m with the smallest m <= 24 and the first
    periodic weights (axis 0 fastest) for which every conflicting offset that
    names another site changes the colour, else a greedy colouring in site
    order; phases are the non-empty colour classes in colour order, sites
    ascending.  Returns (phase_dir int32, phase_len uint32, sites uint32)."""
    ext = [Nt] + [Nx] * (D - 1)
    V = int(np.prod(ext))
    idx = np.arange(V)
    coords = []
    rem = idx.copy()
    for b in range(D):
        coords.append(rem % ext[b])
        rem //= ext[b]
    coords = np.stack(coords, 1)
    strides = np.cumprod([1] + ext[:-1])
    pd, pl, sites = [], [], []
    for d in range(D):
        offs = _conflict_offsets(D, d)
        need = [v for v in offs if any(v[b] % ext[b] for b in range(D))]
        colour, ncol = None, 0
        for m in range(2, 25):
            cand = [[w for w in range(m) if (ext[b] * w) % m == 0] for b in range(D)]
            found = None
            for wi in np.ndindex(*[len(c) for c in reversed(cand)]):
                w = [cand[b][wi[D - 1 - b]] for b in range(D)]
                if all(sum(w[b] * v[b] for b in range(D)) % m for v in need):
                    found = w
                    break
            if found is not None:
                colour, ncol = (coords @ np.array(found)) % m, m
                break
        if colour is None:
            colour = -np.ones(V, np.int64)
            for i in range(V):
                used = set()
                for v in offs:
                    j = int((((coords[i] + v) % ext) * strides).sum())
                    if j != i and colour[j] >= 0:
                        used.add(int(colour[j]))
                c = 0
                while c in used:
                    c += 1
                colour[i] = c
            ncol = int(colour.max()) + 1
        for c in range(ncol):
            lst = idx[colour == c]
            if len(lst):
                pd.append(d)
                pl.append(len(lst))
                sites.append(lst)
    return (np.array(pd, np.int32), np.array(pl, np.uint32), np.concatenate(sites).astype(np.uint32))


# TM_END line of the reference's timer (timer.cpp:19-26) around the K
# update() calls of one measurement block (dym-mod-metro.cpp:273-278).
_TM_UPDATE = re.compile(r"^TM_END:\s+update\s.*done in\s+([0-9.eE+-]+)\s+sec", re.M)


def run_reference_metro(table: str, D: int, Nt: int, Nx: int, beta, seed: int, K: int, N: int, Ntherm: int,
                        start: str = "hot", nhit10: bool = True, threads: int | None = None, timeout: float = 1800):
    """Run the unmodified reference executable (oracle/_ref/dym-mod-metro, or
    its NHIT = 10 build) and return (stdout, [seconds of every TM_END update
    block]).  It runs in a scratch directory (the -pg build writes gmon.out
    into its working directory) with OMP_NUM_THREADS = threads (all host cores
    by default)."""
    exe = os.path.join(REF_BIN, "dym-mod-metro-nhit10" if nhit10 else "dym-mod-metro")
    if not os.path.exists(exe):
        raise FileNotFoundError(exe)
    env = dict(os.environ, OMP_NUM_THREADS=str(threads or os.cpu_count() or 1))
    args = [exe, table, str(D), str(Nt), str(Nx), *(repr(float(b)) for b in beta), str(seed), str(K), str(N),
            str(Ntherm), start]
    with tempfile.TemporaryDirectory() as td:
        r = subprocess.run(args, cwd=td, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                           timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"reference dym-mod-metro failed ({r.returncode}):\n{r.stdout[-2000:]}")
    return r.stdout, [float(x) for x in _TM_UPDATE.findall(r.stdout)]


class RefHarness:
    """The reference's own functions (oracle/_ref/libdymref.so, built here from
    the reference sources by oracle/build_ref.sh); one lattice per process."""

    def __init__(self):
        if not os.path.exists(REF_LIB):
            raise FileNotFoundError(REF_LIB)
        l = C.CDLL(REF_LIB)
        P = C.POINTER
        l.refh_init.restype = C.c_int
        l.refh_init.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int]
        l.refh_set_links.argtypes = [P(C.c_uint16)]
        l.refh_get_links.argtypes = [P(C.c_uint16)]
        l.refh_staples.argtypes = [C.c_uint, C.c_uint, P(C.c_int), P(C.c_int)]
        l.refh_sweep.argtypes = [P(C.c_int), P(C.c_uint32), P(C.c_uint32), C.c_int, C.c_double, C.c_double,
                                 C.c_double, C.c_uint64, C.c_uint32, C.c_int, C.c_int, C.c_int, P(C.c_uint64)]
        l.refh_measure.argtypes = [C.c_int, C.c_int, P(C.c_double)]
        self.l = l

    def init(self, path, D, Nt, Nx):
        self.D, self.Nt, self.Nx = D, Nt, Nx
        self.V = Nt * Nx ** (D - 1)
        return self.l.refh_init(path.encode(), D, Nt, Nx)

    def set_links(self, dm):
        dm = np.ascontiguousarray(dm, np.uint16)
        self.l.refh_set_links(_p(dm, C.c_uint16))

    def get_links(self):
        out = np.zeros(self.V * self.D, np.uint16)
        self.l.refh_get_links(_p(out, C.c_uint16))
        return out

    def staples(self, i, d):
        st = np.zeros(2 * (self.D - 1), np.int32)
        re = np.zeros(6 * (self.D - 1), np.int32)
        self.l.refh_staples(i, d, _p(st, C.c_int), _p(re, C.c_int))
        return st, re

    def sweep(self, sched, beta, seed, first_sweep, nsweeps, nhit, pool_all=False):
        pd, pl, sites = sched
        ctr = np.zeros(2, np.uint64)
        self.l.refh_sweep(_p(pd, C.c_int), _p(pl, C.c_uint32), _p(sites, C.c_uint32), len(pd), float(beta[0]),
                          float(beta[1]), float(beta[2]), seed, first_sweep, nsweeps, nhit, 1 if pool_all else 0,
                          _p(ctr, C.c_uint64))
        return int(ctr[0]), int(ctr[1])

    def measure(self, wl_nx, wl_nt):
        out = np.zeros(4 + wl_nx * wl_nt)
        self.l.refh_measure(wl_nx, wl_nt, _p(out, C.c_double))
        return out
