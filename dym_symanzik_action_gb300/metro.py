"""Python host interface mirroring the reference's Metropolis program.

The reference (hlammiv/dym_symanzik_action) keeps its state in globals:
group.h:8-16 (P, ReTr, ImTr, mult, inv, id, load_group) and lattice.h:7-16
(D, Nt, Nx, V, beta0..2, the link array `a`), and drives them with update()
and the measurement block of dym-mod-metro.cpp:146-337.  Here the same state
lives in two handles of libdymgpu: a Group (load_group) and a Lattice (one
Markov chain on the GPU).  Names, argument meaning and error behaviour follow
the reference; errors raise DymError instead of aborting.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import check, lib, ptr


class Group:
    """A finite group read from a Cayley-table file (load_group, group.c:13-98)."""

    def __init__(self, path: str):
        h = C.c_void_p()
        check(lib().dym_group_load(str(path).encode(), C.byref(h)))
        self._h = h
        info = _lib.GroupInfo()
        check(lib().dym_group_get_info(h, C.byref(info)))
        self.path = str(path)
        self.P = int(info.order)
        self.id = int(info.identity)
        self.min_retr = float(info.min_retr)
        self.nn_retr = float(info.nn_retr)
        self.n_classes = int(info.n_classes)
        self.classes_exact = bool(info.classes_exact)
        self.fast_path = bool(info.fast_path)
        self.class_spread = float(info.class_spread)
        self._npool = int(info.pool_nearest)
        self._tables = None

    def _load_tables(self):
        if self._tables is None:
            P = self.P
            mult = np.zeros((P, P), np.int32)
            inv = np.zeros(P, np.int32)
            re = np.zeros(P)
            im = np.zeros(P)
            pool = np.zeros(max(self._npool, 1), np.int32)
            check(lib().dym_group_get_tables(self._h, ptr(mult, C.c_int32), ptr(inv, C.c_int32),
                                             ptr(re, C.c_double), ptr(im, C.c_double), ptr(pool, C.c_int32)))
            self._tables = (mult, inv, re, im, pool[: self._npool])
        return self._tables

    @property
    def mult(self) -> np.ndarray:
        return self._load_tables()[0]

    @property
    def inv(self) -> np.ndarray:
        return self._load_tables()[1]

    @property
    def ReTr(self) -> np.ndarray:
        return self._load_tables()[2]

    @property
    def ImTr(self) -> np.ndarray:
        return self._load_tables()[3]

    @property
    def smallgroup(self) -> np.ndarray:
        """Proposal pool nearest the identity (dym-mod-metro.cpp:239-245)."""
        return self._load_tables()[4]

    @property
    def table_hash(self) -> int:
        """FNV-1a 64 of the Cayley table, as checkpoints record it."""
        h = C.c_uint64()
        check(lib().dym_group_table_hash(self._h, C.byref(h)))
        return h.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().dym_group_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def load_group(path: str) -> Group:
    return Group(path)


def checkpoint_info(path: str) -> dict:
    """Header of a chain checkpoint file (dym_checkpoint_read_info; host only)."""
    h = _lib.CheckpointInfo()
    check(lib().dym_checkpoint_read_info(str(path).encode(), C.byref(h)))
    return {k: getattr(h, k) for k, _ in h._fields_}


@dataclass
class Measurement:
    """One GMES/RMES record (dym-mod-metro.cpp:282-329)."""
    poly_re: float
    poly_im: float
    plaq: float
    rect: float
    wloop: np.ndarray = field(repr=False)  # [wl_nx, wl_nt], spatial extent outer

    def gmes_line(self) -> str:
        s = "GMES: %e %e %e %e" % (999.0, self.poly_re, self.poly_im, self.plaq)
        return s + "".join(" %e" % w for w in self.wloop.ravel())

    def rmes_line(self) -> str:
        return "RMES: %e %e" % (self.plaq, self.rect)


@dataclass
class LlrResult:
    """One LLR window (seed_window + rm_solve, llr.cpp:223-250)."""
    a: float
    S1: float
    S2: float
    status: str
    drive_sweeps: int
    sweeps: int
    hits: int
    accepts: int
    phase_accepts: int
    phase_rejects: int
    a_hist: np.ndarray = field(repr=False)


@dataclass
class Llr2dResult:
    """One two-dimensional LLR cell (seed_cell + rm_solve2d, llr2d.cpp:225-259)."""
    a1: float
    a2: float
    S1: float
    S2: float
    status: str
    drive_sweeps: int
    sweeps: int
    hits: int
    accepts: int
    phase_accepts: int
    phase_rejects: int
    a_hist: np.ndarray = field(repr=False)  # [NRM, 2]: (a1, a2) after each iteration


@dataclass
class SweepStats:
    hits: int
    accepts: int
    rechecks: int
    max_ds_err: float
    sweep: int
    launches: int
    device_ms: float
    kernel: int = 0  # DYM_KERNEL_*: 1 direct, 2 shared, 3 mixed, 4 mixed with the value table


class Lattice:
    """One Markov chain on the device: the reference's lattice globals, the
    per-site RNG state (here a Philox key and sweep counter) and the start
    configuration (dym-mod-metro.cpp:221-268)."""

    def __init__(self, group: Group, D: int, Nt: int, Nx: int, beta0: float, beta1: float, beta2: float,
                 seed: int, start: str = "hot", pool: str = "nearest", precision: str = "mixed", device: int = 0):
        p = _lib.ChainParams(D=D, Nt=Nt, Nx=Nx, beta0=beta0, beta1=beta1, beta2=beta2, seed=seed & (2**64 - 1),
                             start=_lib.START[start], pool=_lib.POOL[pool], precision=_lib.PRECISION[precision],
                             device=device)
        h = C.c_void_p()
        check(lib().dym_chain_create(group._h, C.byref(p), C.byref(h)))
        self._h = h
        self.group = group
        self.D, self.Nt, self.Nx = D, Nt, Nx
        self.V = Nt * Nx ** (D - 1)
        self.beta = (beta0, beta1, beta2)
        self.seed = seed
        self.start, self.pool, self.precision = start, pool, precision
        self.hit = 0  # running counters, as the reference's globals hit/acc
        self.acc = 0
        self.rechecks = 0
        self.max_ds_err = 0.0
        self.sweeps = 0

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().dym_chain_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_beta(self, beta0: float, beta1: float, beta2: float) -> None:
        check(lib().dym_chain_set_beta(self._h, beta0, beta1, beta2))
        self.beta = (beta0, beta1, beta2)

    def set_l2_window(self, on: bool = True) -> None:
        """Pin the group's Cayley table in L2 for this chain's kernels (an
        access-policy window on the chain's stream); opt-in, results unchanged."""
        check(lib().dym_chain_set_l2_window(self._h, 1 if on else 0))

    def save_checkpoint(self, path: str) -> None:
        """Links, seed, sweeps done and couplings to `path`; a chain loaded
        from it continues bit for bit (dym_chain_checkpoint_save)."""
        check(lib().dym_chain_checkpoint_save(self._h, str(path).encode()))

    def load_checkpoint(self, path: str) -> None:
        """Resume from a checkpoint of a chain with the same shape, pool and
        group table (dym_chain_checkpoint_load)."""
        check(lib().dym_chain_checkpoint_load(self._h, str(path).encode()))
        info = checkpoint_info(path)
        self.seed = info["seed"]
        self.beta = (info["beta0"], info["beta1"], info["beta2"])

    def update(self, nsweeps: int = 1, nhit: int = 20) -> SweepStats:
        """nsweeps calls of the reference's update() (dym-mod-metro.cpp:146-197)."""
        st = _lib.Stats()
        check(lib().dym_sweep(self._h, nsweeps, nhit, C.byref(st)))
        self.hit += st.hits
        self.acc += st.accepts
        self.rechecks += st.rechecks
        self.max_ds_err = max(self.max_ds_err, st.max_ds_err)
        self.sweeps = st.sweep
        return SweepStats(st.hits, st.accepts, st.rechecks, st.max_ds_err, st.sweep, st.launches, st.device_ms,
                          st.kernel)

    def update_host(self, links_in, links_out=None, nsweeps: int = 1, nhit: int = 20) -> SweepStats:
        """update() on a configuration held in host memory (dym_sweep_host):
        links_in (uint16, D*V entries, or None to keep the chain's) is
        uploaded and checked, nsweeps sweeps run, and the result is written
        into links_out (or not read back when None), with one synchronisation.
        Both must be C-contiguous uint16 arrays; page-locked ones (e.g. from
        torch's pin_memory) are read and written without a staging copy."""
        n = self.D * self.V
        for x in (links_in, links_out):
            if x is not None and (x.dtype != np.uint16 or x.size != n or not x.flags["C_CONTIGUOUS"]):
                raise ValueError("links must be C-contiguous uint16 arrays of D*V entries")
        if links_out is not None and not links_out.flags["WRITEABLE"]:
            raise ValueError("links_out must be writeable")
        st = _lib.Stats()
        check(lib().dym_sweep_host(self._h, None if links_in is None else ptr(links_in, C.c_uint16),
                                   None if links_out is None else ptr(links_out, C.c_uint16), nsweeps, nhit,
                                   C.byref(st)))
        self.hit += st.hits
        self.acc += st.accepts
        self.rechecks += st.rechecks
        self.max_ds_err = max(self.max_ds_err, st.max_ds_err)
        self.sweeps = st.sweep
        return SweepStats(st.hits, st.accepts, st.rechecks, st.max_ds_err, st.sweep, st.launches, st.device_ms,
                          st.kernel)

    def update_refarray(self, a: np.ndarray, nsweeps: int = 1, nhit: int = 20) -> SweepStats:
        """update() applied in place to a link array in the reference's layout
        (dym_sweep_refarray): `a` is int32 with a[i*D + d] the id of link
        (site i, direction d), C-contiguous and writeable."""
        if a.dtype != np.int32 or a.size != self.D * self.V or not a.flags["C_CONTIGUOUS"] or \
                not a.flags["WRITEABLE"]:
            raise ValueError("a must be a writeable C-contiguous int32 array of V*D entries")
        st = _lib.Stats()
        check(lib().dym_sweep_refarray(self._h, ptr(a, C.c_int32), nsweeps, nhit, C.byref(st)))
        self.hit += st.hits
        self.acc += st.accepts
        self.rechecks += st.rechecks
        self.max_ds_err = max(self.max_ds_err, st.max_ds_err)
        self.sweeps = st.sweep
        return SweepStats(st.hits, st.accepts, st.rechecks, st.max_ds_err, st.sweep, st.launches, st.device_ms,
                          st.kernel)

    def measure(self, wl_nx: int = 0, wl_nt: int = 0) -> Measurement:
        """Observables (dym-mod-metro.cpp:282-318); wl_nx/wl_nt 0 = full Nx x Nt
        grid as the reference, -1 = no Wilson grid."""
        nx = self.Nx if wl_nx == 0 else max(wl_nx, 0)
        nt = self.Nt if wl_nt == 0 else max(wl_nt, 0)
        if wl_nx < 0 or wl_nt < 0:
            nx = nt = 0
        w = np.zeros(max(nx * nt, 1))
        o = _lib.Obs()
        opts = _lib.MeasOpts(wl_nx=wl_nx, wl_nt=wl_nt)
        check(lib().dym_measure(self._h, C.byref(opts), C.byref(o), ptr(w, C.c_double)))
        return Measurement(o.poly_re, o.poly_im, o.plaq, o.rect, w[: o.wl_nx * o.wl_nt].reshape(o.wl_nx, o.wl_nt))

    @property
    def links(self) -> np.ndarray:
        """Configuration as uint16 [D, V] (direction-major)."""
        out = np.zeros(self.D * self.V, np.uint16)
        check(lib().dym_links_get(self._h, ptr(out, C.c_uint16)))
        return out.reshape(self.D, self.V)

    @links.setter
    def links(self, value: np.ndarray) -> None:
        v = np.ascontiguousarray(value, np.uint16).ravel()
        if v.size != self.D * self.V:
            raise ValueError("links must hold D*V entries")
        check(lib().dym_links_set(self._h, ptr(v, C.c_uint16)))

    def staples(self, d: int, sites) -> np.ndarray:
        """[n, 8(D-1)]: get_staples then get_rect_loops of links (site, d)."""
        s = np.ascontiguousarray(sites, np.uint32)
        out = np.zeros((s.size, 8 * (self.D - 1)), np.uint16)
        check(lib().dym_chain_staples(self._h, d, ptr(s, C.c_uint32), s.size, ptr(out, C.c_uint16)))
        return out

    def llr_energy(self):
        """(S1, S2): exact plaquette and rectangle action sums (llr.cpp:46-55, 139-151)."""
        s1, s2 = C.c_double(), C.c_double()
        check(lib().dym_llr_energy(self._h, C.byref(s1), C.byref(s2)))
        return s1.value, s2.value

    def llr_run(self, ewin: float, hw: float, a0: float, axis: int = 1, bg: float = 0.0, K: int = 50,
                NRM: int = 80, nhit: int = 20, drive_cap: int = 20000) -> LlrResult:
        """Drive into [ewin-hw, ewin+hw], then NRM Robbins-Monro iterations of K
        constrained sweeps (llr.cpp:223-250); defaults are llr.cpp's."""
        req = _lib.LlrReq(axis=axis, bg=bg, ewin=ewin, hw=hw, a0=a0, K=K, NRM=NRM, nhit=nhit, drive_cap=drive_cap)
        res = _lib.LlrResult()
        hist = np.zeros(max(NRM, 1))
        check(lib().dym_llr_run(self._h, C.byref(req), C.byref(res), ptr(hist, C.c_double)))
        return LlrResult(res.a, res.S1, res.S2, _lib.LLR_STATUS.get(res.status, str(res.status)), res.drive_sweeps,
                         res.sweeps, res.hits, res.accepts, res.phase_accepts, res.phase_rejects, hist[:NRM].copy())

    def llr2d_run(self, E1: float, hw1: float, E2: float, hw2: float, a1: float, a2: float, K: int = 40,
                  NRM: int = 70, nhit: int = 20, drive_cap: int = 4000) -> Llr2dResult:
        """Drive (S1, S2) into the cell [E1 +- hw1] x [E2 +- hw2], then NRM pairs of
        Robbins-Monro iterations of K constrained sweeps (llr2d.cpp:225-259);
        defaults are llr2d.cpp's (K 40, NRM 70, drive-in cap 4000)."""
        req = _lib.Llr2dReq(E1=E1, hw1=hw1, E2=E2, hw2=hw2, a1=a1, a2=a2, K=K, NRM=NRM, nhit=nhit,
                            drive_cap=drive_cap)
        res = _lib.Llr2dResult()
        hist = np.zeros(2 * max(NRM, 1))
        check(lib().dym_llr2d_run(self._h, C.byref(req), C.byref(res), ptr(hist, C.c_double)))
        return Llr2dResult(res.a1, res.a2, res.S1, res.S2, _lib.LLR_STATUS.get(res.status, str(res.status)),
                           res.drive_sweeps, res.sweeps, res.hits, res.accepts, res.phase_accepts, res.phase_rejects,
                           hist[: 2 * NRM].reshape(NRM, 2).copy())

    def schedule(self):
        V = C.c_uint32()
        n = C.c_int32()
        check(lib().dym_chain_get_schedule(self._h, C.byref(V), C.byref(n), None, None, None))
        pd = np.zeros(n.value, np.int32)
        pl = np.zeros(n.value, np.uint32)
        sites = np.zeros(self.V * self.D, np.uint32)
        check(lib().dym_chain_get_schedule(self._h, None, None, ptr(pd, C.c_int32), ptr(pl, C.c_uint32),
                                           ptr(sites, C.c_uint32)))
        return pd, pl, sites
