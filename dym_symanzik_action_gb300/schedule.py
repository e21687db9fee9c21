"""Host access to the race-free colour schedule (no device needed)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, lib, ptr


def schedule(D: int, Nt: int, Nx: int):
    """(phase_dir int32[nphase], phase_len uint32[nphase], sites uint32[V*D])."""
    V = C.c_uint32()
    n = C.c_int32()
    check(lib().dym_schedule_get(D, Nt, Nx, C.byref(V), C.byref(n), None, None, None))
    pd = np.zeros(n.value, np.int32)
    pl = np.zeros(n.value, np.uint32)
    sites = np.zeros(V.value * D, np.uint32)
    check(lib().dym_schedule_get(D, Nt, Nx, None, None, ptr(pd, C.c_int32), ptr(pl, C.c_uint32),
                                 ptr(sites, C.c_uint32)))
    return pd, pl, sites


def conflicts(D: int, Nt: int, Nx: int) -> tuple[int, int]:
    """(number of phases, same-phase conflicts found by the library's own check)."""
    n = C.c_int32()
    c = C.c_uint64()
    check(lib().dym_schedule_check(D, Nt, Nx, C.byref(n), C.byref(c)))
    return n.value, c.value
