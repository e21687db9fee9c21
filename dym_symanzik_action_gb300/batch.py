"""Batched ensemble of independent chains (many lattices of uneven size).

The reference runs one process per chain (evermore.sh, jobs2run); here the
chains stay separate Lattice objects, and a Batch updates all of them with one
kernel per colour-phase slot, replayed as a CUDA graph.  Every chain's
configuration is bit-identical to running it alone with Lattice.update.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

from . import _lib
from ._lib import check, lib
from .metro import Lattice, SweepStats


@dataclass
class Tuning:
    tile: int = 256
    threads: int = 256
    grid_per_sm: int = 1
    use_graph: bool = True
    hit_unroll: int = 1


class Batch:
    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().dym_batch_create(device, C.byref(h)))
        self._h = h
        self.chains: list[Lattice] = []

    def add(self, lat: Lattice) -> None:
        check(lib().dym_batch_add(self._h, lat._h))
        self.chains.append(lat)

    @property
    def size(self):
        n, links, slots = C.c_int32(), C.c_uint64(), C.c_int32()
        check(lib().dym_batch_size(self._h, C.byref(n), C.byref(links), C.byref(slots)))
        return n.value, links.value, slots.value

    @property
    def tuning(self) -> Tuning:
        t = _lib.BatchTuning()
        check(lib().dym_batch_get_tuning(self._h, C.byref(t)))
        return Tuning(t.tile, t.threads, t.grid_per_sm, bool(t.use_graph), t.hit_unroll or 1)

    @tuning.setter
    def tuning(self, t: Tuning) -> None:
        bt = _lib.BatchTuning(tile=t.tile, threads=t.threads, grid_per_sm=t.grid_per_sm, use_graph=int(t.use_graph),
                              hit_unroll=t.hit_unroll)
        check(lib().dym_batch_set_tuning(self._h, C.byref(bt)))

    def update(self, nsweeps: int = 1, nhit: int = 20) -> SweepStats:
        st = _lib.Stats()
        check(lib().dym_batch_sweep(self._h, nsweeps, nhit, C.byref(st)))
        for lat in self.chains:
            lat.sweeps += nsweeps
        return SweepStats(st.hits, st.accepts, st.rechecks, st.max_ds_err, st.sweep, st.launches, st.device_ms)

    def chain_counters(self, idx: int):
        h, a = C.c_uint64(), C.c_uint64()
        check(lib().dym_batch_chain_counters(self._h, idx, C.byref(h), C.byref(a)))
        return h.value, a.value

    def autotune(self, nhit: int = 10, nsweeps_per_trial: int = 2) -> Tuning:
        t = _lib.BatchTuning()
        check(lib().dym_batch_autotune(self._h, nhit, nsweeps_per_trial, C.byref(t)))
        return Tuning(t.tile, t.threads, t.grid_per_sm, bool(t.use_graph), t.hit_unroll or 1)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().dym_batch_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
