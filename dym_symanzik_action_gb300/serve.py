"""Request server for LLR windows (continuous batching on one GPU).

Requests are queued with submit(); every step() admits queued requests while
the resident-chain count and the device-memory budget allow, runs LLR sweeps
of all resident chains together, and retires finished ones, whose responses
poll() returns.  A request's result does not depend on what else is resident.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import check, lib
from .metro import Group


@dataclass
class Response:
    id: int
    a: float
    S1: float
    S2: float
    status: str
    sweeps: int
    drive_sweeps: int
    hits: int
    accepts: int
    a_hist: np.ndarray


class Server:
    def __init__(self, group: Group, max_chains: int = 64, hbm_budget: int = 8 << 30, nhit: int = 20,
                 device: int = 0, max_links: int = 0):
        p = _lib.ServerParams(max_chains=max_chains, hbm_budget=hbm_budget, nhit=nhit, device=device,
                              max_links=max_links)
        h = C.c_void_p()
        check(lib().dym_server_create(group._h, C.byref(p), C.byref(h)))
        self._h = h
        self.group = group

    def submit(self, rid: int, Nt: int, Nx: int, ewin: float, hw: float, a0: float, seed: int, start: str = "hot",
               axis: int = 1, bg: float = 0.0, K: int = 50, NRM: int = 20, drive_cap: int = 20000, D: int = 4):
        r = _lib.LlrRequest(id=rid, D=D, Nt=Nt, Nx=Nx, start=_lib.START[start], seed=seed, axis=axis, bg=bg,
                            ewin=ewin, hw=hw, a0=a0, K=K, NRM=NRM, drive_cap=drive_cap)
        check(lib().dym_server_submit(self._h, C.byref(r)))

    def cancel(self, rid: int) -> None:
        """Withdraw a queued or resident request; its "cancelled" response is
        returned by the next poll."""
        check(lib().dym_server_cancel(self._h, rid))

    def step(self, nsweeps: int = 1) -> None:
        check(lib().dym_server_step(self._h, nsweeps))

    def poll(self, max_n: int = 256) -> list[Response]:
        buf = (_lib.LlrResponse * max_n)()
        n = C.c_int32()
        check(lib().dym_server_poll(self._h, buf, max_n, C.byref(n)))
        out = []
        for r in buf[: n.value]:
            out.append(Response(r.id, r.a, r.S1, r.S2, _lib.LLR_STATUS.get(r.status, str(r.status)), r.sweeps,
                                r.drive_sweeps, r.hits, r.accepts, np.array(r.a_hist[: r.NRM])))
        return out

    def status(self):
        a, q, b, h = C.c_int32(), C.c_int32(), C.c_uint64(), C.c_uint64()
        check(lib().dym_server_status(self._h, C.byref(a), C.byref(q), C.byref(b), C.byref(h)))
        return dict(active=a.value, queued=q.value, hbm_used=b.value, link_hits=h.value)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().dym_server_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def serve_stream(srv: Server, requests, step_sweeps: int = 5, drive_cap: int = 2000):
    """Serve `requests` (workloads.LlrRequest, sorted by arrival) on `srv` as
    they arrive: a request is submitted once its arrival time (seconds after
    the call starts) has passed, the server steps while anything is resident
    or queued, and finished responses are collected.  Returns
    ({request id: [status, a, sweeps, latency in s]}, wall seconds)."""
    import time
    reqs = sorted(requests, key=lambda r: r.arrival)
    arrival = {r.rid: r.arrival for r in reqs}
    out = {}
    i = 0
    t0 = time.perf_counter()
    while len(out) < len(reqs):
        now = time.perf_counter() - t0
        while i < len(reqs) and reqs[i].arrival <= now:
            r = reqs[i]
            srv.submit(r.rid, r.Nt, r.Nx, r.ewin, r.hw, r.a0, r.seed, start=r.start, axis=1, bg=r.bg, K=r.K,
                       NRM=r.NRM, drive_cap=drive_cap)
            i += 1
        st = srv.status()
        if st["active"] or st["queued"]:
            srv.step(step_sweeps)
        elif i < len(reqs):
            time.sleep(max(0.0, reqs[i].arrival - (time.perf_counter() - t0)))
        for resp in srv.poll():
            out[resp.id] = [resp.status, float(resp.a), int(resp.sweeps),
                            time.perf_counter() - t0 - arrival[resp.id]]
    return out, time.perf_counter() - t0
