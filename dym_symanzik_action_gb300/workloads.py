"""Synthetic workloads of the benchmark configurations (seeded, no datasets).

* ensemble(): the batched ensemble of 256 independent chains -- Nx uniform in
  {8, 12, 16, 20, 24}, Nt uniform in {2, 4, 6, 8} (Philox-drawn from the chain
  index), 200 chains on S(1080) and 56 on the binary icosahedral group,
  (beta1, beta2) on a 16x16 grid over [0.5, 4.0] x [-0.3, 0.3], hot starts.
* llr_requests(): the served LLR stream -- Poisson arrivals at a mean rate,
  each request one energy window of width 0.5% of the plaquette-energy range
  on an S(1080) lattice with Nx in {6, 8, 12, 16}, Nt in {2, 4}, beta2 in
  {0, -0.1}; 20 Robbins-Monro iterations of 50 sweeps.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

BASE_SEED = 20261203


def _philox_uniforms(key: int, n: int, stream: int) -> np.ndarray:
    """n uniforms in [0,1) from Philox4x32-10 (counter (i, stream, 0, 0))."""
    M0, M1, W0, W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85
    out = np.empty(n)
    for i in range(n):
        c = [i & 0xFFFFFFFF, stream & 0xFFFFFFFF, 0, 0]
        k0, k1 = key & 0xFFFFFFFF, (key >> 32) & 0xFFFFFFFF
        for _ in range(10):
            p0 = M0 * c[0]
            p1 = M1 * c[2]
            c = [((p1 >> 32) ^ c[1] ^ k0) & 0xFFFFFFFF, p1 & 0xFFFFFFFF, ((p0 >> 32) ^ c[3] ^ k1) & 0xFFFFFFFF,
                 p0 & 0xFFFFFFFF]
            k0 = (k0 + W0) & 0xFFFFFFFF
            k1 = (k1 + W1) & 0xFFFFFFFF
        out[i] = c[0] * 2.0 ** -32
    return out


@dataclass
class ChainSpec:
    group: str
    Nt: int
    Nx: int
    beta: tuple
    seed: int
    start: str = "hot"

    @property
    def links(self) -> int:
        return 4 * self.Nt * self.Nx ** 3


def ensemble(n: int = 256, n_s1080: int = 200, seed: int = BASE_SEED) -> list[ChainSpec]:
    u = _philox_uniforms(seed, 2 * n, stream=3)
    nxs, nts = (8, 12, 16, 20, 24), (2, 4, 6, 8)
    out = []
    for c in range(n):
        i, j = divmod(c, 16)
        b1 = 0.5 + 3.5 * (i % 16) / 15.0
        b2 = -0.3 + 0.6 * j / 15.0
        out.append(ChainSpec("S1080" if c < n_s1080 else "BI", nts[int(u[2 * c + 1] * 4)], nxs[int(u[2 * c] * 5)],
                             (0.0, b1, b2), seed + c))
    return out


@dataclass
class LlrRequest:
    rid: int
    arrival: float      # seconds after the stream starts
    Nt: int
    Nx: int
    bg: float           # beta2 background (window on the plaquette action S1)
    ewin: float         # window centre
    hw: float           # half-width (window = 0.5% of the plaquette-energy range)
    a0: float
    start: str
    seed: int
    K: int = 50
    NRM: int = 20

    @property
    def nplaq(self) -> int:
        return 6 * self.Nt * self.Nx ** 3


def llr_requests(n: int = 2000, rate: float = 200.0, seed: int = BASE_SEED, retr_range=(-3.0, 1.5)) -> list:
    """Poisson stream; window centres drawn in [-2.6, -0.4] x NPLAQ (reachable
    from a hot or a cold start), cold starts below -1.5 x NPLAQ."""
    u = _philox_uniforms(seed, 6 * n, stream=5)
    t = 0.0
    out = []
    width = 0.005 * (retr_range[1] - retr_range[0])  # per plaquette
    for r in range(n):
        t += -math.log(max(1.0 - u[6 * r], 1e-300)) / rate
        Nx = (6, 8, 12, 16)[int(u[6 * r + 1] * 4)]
        Nt = (2, 4)[int(u[6 * r + 2] * 2)]
        bg = (0.0, -0.1)[int(u[6 * r + 3] * 2)]
        cen = -2.6 + 2.2 * u[6 * r + 4]
        npl = 6 * Nt * Nx ** 3
        out.append(LlrRequest(r, t, Nt, Nx, bg, cen * npl, 0.5 * width * npl, a0=2.0,
                              start="cold" if cen < -1.5 else "hot", seed=seed + 7919 * r))
    return out
