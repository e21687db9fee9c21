"""dym-mod-metro-savecfg (drop-in for the reference's configuration writer):
the files hold, in the reference's big-endian Kentucky/NERSC layout, the SU(3)
matrices of exactly the configuration the Python API reaches with the same
arguments, and their plaquette is the GMES line's."""
import subprocess

import numpy as np
import pytest

from dym_symanzik_action_gb300 import build, tables

pytestmark = pytest.mark.gpu

Nt, Nx, SEED, BETA = 4, 4, 5, (0.0, 2.0, -0.1)
K, N, NTHERM = 2, 2, 1


def group_matrices(path, P):
    toks = open(path).read().split()
    m = np.array(toks[1 + 2 * P + P * P:], dtype=np.float64).reshape(P, 3, 3, 2)
    return m[..., 0] + 1j * m[..., 1]


def test_savecfg_files_hold_the_configuration(engine, tmp_path):
    path = tables.ensure_table("S1080")
    out = subprocess.run([build.SAVECFG_CLI, path, "4", str(Nt), str(Nx), *map(str, BETA), str(SEED),
                          str(tmp_path) + "/", str(K), str(N), str(NTHERM)], capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr
    gmes = [l.split() for l in out.stdout.splitlines() if l.startswith("GMES:")]
    assert len(gmes) == N and all(len(f) == 5 for f in gmes)
    g = engine.load_group(path)
    mats = group_matrices(path, g.P)
    lat = engine.Lattice(g, 4, Nt, Nx, *BETA, SEED, start="hot")
    lat.update(NTHERM, 20)
    V = lat.V
    for n in range(N):
        lat.update(K, 20)
        name = tmp_path / ("lat-beta1%.3f-beta2%.3f-nt%02d-nx%02d-num%04d" % (BETA[1], BETA[2], Nt, Nx, n))
        raw = np.fromfile(name, ">f8")
        assert raw.size == V * 4 * 18
        # index x + Nx(y + Nx(z + Nx(t + Nt(part + 2(row + 3(col + 3 dir)))))), dir = (d + 3) mod 4
        arr = raw.reshape(4, 3, 3, 2, Nt, Nx, Nx, Nx)  # [dir][col][row][part][t][z][y][x]
        U = (arr[:, :, :, 0] + 1j * arr[:, :, :, 1]).transpose(0, 3, 4, 5, 6, 2, 1)  # [dir][t][z][y][x][row][col]
        links = lat.links  # [d][site], site = t + Nt(x + Nx(y + Nx z))
        want = mats[links].reshape(4, Nx, Nx, Nx, Nt, 3, 3).transpose(0, 4, 1, 2, 3, 5, 6)  # [d][t][z][y][x]
        for d in range(4):
            assert np.array_equal(U[(d + 3) % 4], want[d]), (n, d)
        # plaquette of the file's matrices = the GMES line's (printed %e)
        Ud = [U[(d + 3) % 4] for d in range(4)]  # engine directions: 0 = t, 1 = x, 2 = y, 3 = z
        axis = {0: 0, 1: 3, 2: 2, 3: 1}  # array axis of direction d in [t][z][y][x]
        tot = 0.0
        for mu in range(4):
            for nu in range(mu + 1, 4):
                a = Ud[mu]
                b = np.roll(Ud[nu], -1, axis=axis[mu])
                c = np.roll(Ud[mu], -1, axis=axis[nu])
                p = a @ b @ np.conj(np.swapaxes(c, -1, -2)) @ np.conj(np.swapaxes(Ud[nu], -1, -2))
                tot += -np.trace(p, axis1=-2, axis2=-1).real.sum()
        assert abs(tot / (V * 6) - float(gmes[n][4])) < 1e-5 * max(1.0, abs(float(gmes[n][4])))
