"""Chain checkpoint files on the host: the C ABI reads a file written here
from the documented layout (an independent writer), records the group by the
FNV-1a 64 hash of its Cayley table, and refuses malformed files by code
(DYM_EFORMAT, DYM_EIO) without a device.  The resume itself (a loaded chain
continues bit for bit) is tested on the GPU in test_gpu_1_parity.py."""
import struct

import numpy as np
import pytest

from dym_symanzik_action_gb300 import tables

FNV_OFFSET, FNV_PRIME = 0xCBF29CE484222325, 0x100000001B3


def fnv1a64(data: bytes) -> int:
    h = FNV_OFFSET
    for b in data:
        h = ((h ^ b) * FNV_PRIME) & 0xFFFFFFFFFFFFFFFF
    return h


def write_checkpoint(path, D, Nt, Nx, P, pool, table_hash, seed, sweep, betas, links, version=1,
                     magic=b"DYMCKPT1"):
    body = np.asarray(links, dtype="<u2").tobytes()
    head = magic + struct.pack("<I3iIiQQII3d", version, D, Nt, Nx, P, pool, table_hash, seed, sweep, 0, *betas)
    assert len(head) == 80
    with open(path, "wb") as f:
        f.write(head + body + struct.pack("<Q", fnv1a64(body)))


@pytest.fixture(scope="module")
def bt(engine):
    return engine.load_group(tables.ensure_table("BT"))


def test_table_hash_is_fnv1a_of_the_cayley_table(bt):
    assert bt.table_hash == fnv1a64(bt.mult.astype("<u2").tobytes())


def test_read_info_of_an_independently_written_file(engine, bt, tmp_path):
    D, Nt, Nx = 4, 2, 3
    n = D * Nt * Nx ** (D - 1)
    links = np.random.default_rng(5).integers(0, bt.P, n)
    p = tmp_path / "c.ckpt"
    write_checkpoint(p, D, Nt, Nx, bt.P, 0, bt.table_hash, 2**63 + 7, 4242, (0.25, 2.5, -0.125), links)
    info = engine.checkpoint_info(p)
    assert (info["D"], info["Nt"], info["Nx"], info["order"], info["pool"]) == (D, Nt, Nx, bt.P, 0)
    assert info["table_hash"] == bt.table_hash
    assert info["seed"] == 2**63 + 7 and info["sweep"] == 4242
    assert (info["beta0"], info["beta1"], info["beta2"]) == (0.25, 2.5, -0.125)


@pytest.mark.parametrize("case", ["missing", "magic", "version", "short", "long", "checksum", "shape", "order"])
def test_malformed_checkpoints_are_refused(engine, bt, tmp_path, case):
    from dym_symanzik_action_gb300._lib import DymError
    D, Nt, Nx = 3, 2, 4
    n = D * Nt * Nx ** (D - 1)
    links = np.arange(n) % bt.P
    p = tmp_path / case
    args = dict(D=D, Nt=Nt, Nx=Nx, P=bt.P, pool=0, table_hash=bt.table_hash, seed=1, sweep=3,
                betas=(0.0, 1.0, 0.0), links=links)
    if case == "magic":
        args["magic"] = b"DYMCKPT0"
    elif case == "version":
        args["version"] = 2
    elif case == "shape":
        args["D"] = 1
    elif case == "order":
        args["P"] = 5041
    if case != "missing":
        write_checkpoint(p, **args)
    raw = p.read_bytes() if case != "missing" else b""
    if case == "short":
        p.write_bytes(raw[:-3])
    elif case == "long":
        p.write_bytes(raw + b"\0\0")
    elif case == "checksum":
        b = bytearray(raw)
        b[80] ^= 1  # first link byte
        p.write_bytes(bytes(b))
    with pytest.raises(DymError) as e:
        engine.checkpoint_info(p)
    assert e.value.code == (-2 if case == "missing" else -3), str(e.value)


def test_mutated_checkpoints_never_crash_the_reader(engine, bt, tmp_path):
    """Random truncations and byte flips of a valid file either still parse
    (a flip in the seed, couplings or sweep count changes only those fields)
    or are refused with DYM_EFORMAT; the reader never crashes or reads past
    the file."""
    from dym_symanzik_action_gb300._lib import DymError
    D, Nt, Nx = 4, 2, 2
    n = D * Nt * Nx ** (D - 1)
    good = tmp_path / "good"
    write_checkpoint(good, D, Nt, Nx, bt.P, 0, bt.table_hash, 9, 1, (0.0, 1.0, 0.0), np.arange(n) % bt.P)
    raw = good.read_bytes()
    rng = np.random.default_rng(17)
    p = tmp_path / "m"
    refused = 0
    for k in range(300):
        b = bytearray(raw)
        if k % 3 == 0:
            b = b[: int(rng.integers(0, len(raw)))]
        else:
            for _ in range(int(rng.integers(1, 4))):
                b[int(rng.integers(0, len(b)))] ^= int(rng.integers(1, 256))
        p.write_bytes(bytes(b))
        try:
            engine.checkpoint_info(p)
        except DymError as e:
            assert e.code == -3, str(e)
            refused += 1
    assert refused >= 100
