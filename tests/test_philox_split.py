"""The sweep kernels' Metropolis draws with the per-link part of the first
two Philox4x32-10 rounds computed once per link and the round keys passed in
(dym_core.h dym_metro_link_init / dym_metro_hit) are the bits of the plain
counter-based draw dym_hit_random (tests/philox_split_check.c, compiled for
the host with gcc)."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "dym_symanzik_action_gb300", "csrc")


def test_metro_hit_equals_hit_random():
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "check")
        subprocess.run(["gcc", "-std=gnu99", "-O2", "-I", CSRC, os.path.join(HERE, "philox_split_check.c"), "-o", exe,
                        "-lm"], check=True)
        r = subprocess.run([exe], stdout=subprocess.PIPE, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    assert " 0 differ" in r.stdout
