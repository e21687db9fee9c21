"""The neighbour offsets of the mixed-precision sweep kernels (staples.cuh
site_geo_fast, one compare and select per offset) equal the periodic wrap of
the reference's getidx/getpos (lattice.c:119-132) as staples.cuh site_geo_xyz
restates it, for every coordinate and extent checked by
tests/site_geometry_check.cpp (compiled for the host with g++)."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "dym_symanzik_action_gb300", "csrc")


def test_site_geo_fast_equals_wrap():
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "check")
        subprocess.run(["g++", "-std=c++17", "-O1", "-I", CSRC, os.path.join(HERE, "site_geometry_check.cpp"), "-o",
                        exe], check=True)
        r = subprocess.run([exe], stdout=subprocess.PIPE, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    assert " 0 differ" in r.stdout
