"""Build libdymgpu.so (CUDA, sm_103a) and the dym-mod-metro executable in-tree.

    python -m dym_symanzik_action_gb300.build

Translation units compile in parallel; outputs go to
dym_symanzik_action_gb300/lib/ and dym_symanzik_action_gb300/bin/ (git-ignored).
Host code is built with -ffp-contract=off so that FP64 arithmetic shared with
the device gives identical bits on x86-64 and aarch64.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(PKG, "lib")
BINDIR = os.path.join(PKG, "bin")
OBJDIR = os.path.join(PKG, "_build")
LIB = os.path.join(LIBDIR, "libdymgpu.so")
CLI = os.path.join(BINDIR, "dym-mod-metro")
LLR_CLI = os.path.join(BINDIR, "dym-llr")
LLR2D_CLI = os.path.join(BINDIR, "dym-llr2d")
SAVECFG_CLI = os.path.join(BINDIR, "dym-mod-metro-savecfg")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# DYM_BOUNDS_CHECK=1 builds the self-checking kernels (every index checked,
# first bad one reported by dym_sweep) into a separate object directory.
BOUNDS = os.environ.get("DYM_BOUNDS_CHECK") == "1"
if BOUNDS:
    OBJDIR = os.path.join(PKG, "_build_bounds")
CU_SOURCES = ["sweep.cu", "sweep_mixed.cu", "sweep_vt.cu", "measure.cu", "capi.cu", "probe.cu", "llr.cu", "batch.cu",
              "serve.cu", "noalloc.cu"]
CXX_SOURCES = ["group.cpp", "schedule.cpp", "checkpoint.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]


def build(verbose: bool = False) -> str:
    """Compile every translation unit that changed and link; return the .so path."""
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    inc = ["-I", CSRC, "-I", INCLUDE]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr", *inc,
                         *(["-DDYM_BOUNDS_CHECK"] if BOUNDS else []),
                         "-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", *inc,
                         "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        for cmd in jobs:
            if verbose:
                print(" ".join(cmd), flush=True)
        list(ex.map(_run, jobs))
    flavor_file = LIB + ".flavor"
    flavor = "bounds" if BOUNDS else "release"
    old_flavor = open(flavor_file).read() if os.path.exists(flavor_file) else ""
    if jobs or not os.path.exists(LIB) or old_flavor != flavor:
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs])
        with open(flavor_file, "w") as f:
            f.write(flavor)
    for name, exe in (("dym_mod_metro.cpp", CLI), ("dym_llr.cpp", LLR_CLI), ("dym_llr2d.cpp", LLR2D_CLI),
                      ("dym_mod_metro_savecfg.cpp", SAVECFG_CLI)):
        cli_src = os.path.join(CSRC, name)
        if os.path.exists(cli_src) and (_stale(exe, [cli_src, LIB] + hdrs)):
            _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-Wall", "-pthread", *inc, cli_src, "-o", exe,
                  "-L", LIBDIR, "-ldymgpu", "-Wl,-rpath,$ORIGIN/../lib"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
