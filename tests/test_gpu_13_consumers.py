"""The reference's own log consumers read the engine's logs unchanged.

scripts/getavgsimpplaq.py (GMES field 4, the plaquette, as <P>/3 + 1 against
3 x the beta in the file name), scripts/pltabsvalpolyakov.py (GMES field 2,
Re of the Polyakov loop, against beta' from the b1/b2 file name) and
scripts/llr_reconstruct.py (its parse() of the ANE:/NPLAQ:/AXIS: lines) are
taken from the staged reference (baseline/_ref, or $REF_DIR) and run as they
are on logs of the engine's dym-mod-metro and dym-llr, and on a log of the
unmodified reference dym-mod-metro with the same arguments: each script must
read from every log the same fields a direct parse of its lines gives.  The
two plotting scripts are top-level code with hard-coded input directories:
they run with those directories mapped to scratch directories and
matplotlib absorbed by a recorder of their plot calls (no display, no
files).  Skipped where the reference is not staged."""
import builtins
import importlib.util
import os
import subprocess

import numpy as np
import pytest

from conftest import staged_reference
from dym_symanzik_action_gb300 import build, tables
from oracle.oracle import REF_BIN

pytestmark = pytest.mark.gpu


class PlotRecorder:
    """Stands in for matplotlib and its submodules: any attribute is another
    stand-in, and every call is recorded as (attribute name, args, kwargs)."""

    def __init__(self, calls=None, name="matplotlib"):
        self.calls = [] if calls is None else calls
        self.name = name

    def __getattr__(self, name):
        return PlotRecorder(self.calls, name)

    def __call__(self, *a, **k):
        self.calls.append((self.name, a, k))
        return PlotRecorder(self.calls, self.name)


def run_consumer_script(path, dirs):
    """Execute the script at `path` unchanged; a directory it names is read
    from dirs[basename of that directory].  Returns the plot recorder."""
    rec = PlotRecorder()
    real_os = os

    def remap(p):
        d, f = real_os.path.split(str(p))
        if real_os.path.basename(d) in dirs:
            return real_os.path.join(dirs[real_os.path.basename(d)], f)
        if real_os.path.basename(str(p).rstrip("/")) in dirs:
            return dirs[real_os.path.basename(str(p).rstrip("/"))]
        return p

    class FakeOs:
        path = real_os.path

        @staticmethod
        def listdir(p):
            return sorted(real_os.listdir(remap(p)))

    real_import = builtins.__import__

    def fake_import(name, *a, **k):
        if name == "os":
            return FakeOs
        if name.startswith("matplotlib"):
            return rec
        return real_import(name, *a, **k)

    bi = dict(vars(builtins), __import__=fake_import, open=lambda p, *a, **k: builtins.open(remap(p), *a, **k),
              print=lambda *a, **k: None)
    code = compile(open(path).read(), path, "exec")
    exec(code, {"__builtins__": bi, "__name__": "__consumer__"})
    return rec


def gmes_rows(log):
    return [l.split(" ") for l in open(log) if "GMES: " in l]


def run_metro(exe, table, beta, seed, out, D=4, Nt=4, Nx=4, K=2, N=3, Ntherm=2):
    import tempfile
    with tempfile.TemporaryDirectory() as td:  # the reference's -pg build writes gmon.out into its cwd
        r = subprocess.run([exe, table, str(D), str(Nt), str(Nx), *(repr(float(b)) for b in beta), str(seed),
                            str(K), str(N), str(Ntherm)], capture_output=True, text=True, timeout=600, cwd=td)
    assert r.returncode == 0, r.stderr
    with open(out, "w") as f:
        f.write(r.stdout)


@pytest.fixture(scope="module")
def ref():
    r = staged_reference()
    if r is None or not os.path.exists(os.path.join(r, "scripts", "getavgsimpplaq.py")):
        pytest.skip("reference not staged (oracle/stage_ref.sh)")
    return r


def test_getavgsimpplaq_reads_engine_and_reference_logs(engine, ref, tmp_path):
    table = os.path.join(ref, "groups", "mys1080-v4")
    ref_exe = os.path.join(REF_BIN, "dym-mod-metro")
    dirs = {}
    expect = {}
    for b2 in ("-0.1", "0.1", "0", "-0.2", "0.2"):
        d = tmp_path / f"beta2is{b2}"
        d.mkdir()
        dirs[d.name] = str(d)
        for k, b1n in enumerate(("0.5", "0.8")):  # beta1 / 3 as in the reference's file names
            beta = (0.0, 3 * float(b1n), 3 * float(b2))
            name = f"out_b{b1n}_run.txt"
            if k == 1 and b2 == "0" and os.path.exists(ref_exe):
                run_metro(ref_exe, table, beta, 31, str(d / name))  # the unmodified reference's log
            else:
                run_metro(build.CLI, table, beta, 30 + k, str(d / name))
            p = [float(r[4]) / 3 + 1 for r in gmes_rows(d / name)]
            expect.setdefault(d.name, []).append((3 * float(b1n), sum(p) / len(p), float(np.std(p))))
    rec = run_consumer_script(os.path.join(ref, "scripts", "getavgsimpplaq.py"), dirs)
    bars = [c for c in rec.calls if c[0] == "errorbar"]
    assert len(bars) == 5
    order = ["beta2is-0.1", "beta2is0.1", "beta2is0", "beta2is-0.2", "beta2is0.2"]  # the script's block order
    for (_, (betas, means, sds), _), dname in zip(bars, order):
        got = sorted(zip(betas, means, sds))
        assert got == sorted(expect[dname]), dname


def test_pltabsvalpolyakov_reads_engine_log(engine, ref, tmp_path):
    table = os.path.join(ref, "groups", "mys1080-v4")
    d = tmp_path / "Nt4Ns12datathird"
    d.mkdir()
    expect = []
    for b1n, b2n in (("0.5", "0.0"), ("0.6", "-0.05")):
        name = f"outb1{b1n}_b2{b2n}_x.txt"
        run_metro(build.CLI, table, (0.0, 3 * float(b1n), 3 * float(b2n)), 41, str(d / name), Nt=4, Nx=4)
        re_ = [float(r[2]) for r in gmes_rows(d / name)]
        expect.append((((3 * float(b1n)) ** 2 + (3 * float(b2n)) ** 2) ** 0.5, abs(sum(re_) / len(re_)),
                       float(np.std(re_))))
    rec = run_consumer_script(os.path.join(ref, "scripts", "pltabsvalpolyakov.py"), {d.name: str(d)})
    bars = [c for c in rec.calls if c[0] == "errorbar"]
    assert len(bars) == 1
    betap, means, sds = bars[0][1]
    assert sorted(zip(betap, means, sds)) == sorted(expect)


def test_llr_reconstruct_parses_dym_llr_log(engine, ref, tmp_path):
    spec = importlib.util.spec_from_file_location("llr_reconstruct", os.path.join(ref, "scripts",
                                                                                   "llr_reconstruct.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    D, Nt, Nx = 4, 4, 4
    nplaq = Nt * Nx ** 3 * 6
    args = [tables.ensure_table("S1080"), D, Nt, Nx, 1, 0.0, -0.6 * nplaq, -1.2 * nplaq, 0.2 * nplaq,
            0.0225 * nplaq / 2, 1.5, 7, 5, 4, 1]
    out = subprocess.run([build.LLR_CLI, *map(str, args)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    log = tmp_path / "ladder.out"
    log.write_text(out.stdout)
    E, a, norm, axis = mod.parse(str(log))
    rows = [l.split() for l in out.stdout.splitlines() if l.startswith("ANE:") and "unreached" not in l]
    want = sorted((float(r[1]), float(r[2])) for r in rows)
    assert list(zip(E.tolist(), a.tolist())) == want
    assert norm == nplaq and axis == 1
