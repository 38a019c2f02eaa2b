"""The C++ host API (include/goofit_gb300.hpp): it compiles against libgfengine.so here (no GPU), and on a GPU
its fits agree with the Python layer's on the same data."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import goofit_gb300 as gf
from goofit_gb300 import _abi as A
from goofit_gb300 import workloads as W

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "fit_examples.cpp"


def build_example(tmp_path: Path) -> Path:
    lib = A.LIB_PATH
    exe = tmp_path / "fit_examples"
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", f"-I{ROOT / 'include'}", str(SRC), "-o", str(exe), f"-L{lib.parent}",
           "-lgfengine", f"-Wl,-rpath,{lib.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_api_compiles_and_links(tmp_path):
    assert build_example(tmp_path).exists()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_cpp_fits_match_python_fits(tmp_path, prec):
    exe = build_example(tmp_path)
    wl = W.make_c2(50_000, seed=21)
    xs = wl.data.to_numpy()[0]
    np.savetxt(tmp_path / "x.txt", xs, fmt="%.17g")
    r = subprocess.run([str(exe), prec, str(tmp_path / "x.txt")], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = {ln.split()[0]: [float(v) for v in ln.split()[1:]] for ln in r.stdout.splitlines()}
    # the exponential scenario of tests/simple/BinningTest.cpp: alpha within 3/sqrt(N) of -1.5
    valid, a, ea = lines["exp"]
    assert valid == 1 and a == pytest.approx(-1.5, rel=3 / np.sqrt(100_000))
    # the composite fit equals the Python FitManager's on the same events
    wl.reset()
    fm = gf.FitManager(wl.pdf, precision=prec, tolerance=0.01)
    fm.verbosity = 0
    assert fm.fit().valid
    valid, *vals = lines["composite"]
    assert valid == 1
    for k, name in enumerate(("fsig", "alpha", "mu", "sigma")):
        v = wl.variables[name]
        assert vals[2 * k] == pytest.approx(v.value, abs=0.01 * v.error), name
        assert vals[2 * k + 1] == pytest.approx(v.error, rel=0.01), name
