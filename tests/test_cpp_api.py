"""The C++ host API (include/goofit_gb300.hpp).

On the CPU:
* Both example programs compile and link against libgfengine.so.
* The 4-body classes (Amp4Body, DecayInfo4, Amplitude, SpinFactor, Lineshapes::RBW/SBW) flatten the D0 -> K3pi
  model into the same gf_node tree as the Python layer: ops, flags, parameter slots, constants, observables,
  children and parameter order.
* The header's Dim5 equals the Python restatement at 1e-12 on the same 4-vectors.
* Its phase-space generator is flat: every variable's histogram agrees with the Python generator's
  (chi2 / ndf < 1.6 over 40 bins of 4e5 events each).

On a GPU, its fits agree with the Python layer's on the same data:
* The unbinned exponential, with MINOS errors.
* The binned Poisson likelihood and the chi-square.
* The composite model.
* A C5 Amp4Body fit, given the same normalisation events.
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import goofit_gb300 as gf
from goofit_gb300 import _abi as A
from goofit_gb300 import phasespace as PS
from goofit_gb300 import workloads as W
from oracle import oracle as O

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "fit_examples.cpp"
SRC4 = ROOT / "tests" / "cpp" / "amp4_examples.cpp"
C5_CHAINS = ["K*rho_S", "K*rho_P", "K*rho_D", "K1rho", "a1rho", "K*f0"]


def build_example(tmp_path: Path, src: Path = SRC) -> Path:
    lib = A.LIB_PATH
    exe = tmp_path / src.stem
    # no FMA contraction, so that Dim5 rounds as the numpy restatement does
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-ffp-contract=off", f"-I{ROOT / 'include'}", str(src), "-o",
           str(exe), f"-L{lib.parent}", "-lgfengine", f"-Wl,-rpath,{lib.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_api_compiles_and_links(tmp_path):
    assert build_example(tmp_path).exists()
    assert build_example(tmp_path, SRC4).exists()


def c5_coefs(pdf, path: Path) -> None:
    params = pdf._flatten()[1]
    names = [v.name for v in params]
    vals = [params[names.index(f"{c}_{s}")].value for c in C5_CHAINS for s in ("re", "im")]
    path.write_text("\n".join(f"{v:.17g}" for v in vals))


def test_cpp_amp4body_tree_matches_python(tmp_path):
    exe = build_example(tmp_path, SRC4)
    pdf = W.c5_model(1000, norm_seed=55)[0]
    nodes, params, obs = pdf._flatten()
    c5_coefs(pdf, tmp_path / "coefs.txt")
    out = subprocess.run([str(exe), "tree", str(tmp_path / "coefs.txt")], capture_output=True, text=True,
                         check=True).stdout.splitlines()
    cp = [ln.split() for ln in out if ln.startswith("param ")]
    co = [ln.split() for ln in out if ln.startswith("obs ")]
    cn = [ln[5:].split("|") for ln in out if ln.startswith("node ")]
    assert [(t[1], float(t[2]), int(t[3])) for t in cp] == [(v.name, v.value, int(v.fixed)) for v in params]
    assert [(t[1], float(t[2]), float(t[3]), int(t[4])) for t in co] == \
        [(o.name, o.lowerlimit, o.upperlimit, int(o.is_event_number)) for o in obs]
    assert len(cn) == len(nodes) == 44
    for parts, n in zip(cn, nodes):
        op, flags = map(int, parts[0].split())
        got = (op, flags, [int(x) for x in parts[1].split()], [float(x) for x in parts[2].split()],
               [int(x) for x in parts[3].split()], [int(x) for x in parts[4].split()])
        # the cache index constant of the Amp4Body node counts the objects made in each process
        want = (n["op"], n["flags"], n["params"], [float(c) for c in n["consts"]], n["obs"], n["children"])
        if op == A.GF_OP_AMP4BODY:
            got[3].pop(5), want[3].pop(5)
        assert got == want


def test_cpp_dim5_matches_python(tmp_path):
    exe = build_example(tmp_path, SRC4)
    p4 = PS.generate(W.C5_M, W.C5_MASSES, 5000, np.random.Generator(np.random.PCG64(3)))
    p4.astype(np.float64).tofile(tmp_path / "p4.bin")
    subprocess.run([str(exe), "dim5", "5000", str(tmp_path / "p4.bin"), str(tmp_path / "d5.bin")], check=True)
    got = np.fromfile(tmp_path / "d5.bin").reshape(5, -1)
    np.testing.assert_allclose(got, PS.dim5(p4), rtol=0, atol=1e-12)


def test_cpp_phase_space_is_flat(tmp_path):
    exe = build_example(tmp_path, SRC4)
    n = 400_000
    subprocess.run([str(exe), "gen", str(n), "11", str(tmp_path / "g.bin")], check=True)
    got = np.fromfile(tmp_path / "g.bin").reshape(5, -1)
    ref = PS.norm_events(W.C5_M, W.C5_MASSES, n, 12)
    assert np.all(np.isfinite(got))
    assert got[0].min() >= 2 * 0.13957 and got[1].min() >= 0.13957 + 0.4937
    assert np.abs(got[2:4]).max() <= 1 and np.abs(got[4]).max() <= np.pi
    for k in range(5):
        h1, edges = np.histogram(got[k], bins=40)
        h2, _ = np.histogram(ref[k], bins=edges)
        ok = (h1 + h2) > 0
        assert ((h1 - h2)[ok] ** 2 / (h1 + h2)[ok]).sum() / ok.sum() < 1.6, k


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
    # MINOS on the same fit, against the Python FitManager's on the same draws
    draws = O.mt19937_exponential(137, 1.5, 100_000)
    x = gf.Observable("xvar", 0, 10)
    ds = gf.UnbinnedDataSet(x)
    ds.from_numpy(draws[draws < 10].reshape(1, -1))
    alpha = gf.Variable("alpha", -2, 0.1, -10, 10)
    pdf = gf.ExpPdf("exppdf", x, alpha)
    pdf.setData(ds)
    fm = gf.FitManager(pdf, precision=prec, tolerance=0.01)
    fm.verbosity = 0
    fm.setMinos()
    assert fm.fit().valid
    valid, a, ea, mlo, mhi = lines["minos"]
    assert valid == 1 and a == pytest.approx(alpha.value, abs=0.01 * alpha.error)
    assert mlo < 0 < mhi
    assert (mlo, mhi) == pytest.approx(alpha.minos_error, rel=0.01)
    # the binned fits, against the Python layer's on the same bins
    for key, fc in (("binned_nll", gf.BinnedNllFit), ("binned_chisq", gf.BinnedChisqFit)):
        xb = gf.Observable("xvar", 0, 10)
        bd = gf.BinnedDataSet(xb)
        bd.fill(draws[draws < 10].reshape(1, -1))
        ab = gf.Variable("alpha", -1.4, 0.1, -10, 10)
        bp = gf.ExpPdf("exppdf", xb, ab)
        bp.setData(bd)
        bp.setFitControl(fc())
        fb = gf.FitManager(bp, precision=prec, tolerance=0.01)
        fb.verbosity = 0
        assert fb.fit().valid
        valid, a, ea = lines[key]
        assert valid == 1 and a == pytest.approx(ab.value, abs=0.01 * ab.error), key
        assert ea == pytest.approx(ab.error, rel=0.01), key
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


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_cpp_amp4body_fit_matches_python(tmp_path, prec):
    """A C5 Amp4Body fit (20,000 events, 100,000 normalisation events) through the C++ API equals the Python
    FitManager's on the same events: values within 0.01 sigma, errors within 1%."""
    exe = build_example(tmp_path, SRC4)
    wl = W.make_c5(20_000, n_norm=100_000, seed=7)
    c5_coefs(wl.pdf, tmp_path / "coefs.txt")   # the truth (the C++ program starts at 1.05 times it)
    cols = wl.data.to_numpy()
    np.ascontiguousarray(cols, dtype=np.float64).tofile(tmp_path / "data.bin")
    np.ascontiguousarray(wl.pdf.norm_events, dtype=np.float64).tofile(tmp_path / "norm.bin")
    r = subprocess.run([str(exe), "fit", prec, str(tmp_path / "coefs.txt"), str(cols.shape[1]),
                        str(tmp_path / "data.bin"), str(wl.pdf.norm_events.shape[1]), str(tmp_path / "norm.bin")],
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr
    lines = {ln.split()[0]: [float(v) for v in ln.split()[1:]] for ln in r.stdout.splitlines()}
    wl.reset()
    fm = gf.FitManager(wl.pdf, precision=prec, tolerance=0.01)
    fm.verbosity = 0
    res = fm.fit()
    assert res.valid and lines["valid"][0] == 1
    assert lines["valid"][1] == pytest.approx(res.fmin, rel=1e-9)
    for name, v in wl.variables.items():
        val, err = lines[name]
        assert val == pytest.approx(v.value, abs=0.01 * v.error), name
        assert err == pytest.approx(v.error, rel=0.01), name
