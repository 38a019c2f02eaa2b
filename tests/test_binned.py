"""Binned fits: BinnedDataSet's bin numbering (src/goofit/BinnedDataSet.cpp) on the CPU; on a GPU the three
binned metrics against the FP64 oracle and the reference's binned fit scenarios (tests/simple/BinningTest.cpp).

Tolerances: objective 1e-10 relative (FP64) / 1e-6 (mixed); fitted values as the reference test checks them
(Approx(...).epsilon(3 / sqrt(N))) and within 0.01 sigma of the FP64 fit for the mixed path."""
import math

import numpy as np
import pytest

import goofit_gb300 as gf
from goofit_gb300 import _abi as A
from oracle import oracle as O


def test_bin_numbering_and_centres():
    x = gf.Observable("x", 0, 10)
    y = gf.Observable("y", -1, 1)
    x.setNumBins(5)
    y.setNumBins(4)
    b = gf.BinnedDataSet([x, y])
    assert b.getNumBins() == 20
    x.value, y.value = 4.5, 0.1      # local (2, 2) -> 2 + 2 * 5
    b.addEvent()
    assert b.getBinContent(12) == 1
    assert b.getBinCenter(x, 12) == pytest.approx(5.0) and b.getBinCenter(y, 12) == pytest.approx(0.25)
    assert b.getBinVolume(0) == pytest.approx(2.0 * 0.5)
    assert b.getBinError(12) == 1.0
    b.setBinError(3, 0.5)             # explicit errors: zero where unset
    assert b.getBinError(12) == 0.0 and b.getBinError(3) == 0.5
    cols = b.engine_columns([x, y], False)
    assert cols.shape == (4, 20) and cols[0, 12] == b.getBinCenter(x, 12) and cols[2, 12] == 1


def exp_binned(N, lam=1.5):
    d = O.mt19937_exponential(137, lam, N)
    return d[d < 10]


def tree(pdf):
    nodes, params, obs = pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    return nodes, olist, params


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["mixed", "fp64"])
@pytest.mark.parametrize("fc", [gf.BinnedNllFit, gf.BinnedChisqFit, gf.BinnedErrorFit])
def test_binned_metrics_match_oracle(prec, fc):
    x = gf.Observable("xvar", 0, 10)
    data = gf.BinnedDataSet(x)
    data.fill(exp_binned(100_000).reshape(1, -1))
    for b in range(0, 100, 7):
        if fc is gf.BinnedErrorFit:
            data.setBinError(b, 1.0 + b)
    alpha = gf.Variable("alpha", -1.4, 0.1, -10, 10)
    pdf = gf.ExpPdf("exppdf", x, alpha)
    pdf.setData(data)
    pdf.setFitControl(fc())
    eng, params = pdf._engine_for(data, prec)
    nodes, olist, _ = tree(pdf)
    cols = data.engine_columns([x], fc is gf.BinnedErrorFit)
    if fc is gf.BinnedErrorFit:
        cols = cols[:, np.nonzero(cols[2])[0]]  # bins with an error
        eng.upload(cols)
    tol = 1e-10 if prec == "fp64" else 1e-6
    for a in (-1.4, -1.5, -1.6):
        ref = O.binned(nodes, olist, np.array([a]), cols, fc.metric)
        got, g = eng.nll_grad(np.array([a]))
        assert got == pytest.approx(ref, rel=tol), (a, got, ref)
        step = 1e-6
        fd = (O.binned(nodes, olist, np.array([a + step]), cols, fc.metric) -
              O.binned(nodes, olist, np.array([a - step]), cols, fc.metric)) / (2 * step)
        assert g[0] == pytest.approx(fd, rel=1e-4, abs=1e-3 * math.sqrt(abs(ref) + 1))


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_reference_binned_exp_fit(prec):
    # tests/simple/BinningTest.cpp "Variations on a exp fit", Binned section: N = 100000
    N = 100_000
    x = gf.Observable("xvar", 0, 10)
    data = gf.BinnedDataSet(x)
    data.fill(exp_binned(N).reshape(1, -1))
    alpha = gf.Variable("alpha", -2, 0.1, -10, 10)
    pdf = gf.ExpPdf("exppdf", x, alpha)
    pdf.setData(data)
    fm = gf.FitManager(pdf, precision=prec)
    fm.verbosity = 0
    assert fm.fit().valid
    err = 1 / math.sqrt(N) * abs(alpha.value)
    assert alpha.error < 3 * err
    assert abs(alpha.value + 1.5) <= 3 / math.sqrt(N) * 1.5


@pytest.mark.gpu
def test_reference_binned_dual_exp_fit_and_precision_parity():
    # tests/simple/BinningTest.cpp "Variations on a dual fit", Binned section: N = 200000; x ~ exp(1.5),
    # y ~ exp(0.75) drawn alternately from one mt19937(137)
    N = 200_000
    e = O.mt19937_exponential(137, 1.0, 2 * N)
    xs, ys = e[0::2] / 1.5, e[1::2] / 0.75
    keep = (xs < 10) & (ys < 10)
    out = {}
    for prec in ("fp64", "mixed"):
        x = gf.Observable("xvar", 0, 10)
        y = gf.Observable("yvar", 0, 10)
        data = gf.BinnedDataSet([x, y])
        data.fill(np.vstack([xs[keep], ys[keep]]))
        xa = gf.Variable("xalpha", -2, 0.1, -10, 10)
        ya = gf.Variable("yalpha", -2, 0.1, -10, 10)
        pdf = gf.ProdPdf("totalpdf", [gf.ExpPdf("xpdf", x, xa), gf.ExpPdf("ypdf", y, ya)])
        pdf.setData(data)
        fm = gf.FitManager(pdf, precision=prec, tolerance=0.01)
        fm.verbosity = 0
        assert fm.fit().valid
        assert abs(xa.value + 1.5) <= 3 / math.sqrt(N) * 1.5
        assert abs(ya.value + 0.75) <= 3 / math.sqrt(N) * 0.75
        out[prec] = (xa.value, xa.error, ya.value, ya.error)
    (x64, ex, y64, ey), (xm, _, ym, _) = out["fp64"], out["mixed"]
    assert abs(xm - x64) < 0.01 * ex and abs(ym - y64) < 0.01 * ey
