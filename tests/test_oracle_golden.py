"""The oracle against the reference's own known-answer tests.

Each case restates a reference test scenario (file:line cited) and checks
the oracle's numbers against the values that test asserts, with Catch2's
default Approx tolerance (100 * FLT_EPSILON relative) unless stated.
"""
import math

import numpy as np
import pytest
from scipy.optimize import brentq

import goofit_gb300 as gf
from goofit_gb300 import _abi as A
from oracle import oracle as O

APPROX = 100 * np.finfo(np.float32).eps


def approx(a, b, eps=APPROX):
    return abs(a - b) <= eps * max(abs(a), abs(b))


def flat(pdf):
    nodes, params, obs = pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    pv = np.array([v.value for v in params])
    return nodes, olist, params, pv


def normalize_test_data():
    # tests/simple/NormalizeTest.cpp:16-30: mt19937(137), exponential(1.5), 1000 draws, kept if in [0, 10]
    d = O.mt19937_exponential(137, 1.5, 1000)
    return d[(d >= 0) & (d <= 10)]


def test_known_normalize_integral():
    # tests/simple/NormalizeTest.cpp:38-42: ExpPdf integral over [0,10] at alpha=-2 is 0.5
    x = gf.Observable("xvar", 0, 10)
    alpha = gf.Variable("alpha", -2, 0.1, -10, 10)
    pdf = gf.ExpPdf("exppdf", x, alpha)
    nodes, olist, params, pv = flat(pdf)
    data = normalize_test_data()
    _, I, N = O.evaluate(nodes, olist, pv, data.reshape(1, -1))
    assert approx(I[0], 0.5)
    assert approx(N[0], 2.0)


def test_known_normalize_fit():
    # tests/simple/NormalizeTest.cpp:44-54 asserts alpha ~ -1.5 (5%) and normalize() = 0.665099 after a
    # Minuit2 fit.  That golden value is Minuit2's stopping point (EDM tolerance), so the oracle's exact
    # minimum must agree with it within 0.01 sigma, and the project MIGRAD must land on the exact minimum.
    x = gf.Observable("xvar", 0, 10)
    alpha = gf.Variable("alpha", -2, 0.1, -10, 10)
    pdf = gf.ExpPdf("exppdf", x, alpha)
    nodes, olist, params, pv = flat(pdf)
    data = normalize_test_data().reshape(1, -1)
    f = lambda a: O.nll(nodes, olist, [a], data)
    score = lambda a: (f(a + 1e-6) - f(a - 1e-6)) / 2e-6
    a_hat = brentq(score, -3.0, -0.5, xtol=1e-12)
    integ = lambda a: (math.exp(10 * a) - 1) / a
    curv = (f(a_hat + 1e-3) + f(a_hat - 1e-3) - 2 * f(a_hat)) / 1e-6
    sigma_a = 1 / math.sqrt(curv)
    sigma_I = abs(integ(a_hat + sigma_a) - integ(a_hat - sigma_a)) / 2
    assert abs(a_hat + 1.5) < 0.05 * 1.5
    assert abs(integ(a_hat) - 0.665099) < 0.01 * sigma_I
    m = gf.Minimizer([-2.0], [0.1], [-10.0], [10.0], [1], [0], tolerance=0.001)
    r = m.minimize(lambda p: f(p[0]))
    assert r.valid
    assert abs(r.values[0] - a_hat) < 0.01 * sigma_a
    assert r.errors[0] == pytest.approx(sigma_a, rel=2e-2)


def test_gaussian_fit_mean():
    # tests/convert/GaussianTest.cpp:27-46: the fitted mean of a GaussianPdf (normalised over all R,
    # src/PDFs/basic/GaussianPdf.cu:28-35) is the sample mean; the reference quotes 0.665178392.
    d = normalize_test_data()
    x = gf.Observable("xvar", 0, 10)
    g = gf.GaussianPdf("g", x, gf.Variable("alpha", 1, 0.1, -10, 10), gf.Variable("sigma", 1, 0, 3))
    nodes, olist, params, pv = flat(g)
    f = lambda p: O.nll(nodes, olist, p, d.reshape(1, -1))
    m = gf.Minimizer([1.0, 1.0], [0.1, 0.3], [-10.0, 0.0], [10.0, 3.0], [1, 1], [0, 0], tolerance=0.001)
    r = m.minimize(f)
    assert r.valid
    assert r.values[0] == pytest.approx(d.mean(), abs=0.01 * r.errors[0])
    assert abs(r.values[0] - 0.665178392) < 0.01 * r.errors[0]


def gauss_grid_values():
    return {0: 0.00587129964482, 20: 0.0624318782242, 40: 0.157287605852, 60: 0.0938855055588}


def test_1d_grid_gaussian():
    # tests/simple/NormalizeTest.cpp:57-100
    x = gf.Observable("xvar", -5, 10)
    g = gf.GaussianPdf("gausspdf", x, gf.Variable("mean", 1.5), gf.Variable("sigma", 2.5))
    grid = g.makeGrid()
    assert approx(grid.getValue(x, 0), -4.925) and approx(grid.getValue(x, 20), -1.925)
    nodes, olist, params, pv = flat(g)
    probs, I, N = O.evaluate(nodes, olist, pv, grid.to_numpy())
    assert len(probs) == 100
    for i, v in gauss_grid_values().items():
        assert approx(probs[i], v), (i, probs[i], v)


def test_2d_grid_product():
    # tests/simple/NormalizeTest.cpp:104-174: component probabilities of a 2-D product on its grid
    x = gf.Observable("xvar", -5, 10)
    y = gf.Observable("yvar", -5, 10)
    g1 = gf.GaussianPdf("g1", x, gf.Variable("mean1", 1.5), gf.Variable("sigma1", 2.5))
    g2 = gf.GaussianPdf("g2", y, gf.Variable("mean2", -1), gf.Variable("sigma2", 0.5))
    prod = gf.ProdPdf("product", [g1, g2])
    grid = prod.makeGrid()
    assert approx(grid.getValue(y, 100 * 20), -1.925)
    assert approx(grid.getValue(x, 60), 4.075)
    nodes, olist, params, pv = flat(g1)
    probs, _, _ = O.evaluate(nodes, olist, pv, grid.column(x).reshape(1, -1))
    assert len(probs) == 10000
    for i, v in gauss_grid_values().items():
        assert approx(probs[i], v)
    # the product itself normalises each factor separately
    nodes, olist, params, pv = flat(prod)
    pp, _, _ = O.evaluate(nodes, olist, pv, grid.to_numpy())
    gx = np.exp(-0.5 * (grid.column(x) - 1.5) ** 2 / 6.25) / (2.5 * math.sqrt(2 * math.pi))
    gy = np.exp(-0.5 * (grid.column(y) + 1) ** 2 / 0.25) / (0.5 * math.sqrt(2 * math.pi))
    np.testing.assert_allclose(pp, gx * gy, rtol=1e-12, atol=1e-300)


def test_1d_eval_gaussian():
    # tests/simple/NormalizeTest.cpp:176-219
    x = gf.Observable("xvar", -5, 10)
    g = gf.GaussianPdf("gausspdf", x, gf.Variable("mean", 1.5), gf.Variable("sigma", 2.5))
    nodes, olist, params, pv = flat(g)
    _, I, _ = O.evaluate(nodes, olist, pv, np.array([[1.2, 7.2]]))
    assert approx(I[0], 6.26657, eps=1e-5)
    prob, _, _ = O.evaluate(nodes, olist, pv, np.array([[1.2, 7.2]]), metric=A.GF_METRIC_PROB)
    ev, _, _ = O.evaluate(nodes, olist, pv, np.array([[1.2, 7.2]]), metric=A.GF_METRIC_EVAL)
    assert approx(prob[0], 0.15843208471746245) and approx(ev[0], 0.99282585857903813)
    assert approx(prob[1], 0.0118618339389365) and approx(ev[1], 0.0743330208507896)


def test_addpdf_component_normalisation():
    # tests/simple/AddNormTest.cpp:16-44
    x = gf.Observable("xvar", -5, 10)
    mean = gf.Variable("mean", 1.5)
    ga = gf.GaussianPdf("gaussA", x, mean, gf.Variable("sigmaA", 2.5))
    gb = gf.GaussianPdf("gaussB", x, mean, gf.Variable("sigmaB", 0.8))
    s = gf.AddPdf("sum", gf.Variable("frac", 0.6), ga, gb)
    grid = s.makeGrid()
    vv = []
    for p in (s, ga, gb):
        nodes, olist, params, pv = flat(p)
        vv.append(O.evaluate(nodes, olist, pv, grid.to_numpy())[0])
    for i in range(0, len(vv[0]), 7):
        assert approx(vv[0][i], 0.6 * vv[1][i] + 0.4 * vv[2][i])


def test_min_conv_sums():
    # python/tests/test_min_conv.py:7-50: grid probabilities of a convolution and its components sum to [1, 1, 0]
    x = gf.Observable("xvar", 1690, 1890)
    x.setNumBins(200)
    pure = gf.ExpPdf("pureExp", x, gf.Variable("expAlpha", 0.4676863526561826), gf.Variable("expX0", 1860.0))
    gauss = gf.GaussianPdf("gauss", x, gf.Variable("zero", 0.0), gf.Variable("sigma", 3.4, 0.1, 0.1, 5))
    conv = gf.ConvolutionPdf("convolution", x, pure, gauss)
    conv.setIntegrationConstants(1695, 1885, 0.1)
    grid = conv.makeGrid().to_numpy()
    sums = []
    for p in (conv, pure, gauss):
        nodes, olist, params, pv = flat(p)
        sums.append(O.evaluate(nodes, olist, pv, grid)[0].sum())
    assert sums == pytest.approx([1.0, 1.0, 0.0])


def test_convolution_memo_is_bit_identical():
    # the per-offset memo of the oracle gives the brute-force per-event sums bit for bit
    wl_x = gf.Observable("x", -5.0, 10.0)
    wl_x.setNumBins(500)
    conv = gf.ConvolutionPdf("c", wl_x, gf.ExpPdf("m", wl_x, gf.Variable("a", -0.6)),
                             gf.GaussianPdf("r", wl_x, gf.Variable("mu", 0.0), gf.Variable("s", 0.3)))
    nodes, olist, params, pv = flat(conv)
    xs = np.random.default_rng(3).uniform(-5, 10, 300).reshape(1, -1)
    a = O.evaluate(nodes, olist, pv, xs, metric=A.GF_METRIC_EVAL, brute_force=False)[0]
    b = O.evaluate(nodes, olist, pv, xs, metric=A.GF_METRIC_EVAL, brute_force=True)[0]
    assert np.array_equal(a, b)


def test_extended_add_term():
    # AddPdf::calculateNLL extended term (src/PDFs/combine/AddPdf.cu:187-204)
    x = gf.Observable("x", 0, 10)
    e1 = gf.ExpPdf("e1", x, gf.Variable("a1", -0.5))
    e2 = gf.ExpPdf("e2", x, gf.Variable("a2", -2.0))
    n1, n2 = gf.Variable("n1", 300.0, 1, 0, 1e4), gf.Variable("n2", 700.0, 1, 0, 1e4)
    s = gf.AddPdf("s", [n1, n2], [e1, e2])
    nodes, olist, params, pv = flat(s)
    xs = np.linspace(0.01, 9.9, 1000).reshape(1, -1)
    total = O.nll(nodes, olist, pv, xs)
    probs = O.evaluate(nodes, olist, pv, xs, metric=A.GF_METRIC_PROB)[0]
    manual = -np.log(probs).sum() + (1000.0 - 1000 * math.log(1000.0))
    assert total == pytest.approx(manual, rel=1e-12)
