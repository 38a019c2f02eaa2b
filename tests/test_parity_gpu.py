"""GPU parity: the engine's NLL, gradient, normalisations and fits against the
FP64 oracle on identical seeded inputs.

Tolerances (written per test): NLL 1e-6 relative for the mixed path (FP32
events, FP64 reductions) and 1e-10 for the FP64 path; fitted parameters
within 0.01 sigma of the oracle fit.
"""
import math

import numpy as np
import pytest

import goofit_gb300 as gf
from goofit_gb300 import _abi as A
from goofit_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

NLL_RTOL = {"mixed": 1e-6, "fp64": 1e-10}


def tree(pdf):
    nodes, params, obs = pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    mask = [0 if v.fixed else 1 for v in params]
    pv = np.array([v.value for v in params])
    return nodes, olist, params, mask, pv


def engine_for(pdf, data, prec):
    nodes, olist, params, mask, pv = tree(pdf)
    eng = gf.Engine(prec)
    eng.set_tree(nodes, olist, len(params), mask)
    eng.upload(np.vstack([data.column(o) for o in pdf.getObservables()]))
    return eng, nodes, olist, params, mask, pv


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
@pytest.mark.parametrize("n", [1, 7, 1000, 100_000])
def test_c1_nll_parity(prec, n):
    wl = W.make_c1(n, seed=11)
    eng, nodes, olist, params, mask, pv = engine_for(wl.pdf, wl.data, prec)
    for a in (-0.3, -0.7, -1.3):
        p = np.array([a])
        ref = O.nll(nodes, olist, p, wl.data.to_numpy())
        got, g = eng.nll_grad(p)
        # relative 1e-6 (mixed) / 1e-10 (fp64); for a handful of events the NLL is near zero, so an
        # absolute bound of the same size per event applies as well
        tol = dict(rel=NLL_RTOL[prec], abs=NLL_RTOL[prec] * n)
        assert got == pytest.approx(ref, **tol), (a, got, ref)
        assert eng.nll(p) == pytest.approx(ref, **tol)
        if n >= 1000:
            fd = O.fd_grad(nodes, olist, p, wl.data.to_numpy(), [0])
            # the gradient is a difference of sums of n O(1) terms; an error below 1e-3 sqrt(n) moves
            # the fitted minimum (curvature ~ n) by less than 1e-3 sigma
            assert g[0] == pytest.approx(fd[0], rel=1e-5, abs=1e-3 * math.sqrt(n))


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_nll_over_thirty_decades_of_probability(prec):
    """Event probabilities from 1 down to ~1e-37 (every FP32 exponent the mixed event pass meets in
    practice): its per-iteration log of the product of probabilities (exact mantissa/exponent split) and
    its Newton-refined reciprocal keep the NLL within 1e-6 and the gradient within 1e-5 of FP64."""
    wl = W.make_c1(16, seed=3)
    x = wl.pdf.getObservables()[0]
    data = gf.UnbinnedDataSet(x)
    rng = np.random.Generator(np.random.PCG64(17))
    data.from_numpy(rng.uniform(x.lowerlimit, x.upperlimit, 100_000).reshape(1, -1))
    eng, nodes, olist, params, mask, pv = engine_for(wl.pdf, data, prec)
    for a in (-2.0, -6.0, -8.5):
        p = np.array([a])
        ref = O.nll(nodes, olist, p, data.to_numpy())
        got, g = eng.nll_grad(p)
        assert got == pytest.approx(ref, rel=NLL_RTOL[prec]), (a, got, ref)
        fd = O.fd_grad(nodes, olist, p, data.to_numpy(), [0], h=1e-6)
        assert g[0] == pytest.approx(fd[0], rel=1e-5), (a, g[0], fd[0])


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
@pytest.mark.parametrize("n", [20_000, 2_000_000])
def test_c2_nll_and_gradient_parity(prec, n):
    wl = W.make_c2(n, seed=5)
    eng, nodes, olist, params, mask, pv = engine_for(wl.pdf, wl.data, prec)
    data = wl.data.to_numpy()
    names = [v.name for v in params]
    for shift in (0.0, 0.05):
        p = pv.copy()
        p[names.index("alpha")] += shift
        p[names.index("sigma")] -= shift / 2
        ref = O.nll(nodes, olist, p, data)
        got, g = eng.nll_grad(p)
        assert got == pytest.approx(ref, rel=NLL_RTOL[prec]), (shift, got, ref)
        assert eng.nll(p) == pytest.approx(ref, rel=NLL_RTOL[prec])
        if n <= 20_000:
            free = [i for i, m in enumerate(mask) if m]
            fd = O.fd_grad(nodes, olist, p, data, free, h=1e-6)
            np.testing.assert_allclose(g, fd, rtol=2e-4, atol=2e-3 * math.sqrt(n))


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_c2_normalisations(prec):
    wl = W.make_c2(5000, seed=3)
    eng, nodes, olist, params, mask, pv = engine_for(wl.pdf, wl.data, prec)
    eng.set_params(pv)
    I, N = eng.normalize()
    _, Io, No = O.evaluate(nodes, olist, pv, wl.data.to_numpy())
    np.testing.assert_allclose(I, Io, rtol=1e-6 if prec == "mixed" else 1e-12)
    np.testing.assert_allclose(N, No, rtol=1e-6 if prec == "mixed" else 1e-12)


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_per_event_values(prec):
    wl = W.make_c2(3000, seed=4)
    eng, nodes, olist, params, mask, pv = engine_for(wl.pdf, wl.data, prec)
    eng.set_params(pv)
    for metric in (A.GF_METRIC_PROB, A.GF_METRIC_EVAL, A.GF_METRIC_NLL):
        got = eng.eval_events(metric)
        ref = O.evaluate(nodes, olist, pv, wl.data.to_numpy(), metric=metric)[0]
        np.testing.assert_allclose(got, ref, rtol=1e-5 if prec == "mixed" else 1e-12)


def test_reference_golden_values_through_engine():
    # tests/simple/NormalizeTest.cpp:57-100 and :176-219 through the GPU path
    x = gf.Observable("xvar", -5, 10)
    g = gf.GaussianPdf("gausspdf", x, gf.Variable("mean", 1.5), gf.Variable("sigma", 2.5))
    grid = g.makeGrid()
    g.setData(grid)
    vv = g.getCompProbsAtDataPoints()
    for i, v in {0: 0.00587129964482, 20: 0.0624318782242, 40: 0.157287605852, 60: 0.0938855055588}.items():
        assert vv[0][i] == pytest.approx(v, rel=1.2e-5)
    assert g.normalize() == pytest.approx(6.26657, rel=1e-5)
    x.value = 1.2
    assert g.getValue(gf.EvalFunc.Prob) == pytest.approx(0.15843208471746245, rel=1.2e-5)
    assert g.getValue(gf.EvalFunc.Eval) == pytest.approx(0.99282585857903813, rel=1.2e-5)
    ev = g.evaluateAtPoints(x)
    assert ev[20] == pytest.approx(0.0624318782242, rel=1.2e-5)


def test_min_conv_sums_through_engine():
    # python/tests/test_min_conv.py:7-50 through the GPU path
    x = gf.Observable("xvar", 1690, 1890)
    x.setNumBins(200)
    pure = gf.ExpPdf("pureExp", x, gf.Variable("expAlpha", 0.4676863526561826), gf.Variable("expX0", 1860.0))
    gauss = gf.GaussianPdf("gauss", x, gf.Variable("zero", 0.0), gf.Variable("sigma", 3.4, 0.1, 0.1, 5))
    conv = gf.ConvolutionPdf("convolution", x, pure, gauss)
    conv.setIntegrationConstants(1695, 1885, 0.1)
    grid = conv.makeGrid()
    conv.setData(grid)
    probs = conv.getCompProbsAtDataPoints()
    assert len(probs) == 3
    assert np.asarray(probs).shape == (3, 200)
    assert np.sum(np.asarray(probs), axis=1) == pytest.approx([1.0, 1.0, 0.0], rel=1e-5, abs=1e-12)


def test_known_normalize_through_engine():
    # tests/simple/NormalizeTest.cpp:15-55 through the GPU path (fit with the analytic gradient)
    d = O.mt19937_exponential(137, 1.5, 1000)
    x = gf.Observable("xvar", 0, 10)
    data = gf.UnbinnedDataSet(x)
    data.from_numpy(d[(d >= 0) & (d <= 10)].reshape(1, -1))
    alpha = gf.Variable("alpha", -2, 0.1, -10, 10)
    pdf = gf.ExpPdf("exppdf", x, alpha)
    pdf.setData(data)
    assert pdf.integrate(0, 10) == pytest.approx(0.5, rel=1.2e-5)
    assert pdf.normalize() == pytest.approx(0.5, rel=1.2e-5)
    fm = gf.FitManager(pdf, tolerance=0.01)
    fm.verbosity = 0
    fm.fit()
    assert bool(fm)
    assert alpha.value == pytest.approx(-1.5, rel=0.05)
    # within 0.01 sigma of the reference's quoted normalisation 0.665099
    sig_I = alpha.error / alpha.value ** 2
    assert abs(pdf.normalize() - 0.665099) < 0.01 * sig_I + 1e-5
    assert pdf.normalize() == pytest.approx(pdf.integrate(0, 10), rel=1e-6)


def _oracle_fit(nodes, olist, params, pv, data, tol):
    free = [i for i, v in enumerate(params) if not v.fixed]
    m = gf.Minimizer(pv, [v.error for v in params], [v.lowerlimit for v in params],
                     [v.upperlimit for v in params], [0 if v.fixed else 1 for v in params],
                     [1 if v.fixed else 0 for v in params], tolerance=tol)
    r = m.minimize(lambda p: O.nll(nodes, olist, p, data))
    return r, free


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_c1_fit_parity(prec):
    wl = W.make_c1(100_000, seed=1)
    nodes, olist, params, mask, pv = tree(wl.pdf)
    ro, free = _oracle_fit(nodes, olist, params, pv, wl.data.to_numpy(), 0.001)
    fm = gf.FitManager(wl.pdf, precision=prec, tolerance=0.001)
    fm.verbosity = 0
    r = fm.fit()
    assert r.valid and ro.valid
    for i in free:
        assert abs(r.values[i] - ro.values[i]) < 0.01 * ro.errors[i]
        assert r.errors[i] == pytest.approx(ro.errors[i], rel=0.01)
    assert r.fmin == pytest.approx(ro.fmin, rel=NLL_RTOL[prec])


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_c2_fit_parity_small(prec):
    wl = W.make_c2(20_000, seed=7)
    nodes, olist, params, mask, pv = tree(wl.pdf)
    ro, free = _oracle_fit(nodes, olist, params, pv, wl.data.to_numpy(), 0.001)
    wl.reset()
    fm = gf.FitManager(wl.pdf, precision=prec, tolerance=0.001)
    fm.verbosity = 0
    r = fm.fit()
    assert r.valid and ro.valid
    for i in free:
        assert abs(r.values[i] - ro.values[i]) < 0.01 * ro.errors[i], (params[i].name, r.values[i], ro.values[i])
        assert r.errors[i] == pytest.approx(ro.errors[i], rel=0.02)
    assert r.fmin == pytest.approx(ro.fmin, rel=NLL_RTOL[prec])


def test_numerical_and_analytic_gradient_fits_agree():
    wl = W.make_c2(50_000, seed=8)
    res = {}
    for grad in ("analytic", "numerical"):
        wl.reset()
        fm = gf.FitManager(wl.pdf, precision="fp64", gradient=grad, tolerance=0.001)
        fm.verbosity = 0
        res[grad] = fm.fit()
    a, b = res["analytic"], res["numerical"]
    assert a.valid and b.valid
    assert a.nfcn < b.nfcn
    free = [i for i, v in enumerate(wl.pdf.getParameters()) if not v.fixed]
    for i in free:
        assert abs(a.values[i] - b.values[i]) < 0.01 * b.errors[i]


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_batched_toys_match_single_evaluations(prec):
    sizes = [5_000, 17, 60_000, 1, 20_001, 4096, 0, 333]
    wl = W.make_c2(10, seed=1)
    nodes, olist, params, mask, pv = tree(wl.pdf)
    eng = gf.Engine(prec)
    eng.set_tree(nodes, olist, len(params), mask)
    eng.set_num_toys(len(sizes))
    datas = []
    rng = np.random.default_rng(9)
    for t, n in enumerate(sizes):
        d = W.c2_data(n, seed=100 + t) if n else np.zeros(0)
        datas.append(d.reshape(1, -1))
        eng.upload(datas[-1], toy=t)
    P = np.tile(pv, (len(sizes), 1))
    names = [v.name for v in params]
    P[:, names.index("alpha")] *= 1 + 0.1 * rng.uniform(-1, 1, len(sizes))
    P[:, names.index("sigma")] *= 1 + 0.1 * rng.uniform(-1, 1, len(sizes))
    active = np.array([1 if n else 0 for n in sizes], dtype=np.int32)
    nll, G = eng.nll_batch(P, active=active, grad=True)
    for t, n in enumerate(sizes):
        if not n:
            continue
        ref = O.nll(nodes, olist, P[t], datas[t])
        assert nll[t] == pytest.approx(ref, rel=NLL_RTOL[prec] * 10), (t, n)
    # the empty toy alone reports a zero NLL, as GooFit::abort does
    with pytest.raises(A.EngineError) as ei:
        eng.nll(P[6], toy=6)
    assert ei.value.code == A.GF_ERR_ZERO_NLL


def test_invalid_normalisation_is_reported():
    wl = W.make_c2(1000, seed=2)
    eng, nodes, olist, params, mask, pv = engine_for(wl.pdf, wl.data, "mixed")
    p = pv.copy()
    p[[v.name for v in params].index("sigma")] = float("nan")
    with pytest.raises(A.EngineError) as ei:
        eng.nll(p)
    assert ei.value.code == A.GF_ERR_NAN_NORM
    # the engine stays usable afterwards
    assert eng.nll(pv) == pytest.approx(O.nll(nodes, olist, pv, wl.data.to_numpy()), rel=1e-6)


def test_events_outside_convolution_range_are_rejected():
    wl = W.make_c2(100, seed=2)
    eng, nodes, olist, params, mask, pv = engine_for(wl.pdf, wl.data, "mixed")
    bad = wl.data.to_numpy().copy()
    bad[0, 3] = 50.0
    with pytest.raises(A.EngineError) as ei:
        eng.upload(bad)
    assert ei.value.code == A.GF_ERR_INVALID
