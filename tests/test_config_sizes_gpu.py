"""GPU-vs-oracle parity at the benchmark configurations' own sizes.

* C2 composite model: 2,000,000 events, 10,000-bin numeric normalisation.
* C3 Amp3Body: 500,000 events, 1500 x 1500 normalisation bins (all 64 integrals I_ij).
* C4 batched toys: all 1024 toys of Poisson(20,000) events.
* C5 Amp4Body: 300,000 events, 2,000,000 normalisation events (all 36 sums G_ab).

Each is checked against the FP64 oracle on the same inputs:
* NLL within 1e-6 relative (mixed) and 1e-10 (FP64).
* Integrals within 2e-5 (mixed) and 1e-10 (FP64) relative to the largest entry.
* Analytic gradient within 2e-4 relative + 2e-3 sqrt(n) of the oracle's central differences.

The fits run at MIGRAD tolerance 0.01 (EDM < 1e-5, each fit within ~0.005 sigma of its minimum), so the
comparisons measure the arithmetic, not the stopping rule.
* The mixed-precision fit must lie within 0.01 sigma of the FP64 fit.
* It must also lie within 0.01 sigma of the oracle's own minimum. That distance is one Newton step with
  the oracle's gradient at the fitted point and the fit's covariance (`oracle.minimum_offset_sigma`).
"""
import math

import numpy as np
import pytest

import goofit_gb300 as gf
from goofit_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

NLL_RTOL = {"mixed": 1e-6, "fp64": 1e-10}
AMP_RTOL = {"mixed": 2e-5, "fp64": 1e-10}
FIT_TOL = 0.01
SIGMA = 0.01


def tree(pdf):
    nodes, params, obs = pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    nd = pdf._nondiff_all()
    mask = [0 if (v.fixed or id(v) in nd) else 1 for v in params]
    pv = np.array([v.value for v in params])
    return nodes, olist, params, mask, pv


def engine(pdf, cols, prec, norm=None):
    nodes, olist, params, mask, pv = tree(pdf)
    eng = gf.Engine(prec)
    eng.set_tree(nodes, olist, len(params), mask)
    if norm is not None:
        eng.set_norm_events(0, norm)
    eng.upload(cols)
    eng.set_params(pv)
    return eng, nodes, olist, params, mask, pv


def fit_pair_and_oracle(wl, norm=None):
    """Mixed and FP64 fits of the workload (tolerance 0.01); returns the largest mixed-vs-FP64 and
    mixed-vs-oracle distances in sigma, and the relative NLL error of the mixed minimum."""
    nodes, olist, params, mask, pv = tree(wl.pdf)
    free = [i for i, m in enumerate(mask) if m]
    data = wl.data.to_numpy()
    res = {}
    for prec in ("fp64", "mixed"):
        wl.reset()
        fm = gf.FitManager(wl.pdf, precision=prec, tolerance=FIT_TOL)
        fm.verbosity = 0
        r = fm.fit()
        assert r.valid, prec
        res[prec] = (np.array([v.value for v in params]), np.array([v.error for v in params]), fm.covariance, r)
    xm, em, covm, rm = res["mixed"]
    x64, e64, _, _ = res["fp64"]
    d64 = max(abs(xm[i] - x64[i]) / e64[i] for i in free)
    if norm is not None:
        O.set_amp4_norm_events(norm)
    doff = float(np.max(O.minimum_offset_sigma(nodes, olist, xm, data, covm, free)))
    ref = O.nll(nodes, olist, xm, data)
    return d64, doff, abs(rm.fmin - ref) / abs(ref)


# ---------------------------------------------------------------- C2
def test_c2_full_size_fit():
    wl = W.make_c2(2_000_000, seed=2)
    d64, doff, rel = fit_pair_and_oracle(wl)
    assert d64 < SIGMA, d64
    assert doff < SIGMA, doff
    assert rel < NLL_RTOL["mixed"], rel


# ---------------------------------------------------------------- C3
@pytest.fixture(scope="module")
def c3():
    return W.make_c3(500_000, seed=3)


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_c3_full_size_integrals_and_nll(c3, prec):
    cols = c3.data.to_numpy()
    eng, nodes, olist, params, mask, pv = engine(c3.pdf, cols, prec)
    got = eng.amp3_integrals(0, 8)
    ref = O.amp3_integrals(nodes, olist, pv, 0, 8)
    assert got.shape == (8, 8)
    err = np.abs(got - ref).max() / np.abs(np.diag(ref)).max()
    assert err < AMP_RTOL[prec], err
    free = [i for i, m in enumerate(mask) if m]
    rng = np.random.default_rng(11)
    for trial in range(2):
        p = pv.copy()
        if trial:
            p[free] *= 1 + 0.05 * rng.standard_normal(len(free))
        assert eng.nll(p) == pytest.approx(O.nll(nodes, olist, p, cols), rel=NLL_RTOL[prec]), trial


def test_c3_full_size_gradient(c3):
    cols = c3.data.to_numpy()
    nodes, olist, params, mask, pv = tree(c3.pdf)
    free = [i for i, m in enumerate(mask) if m]
    p = pv.copy()
    p[free] *= 1 + 0.03 * np.random.default_rng(12).standard_normal(len(free))
    fd = O.fd_grad(nodes, olist, p, cols, free, h=1e-5)
    n = cols.shape[1]
    for prec in ("mixed", "fp64"):
        eng = engine(c3.pdf, cols, prec)[0]
        _, g = eng.nll_grad(p)
        np.testing.assert_allclose(g, fd, rtol=2e-4, atol=2e-3 * math.sqrt(n), err_msg=prec)


def test_c3_full_size_fit(c3):
    d64, doff, rel = fit_pair_and_oracle(c3)
    assert d64 < SIGMA, d64
    assert doff < SIGMA, doff
    assert rel < NLL_RTOL["mixed"], rel


# ---------------------------------------------------------------- C5
@pytest.fixture(scope="module")
def c5():
    return W.make_c5(300_000, 2_000_000, seed=5)


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_c5_full_size_sums_and_nll(c5, prec):
    cols = c5.data.to_numpy()
    norm = c5.pdf.norm_events
    assert norm.shape[1] == 2_000_000
    eng, nodes, olist, params, mask, pv = engine(c5.pdf, cols, prec, norm)
    O.set_amp4_norm_events(norm)
    got = eng.amp3_integrals(0, 6)
    ref = O.amp4_gram(nodes, olist, pv, 0, 6)
    err = np.abs(got - ref).max() / np.abs(np.diag(ref)).max()
    assert err < AMP_RTOL[prec], err
    free = [i for i, m in enumerate(mask) if m]
    rng = np.random.default_rng(13)
    for trial in range(2):
        p = pv.copy()
        if trial:
            p[free] *= 1 + 0.05 * rng.standard_normal(len(free))
        assert eng.nll(p) == pytest.approx(O.nll(nodes, olist, p, cols), rel=NLL_RTOL[prec]), trial


def test_c5_full_size_gradient(c5):
    cols = c5.data.to_numpy()
    norm = c5.pdf.norm_events
    nodes, olist, params, mask, pv = tree(c5.pdf)
    free = [i for i, m in enumerate(mask) if m]
    p = pv.copy()
    p[free] *= 1 + 0.03 * np.random.default_rng(14).standard_normal(len(free))
    O.set_amp4_norm_events(norm)
    fd = O.fd_grad(nodes, olist, p, cols, free, h=1e-5)
    n = cols.shape[1]
    for prec in ("mixed", "fp64"):
        eng = engine(c5.pdf, cols, prec, norm)[0]
        _, g = eng.nll_grad(p)
        np.testing.assert_allclose(g, fd, rtol=2e-4, atol=2e-3 * math.sqrt(n), err_msg=prec)


def test_c5_full_size_fit(c5):
    d64, doff, rel = fit_pair_and_oracle(c5, c5.pdf.norm_events)
    assert d64 < SIGMA, d64
    assert doff < SIGMA, doff
    assert rel < NLL_RTOL["mixed"], rel


# ---------------------------------------------------------------- C4
@pytest.fixture(scope="module")
def c4():
    return W.make_c4(n_toys=1024, seed=4)


def toy_engine(study, prec):
    nodes, params, obs = study.pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    mask = [0 if v.fixed else 1 for v in params]
    eng = gf.Engine(prec)
    eng.set_tree(nodes, olist, len(params), mask)
    eng.set_num_toys(len(study.datas))
    for t, d in enumerate(study.datas):
        eng.upload(d, toy=t)
    return eng, nodes, olist, params, mask


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_c4_all_toys_nll_and_gradient(c4, prec):
    eng, nodes, olist, params, mask = toy_engine(c4, prec)
    pv = np.array([v.value for v in params])
    T = len(c4.datas)
    assert T == 1024
    P = np.tile(pv, (T, 1))
    nll = eng.nll_batch(P)
    for t in range(T):
        assert nll[t] == pytest.approx(O.nll(nodes, olist, pv, c4.datas[t]), rel=NLL_RTOL[prec]), t
    free = [i for i, m in enumerate(mask) if m]
    nll, G = eng.nll_batch(P, grad=True)
    for t in range(0, T, 97):
        fd = O.fd_grad(nodes, olist, pv, c4.datas[t], free, h=1e-6)
        n = c4.datas[t].shape[1]
        np.testing.assert_allclose(G[t], fd, rtol=2e-4, atol=2e-3 * math.sqrt(n), err_msg=str(t))


def test_c4_all_toys_fits(c4):
    out = {}
    for prec in ("fp64", "mixed"):
        eng, nodes, olist, params, mask = toy_engine(c4, prec)
        x0 = np.array([c4.start.get(v.name, v.value) for v in params])
        err = np.array([v.error for v in params])
        lo = np.array([v.lowerlimit for v in params])
        hi = np.array([v.upperlimit for v in params])
        fixed = np.array([1 if v.fixed else 0 for v in params], np.int32)
        limited = np.array([0 if v.fixed else 1 for v in params], np.int32)
        res = eng.fit_batch(np.tile(x0, (len(c4.datas), 1)), err, lo, hi, limited, fixed, tolerance=FIT_TOL)
        assert all(r.valid for r in res), prec
        out[prec] = res
        eng.close()
    free = [i for i, m in enumerate(mask) if m]
    worst = 0.0
    for rm, r64 in zip(out["mixed"], out["fp64"]):
        for i in free:
            worst = max(worst, abs(rm.values[i] - r64.values[i]) / r64.errors[i])
    assert worst < SIGMA, worst
    for t in range(0, len(c4.datas), 128):
        rm = out["mixed"][t]
        off = O.minimum_offset_sigma(nodes, olist, rm.values, c4.datas[t], rm.covariance, free, h=1e-6)
        assert off.max() < SIGMA, (t, off)
