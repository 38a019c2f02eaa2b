"""Amplitude recompute mode (gf_set_amp_mode): the derivatives of the amplitudes by floated line-shape (Amp4Body)
or resonance (Amp3Body) parameters recomputed per event in the gradient pass and per normalisation point in the
integrals, instead of stored in per-event and per-point columns.

* Store and recompute gradients agree to 1e-10 (FP64) and 1e-6 (mixed) of the largest component.  The mixed
  comparison uses the CUDA-core Gram kernel in both modes (GF_GRAM=cuda), so that both reduce the same FP32
  products in the same order.
* Both gradients agree with central finite differences of the FP64 oracle at h = 1e-5 (relative to
  max(1, |p|)): rtol 2e-4 (mixed) / 1e-6 (FP64), atol 2e-3 sqrt(n).
* The NLL is the same in both modes; a fit in recompute mode reaches the store-mode fit (values within
  1e-3 sigma).
* Auto mode recomputes only above its memory budget; the mode cannot change once events are uploaded.
"""
import math

import numpy as np
import pytest

import goofit_gb300 as gf
from goofit_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

NLL_RTOL = {"mixed": 1e-6, "fp64": 1e-10}
MODE_RTOL = {"mixed": 1e-6, "fp64": 1e-10}
N_NORM = 100_000
C3_FLOAT = ("rho770_mass", "rho770_width", "kst892_mass", "f2_1270_width")


def tree(pdf):
    nodes, params, obs = pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    nd = pdf._nondiff_all()
    mask = [0 if (v.fixed or id(v) in nd) else 1 for v in params]
    return nodes, olist, params, mask, np.array([v.value for v in params])


def c3_model():
    pdf = W.c3_model(300)[0]
    for v in pdf.getParameters():
        if v.name in C3_FLOAT:
            v.fixed = False
            v.error = 0.01 * v.value
            v.lowerlimit, v.upperlimit = 0.5 * v.value, 1.5 * v.value
    return pdf


@pytest.fixture(scope="module")
def models():
    c5 = W.c5_model(N_NORM, float_lineshapes=True)[0]
    c5_cols = W.c5_generate(W.c5_model(N_NORM)[0], 10_000, seed=52, batch=200_000)
    c3 = c3_model()
    c3_cols = W.c3_generate(W.c3_model(300)[0], 20_000, seed=31, batch=1_000_000)
    return {"c5": (c5, c5_cols), "c3": (c3, c3_cols)}


def engine(pdf, cols, prec, mode, budget=0):
    nodes, olist, params, mask, pv = tree(pdf)
    eng = gf.Engine(prec)
    eng.set_amp_mode(mode, budget)
    eng.set_tree(nodes, olist, len(params), mask)
    if hasattr(pdf, "norm_events"):
        eng.set_norm_events(0, pdf.norm_events)
        O.set_amp4_norm_events(pdf.norm_events)
    eng.upload(cols)
    eng.set_params(pv)
    return eng, nodes, olist, params, mask, pv


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
@pytest.mark.parametrize("model", ["c5", "c3"])
def test_recomputed_gradient_matches_stored_and_finite_differences(models, model, prec, monkeypatch):
    monkeypatch.setenv("GF_GRAM", "cuda")
    pdf, cols = models[model]
    es, nodes, olist, params, mask, pv = engine(pdf, cols, prec, "store")
    er = engine(pdf, cols, prec, "recompute")[0]
    assert es.amp_recomputing() is False and er.amp_recomputing() is True
    free = [i for i, m in enumerate(mask) if m]
    assert len(free) == (20 if model == "c5" else 18)
    p = pv.copy()
    p[free] *= 1 + 0.02 * np.random.default_rng(3).standard_normal(len(free))
    fs, gs = es.nll_grad(p)
    fr, gr = er.nll_grad(p)
    ref = O.nll(nodes, olist, p, cols)
    assert fs == pytest.approx(ref, rel=NLL_RTOL[prec]) and fr == pytest.approx(ref, rel=NLL_RTOL[prec])
    assert fr == pytest.approx(fs, rel=MODE_RTOL[prec])
    assert er.nll(p) == pytest.approx(es.nll(p), rel=MODE_RTOL[prec])
    assert np.abs(gr - gs).max() <= MODE_RTOL[prec] * np.abs(gs).max(), np.abs(gr - gs).max() / np.abs(gs).max()
    fd = O.fd_grad(nodes, olist, p, cols, free, h=1e-5)
    n = cols.shape[1]
    for g in (gs, gr):
        np.testing.assert_allclose(g, fd, rtol=2e-4 if prec == "mixed" else 1e-6, atol=2e-3 * math.sqrt(n))
    # a line-shape / resonance change rebuilds the value columns and the integrals in both modes
    p2 = p.copy()
    p2[free[-1]] *= 1.01
    assert er.nll_grad(p2)[0] == pytest.approx(es.nll_grad(p2)[0], rel=MODE_RTOL[prec])
    es.close()
    er.close()


def test_recompute_mode_fit_reaches_the_store_mode_fit(models):
    pdf, cols = models["c3"]
    nodes, olist, params, mask, pv = tree(pdf)
    free = [i for i, m in enumerate(mask) if m]
    x0 = pv.copy()
    x0[free] *= 1.03
    err = np.array([v.error for v in params])
    lo = np.array([v.lowerlimit for v in params])
    hi = np.array([v.upperlimit for v in params])
    fixed = np.array([0 if m else 1 for m in mask], dtype=np.int32)
    limited = np.array([1 if (m and l != h) else 0 for m, l, h in zip(mask, lo, hi)], dtype=np.int32)
    res = {}
    for mode in ("store", "recompute"):
        eng = engine(pdf, cols, "fp64", mode)[0]
        res[mode] = eng.fit(x0, err, lo, hi, limited, fixed, tolerance=0.01)
        eng.close()
    assert res["store"].valid and res["recompute"].valid
    assert res["recompute"].fmin == pytest.approx(res["store"].fmin, rel=1e-12, abs=1e-6)
    for i in free:
        assert res["recompute"].values[i] == pytest.approx(res["store"].values[i], abs=1e-3 * res["store"].errors[i])


def test_auto_mode_recomputes_above_its_budget(models):
    pdf, cols = models["c3"]
    small = engine(pdf, cols, "mixed", "auto", budget=1 << 20)[0]
    assert small.amp_recomputing() is True
    large = engine(pdf, cols, "mixed", "auto")[0]
    assert large.amp_recomputing() is False
    with pytest.raises(Exception):
        large.set_amp_mode("recompute")
    # no floated resonance parameter: nothing to recompute whatever the mode
    fixed_pdf = W.c3_model(300)[0]
    plain = engine(fixed_pdf, cols, "mixed", "recompute")[0]
    assert plain.amp_recomputing() is False
    for e in (small, large, plain):
        e.close()
