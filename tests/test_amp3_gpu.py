"""GPU parity of the Amp3Body path (Dalitz plot with relativistic Breit-Wigner resonances) against the
FP64 oracle: cached amplitudes, normalisation integrals, NLL, gradient and fits.

Tolerances (written per test): NLL 1e-6 relative for the mixed path and 1e-10 for FP64; amplitudes and
integrals 2e-5 (mixed, FP32 arithmetic) and 1e-10 (FP64) relative to the largest entry; fitted
parameters of the mixed path within 0.01 sigma of the FP64 path.
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
AMP_RTOL = {"mixed": 2e-5, "fp64": 1e-10}


def tree(pdf):
    nodes, params, obs = pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    nd = pdf._nondiff_all()
    mask = [0 if (v.fixed or id(v) in nd) else 1 for v in params]
    pv = np.array([v.value for v in params])
    return nodes, olist, params, mask, pv


@pytest.fixture(scope="module")
def c3_events():
    pdf, _, _ = W.c3_model(300)
    return W.c3_generate(pdf, 20_000, seed=31, batch=1_000_000)


def engine(pdf, cols, prec):
    nodes, olist, params, mask, pv = tree(pdf)
    eng = gf.Engine(prec)
    eng.set_tree(nodes, olist, len(params), mask)
    eng.upload(cols)
    eng.set_params(pv)
    return eng, nodes, olist, params, mask, pv


def test_generated_events_lie_in_the_dalitz_plot(c3_events):
    assert c3_events.shape == (3, 20_000)
    for k in range(0, 20_000, 997):
        assert O.in_dalitz(c3_events[0, k], c3_events[1, k], W.C3_M, W.C3_MK, W.C3_MPI, W.C3_MPI0)


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_cached_amplitudes_match_oracle(c3_events, prec):
    pdf, _, _ = W.c3_model(300)
    eng, nodes, olist, params, mask, pv = engine(pdf, c3_events, prec)
    # the last 5 events are outside the kinematic boundary: their amplitudes are zero
    cols = c3_events.copy()
    cols[0, -5:] = 2.9
    cols[1, -5:] = 2.9
    eng.upload(cols)
    res_nodes = [i for i, n in enumerate(nodes) if n["op"] == A.GF_OP_RES_RBW]
    for r, rn in enumerate(res_nodes):
        got = eng.amp3_cached_wave(0, r)
        ref = O.amp3_resonance(nodes, olist, pv, 0, rn, cols[0], cols[1])
        assert np.all(got[-5:] == 0)
        scale = np.abs(ref).max()
        err = np.abs(got - ref).max() / scale
        assert err < AMP_RTOL[prec], (r, err)


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
@pytest.mark.parametrize("bins", [300, 1500])
def test_integrals_match_oracle(c3_events, prec, bins):
    pdf, _, _ = W.c3_model(bins)
    eng, nodes, olist, params, mask, pv = engine(pdf, c3_events, prec)
    got = eng.amp3_integrals(0, 8)
    ref = O.amp3_integrals(nodes, olist, pv, 0, 8)
    scale = np.abs(np.diag(ref)).max()
    err = np.abs(got - ref).max() / scale
    assert err < AMP_RTOL[prec], err
    np.testing.assert_array_equal(got, got.conj().T)


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_nll_and_gradient_match_oracle(c3_events, prec):
    pdf, _, _ = W.c3_model(300)
    eng, nodes, olist, params, mask, pv = engine(pdf, c3_events, prec)
    free = [i for i, m in enumerate(mask) if m]
    assert len(free) == 14
    rng = np.random.default_rng(7)
    for trial in range(3):
        p = pv.copy()
        if trial:
            p[free] *= 1 + 0.05 * rng.standard_normal(len(free))
        ref = O.nll(nodes, olist, p, c3_events)
        got, g = eng.nll_grad(p)
        assert got == pytest.approx(ref, rel=NLL_RTOL[prec]), (trial, got, ref)
        assert eng.nll(p) == pytest.approx(ref, rel=NLL_RTOL[prec])
        fd = O.fd_grad(nodes, olist, p, c3_events, free, h=1e-6)
        n = c3_events.shape[1]
        # each component is a difference of sums of n O(1) terms: 2e-3 sqrt(n) moves the fitted
        # coefficient (curvature ~ n) by far less than 0.01 sigma
        np.testing.assert_allclose(g, fd, rtol=2e-4, atol=2e-3 * math.sqrt(n))


def test_normalisation_follows_the_coefficients(c3_events):
    """A change of coefficients reuses the cached integrals; a change of a resonance parameter rebuilds them."""
    pdf, _, _ = W.c3_model(300)
    eng, nodes, olist, params, mask, pv = engine(pdf, c3_events, "fp64")
    names = [v.name for v in params]
    p = pv.copy()
    p[names.index("kst892_amp_real")] *= 1.3
    eng.set_params(p)
    Ie, Ne = eng.normalize()
    _, Io, No = O.evaluate(nodes, olist, p, c3_events[:, :1], metric=A.GF_METRIC_EVAL)
    assert Ie[0] == pytest.approx(Io[0], rel=1e-10)
    assert Ne[0] == pytest.approx(No[0], rel=1e-10)
    p2 = p.copy()
    p2[names.index("rho770_mass")] = 0.78
    ref = O.nll(nodes, olist, p2, c3_events)
    assert eng.nll(p2) == pytest.approx(ref, rel=1e-10)
    assert eng.nll(p) == pytest.approx(O.nll(nodes, olist, p, c3_events), rel=1e-10)


def test_fit_fractions_sum_and_cached_waves(c3_events):
    pdf, variables, obs = W.c3_model(300)
    ds = gf.UnbinnedDataSet(obs)
    ds.from_numpy(c3_events)
    pdf.setData(ds)
    ff = np.array(pdf.fit_fractions())
    assert ff.shape == (8, 8)
    assert ff.sum() == pytest.approx(1.0, rel=1e-9)
    w = pdf.getCachedWave(1)
    assert w.shape == (20_000,)
    assert pdf.sumCachedWave(1) == pytest.approx(complex(w.sum()))


def test_mixed_fit_matches_fp64_fit(c3_events):
    out = {}
    for prec in ("fp64", "mixed"):
        pdf, variables, obs = W.c3_model(300)
        ds = gf.UnbinnedDataSet(obs)
        ds.from_numpy(c3_events)
        pdf.setData(ds)
        for v in variables.values():
            v.value *= 1.05
        # tolerance 0.01 (EDM < 1e-5): each fit then sits within ~0.005 sigma of its minimum, so that
        # the 0.01 sigma comparison measures the precision of the NLL, not the stopping rule
        fm = gf.FitManager(pdf, precision=prec, tolerance=0.01)
        fm.verbosity = 0
        r = fm.fit()
        assert r.valid, prec
        assert fm.used_gradient == "analytic"
        out[prec] = {k: (v.value, v.error) for k, v in variables.items()}
    for k, (v64, e64) in out["fp64"].items():
        vm, em = out["mixed"][k]
        assert abs(vm - v64) < 0.01 * e64, (k, vm, v64, e64)
        assert em == pytest.approx(e64, rel=0.01), k


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_resonance_gradient_matches_central_differences(c3_events, prec):
    """dNLL/d(resonance mass, width) through the derivative columns, against central finite differences of
    the FP64 oracle with h = 1e-5."""
    pdf, _, _ = W.c3_model(300)
    for v in pdf.getParameters():
        if v.name in ("rho770_mass", "rho770_width", "kst892_mass", "f2_1270_width"):
            v.fixed = False
    eng, nodes, olist, params, mask, pv = engine(pdf, c3_events, prec)
    free = [i for i, m in enumerate(mask) if m]
    assert len(free) == 18
    p = pv.copy()
    ref = O.nll(nodes, olist, p, c3_events)
    got, g = eng.nll_grad(p)
    assert got == pytest.approx(ref, rel=NLL_RTOL[prec])
    fd = O.fd_grad(nodes, olist, p, c3_events, free, h=1e-5)
    n = c3_events.shape[1]
    np.testing.assert_allclose(g, fd, rtol=2e-4 if prec == "mixed" else 1e-6, atol=2e-3 * math.sqrt(n))


@pytest.mark.parametrize("bins", [300, 1500])
def test_tensor_core_gram_matches_cuda_core_gram(c3_events, bins, monkeypatch):
    """The mixed engine's integrals from the tcgen05 Gram kernel (split-TF32 products, FP32 accumulation
    in tensor memory for 256 points per slice, FP64 beyond) against the CUDA-core kernel (FP32 products,
    FP64 per-CTA sums): within 2e-6 of the largest diagonal entry; the matrix is exactly Hermitian."""
    pdf, _, _ = W.c3_model(bins)
    out = {}
    for mode in ("tc", "cuda"):
        if mode == "cuda":
            monkeypatch.setenv("GF_GRAM", "cuda")
        else:
            monkeypatch.delenv("GF_GRAM", raising=False)
        eng, *_ = engine(pdf, c3_events, "mixed")
        out[mode] = eng.amp3_integrals(0, 8)
    scale = np.abs(np.diag(out["cuda"])).max()
    assert np.abs(out["tc"] - out["cuda"]).max() / scale < 2e-6
    np.testing.assert_array_equal(out["tc"], out["tc"].conj().T)


def test_gram_stage_wait_that_runs_out_is_reported_and_recovered(c3_events, monkeypatch):
    """A per-stage mbarrier wait of the tensor-core Gram kernel that runs out ends the integral rebuild with
    GF_ERR_CUDA and leaves the engine usable.  The wait is made to run out without any fault: the test hook
    GF_GRAM_TEST_STALL_STAGE=0 makes stage 0's wait also wait for a barrier on which nothing ever arrives, under
    a 1 ms limit, while the stage's MMAs complete normally.  The kernel then waits, with its fixed 2 s limit, for
    its last committed MMAs before it frees its tensor memory.  Without the hook and at the default limit, the
    next evaluation's integrals (within 2e-5 of the largest diagonal entry) and NLL (1e-6 relative) match the
    oracle."""
    pdf, _, _ = W.c3_model(300)
    nodes, olist, params, mask, pv = tree(pdf)
    eng = gf.Engine("mixed")
    eng.set_tree(nodes, olist, len(params), mask)
    eng.upload(c3_events)
    monkeypatch.setenv("GF_GRAM_TEST_STALL_STAGE", "0")
    eng.set_gram_wait_limit(1_000_000)
    for _ in range(2):
        with pytest.raises(A.EngineError) as ei:
            eng.nll(pv)
        assert ei.value.code == A.GF_ERR_CUDA
    monkeypatch.delenv("GF_GRAM_TEST_STALL_STAGE")
    eng.set_gram_wait_limit(0)
    nll = eng.nll(pv)
    assert nll == pytest.approx(O.nll(nodes, olist, pv, c3_events), rel=NLL_RTOL["mixed"])
    got = eng.amp3_integrals(0, 8)
    ref = O.amp3_integrals(nodes, olist, pv, 0, 8)
    assert np.abs(got - ref).max() / np.abs(np.diag(ref)).max() < AMP_RTOL["mixed"]
