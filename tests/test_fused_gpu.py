"""The one-launch evaluation (one toy): convolution tables, numeric grids and the event pass of an FCN in
one cooperative launch with a bounded grid barrier, against the FP64 oracle and against the three-launch
chain of the same engine, in both event-pass forms (per-k tabulated terms, per-event arithmetic) and with
the events bulk-copied to shared memory or read from global memory; and the barrier's bounded wait made
to run out on purpose (a limit of 1 ns, which the waiting CTAs exceed while the table CTAs still work),
after which the same engine must return the oracle's values again.

Tolerances as in the other parity tests: NLL 1e-6 relative (mixed) / 1e-10 (FP64); gradient against the
oracle's central differences within 2e-4 relative + 2e-3 sqrt(n).
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


def c2_engine(n, seed, prec, monkeypatch, fused="1", tab="1", stage="1"):
    wl = W.make_c2(n, seed=seed)
    nodes, params, obs = wl.pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    mask = [0 if v.fixed else 1 for v in params]
    pv = np.array([v.value for v in params])
    monkeypatch.setenv("GF_FUSED", fused)
    monkeypatch.setenv("GF_EVT_TAB", tab)
    monkeypatch.setenv("GF_STAGE", stage)
    eng = gf.Engine(prec)
    eng.set_tree(nodes, olist, len(params), mask)
    eng.upload(wl.data.to_numpy())
    return eng, wl, nodes, olist, params, mask, pv


@pytest.mark.parametrize("form", [("1", "1"), ("0", "1"), ("1", "0")], ids=["tab-staged", "perevent-staged",
                                                                        "tab-global"])
@pytest.mark.parametrize("prec", ["mixed", "fp64"])
@pytest.mark.parametrize("n", [5_000, 2_000_000])
def test_one_launch_matches_oracle_and_three_launches(n, prec, form, monkeypatch):
    tab, stage = form
    eng, wl, nodes, olist, params, mask, pv = c2_engine(n, 31, prec, monkeypatch, "1", tab, stage)
    eng3 = c2_engine(n, 31, prec, monkeypatch, "0")[0]
    data = wl.data.to_numpy()
    names = [v.name for v in params]
    free = [i for i, m in enumerate(mask) if m]
    for shift in (0.0, 0.04, -0.03):
        p = pv.copy()
        p[names.index("alpha")] += shift
        p[names.index("mu")] += shift / 3
        got, g = eng.nll_grad(p)
        assert eng.launches_per_eval(True) == 1
        ref = O.nll(nodes, olist, p, data)
        assert got == pytest.approx(ref, rel=NLL_RTOL[prec]), (shift, got, ref)
        assert eng.nll(p) == pytest.approx(ref, rel=NLL_RTOL[prec])
        got3, g3 = eng3.nll_grad(p)
        assert eng3.launches_per_eval(True) > 1
        assert got == pytest.approx(got3, rel=NLL_RTOL[prec])
        np.testing.assert_allclose(g, g3, rtol=1e-5, atol=1e-4 * math.sqrt(n))
        if n <= 5_000:
            fd = O.fd_grad(nodes, olist, p, data, free, h=1e-6)
            np.testing.assert_allclose(g, fd, rtol=2e-4, atol=2e-3 * math.sqrt(n))
    eng.close()
    eng3.close()


def test_invalid_normalisation_in_one_launch(monkeypatch):
    eng, wl, nodes, olist, params, mask, pv = c2_engine(3000, 33, "mixed", monkeypatch)
    p = pv.copy()
    p[[v.name for v in params].index("sigma")] = float("nan")
    with pytest.raises(A.EngineError) as ei:
        eng.nll_grad(p)
    assert ei.value.code == A.GF_ERR_NAN_NORM
    assert eng.nll_grad(pv)[0] == pytest.approx(O.nll(nodes, olist, pv, wl.data.to_numpy()), rel=1e-6)
    eng.close()


def test_barrier_wait_that_runs_out_is_reported_and_recovered(monkeypatch):
    eng, wl, nodes, olist, params, mask, pv = c2_engine(200_000, 32, "mixed", monkeypatch)
    data = wl.data.to_numpy()
    ref = O.nll(nodes, olist, pv, data)
    assert eng.nll_grad(pv)[0] == pytest.approx(ref, rel=1e-6)
    for _ in range(2):
        eng.set_wait_limit(1)
        with pytest.raises(A.EngineError) as ei:
            eng.nll_grad(pv)
        assert ei.value.code == A.GF_ERR_TIMEOUT
        eng.set_wait_limit(0)
        got, g = eng.nll_grad(pv)
        assert got == pytest.approx(ref, rel=1e-6)
        assert eng.nll(pv) == pytest.approx(ref, rel=1e-6)
    eng.close()


def test_tabulated_terms_in_pairs_track_the_oracle(monkeypatch):
    """Mixed precision, tabulated event pass: every bin's event function and -log P are FP32 pairs, so that a
    bin's rounding is not repeated by each of its events.  At 2e6 events the NLL then follows the oracle,
    evaluated at the FP32-rounded parameters the kernels see, up to a smooth offset (the single-precision bin
    centres and exponentials of the table inputs: below 1e-8 relative over a scan of alpha and mu), and its
    changes over steps of 2e-5 in alpha (0.02 sigma) match the oracle's within 1e-3 absolute.  With a
    single-precision term per bin the NLL jumped by 0.02-0.04 between such neighbouring points."""
    eng, wl, nodes, olist, params, mask, pv = c2_engine(2_000_000, 34, "mixed", monkeypatch)
    data = wl.data.to_numpy()
    names = [v.name for v in params]
    for shift in np.linspace(-0.02, 0.02, 5):
        p = pv.copy()
        p[names.index("alpha")] += shift
        p[names.index("mu")] -= shift / 2
        p32 = p.astype(np.float32).astype(np.float64)
        assert eng.nll(p) == pytest.approx(O.nll(nodes, olist, p32, data), rel=1e-8), shift
    prev = None
    for j in range(6):
        p = pv.copy()
        p[names.index("alpha")] += 2e-5 * j
        p32 = p.astype(np.float32).astype(np.float64)
        cur = (eng.nll(p), O.nll(nodes, olist, p32, data))
        if prev is not None:
            assert abs((cur[0] - prev[0]) - (cur[1] - prev[1])) < 1e-3, (j, cur, prev)
        prev = cur
    eng.close()


@pytest.mark.parametrize("seed", [3, 5, 6])
def test_mixed_fit_converges_as_the_fp64_fit(seed, monkeypatch):
    """MIGRAD with the analytic gradient on the 2e6-event composite model: the mixed-precision fit takes at
    most two more FCN calls than the FP64 fit and reaches its minimum within 1e-9 relative and 0.01 sigma
    (datasets on which single-precision per-bin terms made the mixed fit take 300-700 calls)."""
    monkeypatch.setenv("GF_FUSED", "1")
    wl = W.make_c2(2_000_000, seed=seed)
    nodes, params, obs = wl.pdf._flatten()
    free = [i for i, v in enumerate(params) if not v.fixed]
    out = {}
    for prec in ("mixed", "fp64"):
        wl.reset()
        fm = gf.FitManager(wl.pdf, precision=prec, gradient="analytic", tolerance=0.01)
        fm.verbosity = 0
        r = fm.fit()
        assert r.valid
        out[prec] = (r.nfcn, r.fmin, [params[i].value for i in free], [params[i].error for i in free])
    (nm, fm_, vm, _), (nf, ff, vf, ef) = out["mixed"], out["fp64"]
    assert nm <= nf + 2, (nm, nf)
    assert fm_ == pytest.approx(ff, rel=1e-9)
    assert max(abs(a - b) / e for a, b, e in zip(vm, vf, ef)) < 0.01


def test_sorted_events_match_upload_order_and_survive_reuploads(monkeypatch):
    """The tabulated path's events sorted by bin offset (histogram and run offsets built by the upload's
    conversion kernel, then the fill) against the same engine reading them in upload order, at sizes that leave
    padding slots, and across uploads of other sizes into the same engine (the histogram scratch is reused)."""
    eng = c2_engine(20_001, 41, "mixed", monkeypatch)[0]
    monkeypatch.setenv("GF_KSORT", "0")
    eng_u = c2_engine(20_001, 41, "mixed", monkeypatch)[0]
    monkeypatch.delenv("GF_KSORT")
    for n, seed in ((20_001, 41), (1_000_003, 42), (7_777, 43)):
        wl = W.make_c2(n, seed=seed)
        nodes, params, obs = wl.pdf._flatten()
        olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
        pv = np.array([v.value for v in params])
        data = wl.data.to_numpy()
        eng.upload(data)
        eng_u.upload(data)
        for shift in (0.0, 0.05):
            p = pv.copy()
            p[[v.name for v in params].index("alpha")] += shift
            got, g = eng.nll_grad(p)
            got_u, g_u = eng_u.nll_grad(p)
            # the counted sums are exact products of a bin's terms; the per-event loop adds 8 events' FP32 terms
            # pairwise first (a rounding of 2^-24 of the group sum each), about 1e-9 relative over the data set
            assert got == pytest.approx(got_u, rel=1e-8), (n, shift)
            np.testing.assert_allclose(g, g_u, rtol=1e-6, atol=1e-5 * math.sqrt(n))
            assert got == pytest.approx(O.nll(nodes, olist, p, data), rel=1e-6), (n, shift)
    eng.close()
    eng_u.close()


def test_rows_read_as_they_arrive_equal_rows_read_after_the_launch(monkeypatch):
    """The host adds the one-launch rows while the launch is still ending (each word checked against the unset
    mark); with GF_WAIT_SYNC=1 it synchronises the stream first. Both read the same rows in the same order, so
    the results are bit-identical, FCN after FCN (a fixed event chunk, so that both engines cut the events the
    same way)."""
    monkeypatch.setenv("GF_CHUNK", "2048")
    eng, wl, nodes, olist, params, mask, pv = c2_engine(300_001, 51, "mixed", monkeypatch)
    monkeypatch.setenv("GF_WAIT_SYNC", "1")
    eng_s = c2_engine(300_001, 51, "mixed", monkeypatch)[0]
    monkeypatch.delenv("GF_WAIT_SYNC")
    names = [v.name for v in params]
    for it in range(40):
        p = pv.copy()
        p[names.index("alpha")] += 0.002 * (it % 7)
        p[names.index("sigma")] += 0.001 * (it % 5)
        got, g = eng.nll_grad(p)
        got_s, g_s = eng_s.nll_grad(p)
        assert got == got_s, it
        np.testing.assert_array_equal(g, g_s)
        assert eng.nll(p) == eng_s.nll(p)
    assert eng.last_timing()[0] > 0
    eng.close()
    eng_s.close()
