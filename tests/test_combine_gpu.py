"""GPU parity of the combination PDFs that the benchmark trees do not exercise.

* Unbinned ProdPdf:
  * Separate observables: each factor normalised analytically (ProdPdf::normalize,
    src/PDFs/combine/ProdPdf.cu:75-99).
  * Shared observables: the product normalised on a numeric grid (the overlap rule, ProdPdf.cu:28-68).
* Extended AddPdf: the yields' term N_tot - n log N_tot added to the NLL (AddPdf::calculateNLL,
  src/PDFs/combine/AddPdf.cu:187-204).

Each NLL and analytic gradient is compared with the FP64 oracle on the same events. Tolerances:
* NLL: 1e-6 relative (mixed), 1e-10 (FP64).
* Gradient: within 2e-4 relative + 2e-3 sqrt(n) of the oracle's central differences.

An extended fit's yields must add up to the event count.
"""
import math

import numpy as np
import pytest

import goofit_gb300 as gf
from combine_trees import extended_add, prod_overlap, prod_separate
from oracle import oracle as O

pytestmark = pytest.mark.gpu

NLL_RTOL = {"mixed": 1e-6, "fp64": 1e-10}


def engine(pdf, cols, prec):
    nodes, params, obs = pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    mask = [0 if v.fixed else 1 for v in params]
    eng = gf.Engine(prec)
    eng.set_tree(nodes, olist, len(params), mask)
    eng.upload(cols)
    pv = np.array([v.value for v in params])
    return eng, nodes, olist, params, mask, pv


def check(pdf, cols, prec, shifts):
    eng, nodes, olist, params, mask, pv = engine(pdf, cols, prec)
    free = [i for i, m in enumerate(mask) if m]
    n = cols.shape[1]
    for s in shifts:
        p = pv.copy()
        p[free] *= 1 + s
        got, g = eng.nll_grad(p)
        ref = O.nll(nodes, olist, p, cols)
        assert got == pytest.approx(ref, rel=NLL_RTOL[prec]), (s, got, ref)
        assert eng.nll(p) == pytest.approx(ref, rel=NLL_RTOL[prec])
        fd = O.fd_grad(nodes, olist, p, cols, free, h=1e-6)
        np.testing.assert_allclose(g, fd, rtol=2e-4, atol=2e-3 * math.sqrt(n))
    eng.close()


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_unbinned_prodpdf_separate_observables(prec):
    pdf, cols = prod_separate()
    check(pdf, cols, prec, (0.0, 0.03, -0.02))


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_unbinned_prodpdf_shared_observable_numeric_norm(prec):
    pdf, cols = prod_overlap()
    check(pdf, cols, prec, (0.0, 0.03))


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_extended_addpdf(prec):
    pdf, cols, _ = extended_add()
    check(pdf, cols, prec, (0.0, 0.02, -0.04))


def test_extended_fit_yields_add_up_to_the_events():
    pdf, cols, (n1, n2) = extended_add()
    ds = gf.UnbinnedDataSet(pdf.getObservables())
    ds.from_numpy(cols)
    pdf.setData(ds)
    fm = gf.FitManager(pdf, precision="mixed", tolerance=0.01)
    fm.verbosity = 0
    r = fm.fit()
    assert r.valid
    # at the extended likelihood's minimum the yields sum to the number of events
    assert n1.value + n2.value == pytest.approx(cols.shape[1], rel=1e-4)
