"""The launch-shape autotuner (gf_tune_shapes): it picks a shape from its candidate list, the shape is in use
afterwards, and the results do not depend on it.

* Batches of the composite model: table k-tiles from {1, 2, 4, 8}.  The NLLs and gradients are unchanged
  (1e-12 relative in FP64; each table entry is summed the same way whichever CTA computes it).
* A ProdPdf whose factors share an observable (a numeric grid not folded into a table): grid bins per CTA
  from {128 ... 2048}; NLL and gradient within 1e-10 (FP64; the grid sum's partials regroup).
* Amp3Body (mixed precision, tensor-core Gram): slice width of at least 16 real columns; integrals within
  2e-5 of the largest entry of the untuned ones.
* A second engine with the same tree, toys and events takes the remembered shapes.
"""
import numpy as np
import pytest

import goofit_gb300 as gf
from combine_trees import prod_overlap
from goofit_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def tree(pdf):
    nodes, params, obs = pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    nd = pdf._nondiff_all()
    mask = [0 if (v.fixed or id(v) in nd) else 1 for v in params]
    return nodes, olist, params, mask, np.array([v.value for v in params])


def batch_engine(prec):
    study = W.make_c4(n_toys=32, seed=9)
    nodes, olist, params, mask, pv = tree(study.pdf)
    eng = gf.Engine(prec)
    eng.set_tree(nodes, olist, len(params), mask)
    eng.set_num_toys(32)
    for t, d in enumerate(study.datas):
        eng.upload(d, toy=t)
    return eng, np.tile(pv, (32, 1))


def test_table_k_tiles_are_tuned_without_changing_results():
    eng, P = batch_engine("fp64")
    f0, g0 = eng.nll_batch(P, grad=True)
    sh = eng.tune_shapes()
    assert sh["conv_kp"] in (1, 2, 4, 8)
    f1, g1 = eng.nll_batch(P, grad=True)
    np.testing.assert_allclose(f1, f0, rtol=1e-12)
    np.testing.assert_allclose(g1, g0, rtol=1e-12, atol=1e-9)
    # the same tree, toys and events: the remembered shapes, without timing again
    eng2, _ = batch_engine("fp64")
    eng2.nll_batch(P, grad=True)
    assert eng2.tune_shapes()["conv_kp"] == sh["conv_kp"]
    eng.close()
    eng2.close()


def test_grid_bins_per_cta_are_tuned_without_changing_results():
    pdf, cols = prod_overlap()
    nodes, olist, params, mask, pv = tree(pdf)
    eng = gf.Engine("fp64")
    eng.set_tree(nodes, olist, len(params), mask)
    eng.upload(cols)
    f0, g0 = eng.nll_grad(pv)
    sh = eng.tune_shapes()
    assert sh["grid_bins_per_cta"] in (128, 256, 512, 1024, 2048)
    f1, g1 = eng.nll_grad(pv)
    assert f1 == pytest.approx(f0, rel=1e-10)
    np.testing.assert_allclose(g1, g0, rtol=1e-8, atol=1e-8)
    eng.close()


def test_gram_slice_width_is_tuned_without_changing_integrals():
    pdf = W.c3_model(300)[0]
    cols = W.c3_generate(pdf, 20_000, seed=31, batch=1_000_000)
    nodes, olist, params, mask, pv = tree(pdf)
    eng = gf.Engine("mixed")
    eng.set_tree(nodes, olist, len(params), mask)
    eng.upload(cols)
    eng.set_params(pv)
    I0 = eng.amp3_integrals(0, 8)
    f0 = eng.nll(pv)
    sh = eng.tune_shapes()
    assert sh["gram_slice_width"] in (16, 32, 64)
    I1 = eng.amp3_integrals(0, 8)
    assert np.abs(I1 - I0).max() <= 2e-5 * np.abs(np.diag(I0)).max()
    assert eng.nll(pv) == pytest.approx(f0, rel=1e-6)
    eng.close()
