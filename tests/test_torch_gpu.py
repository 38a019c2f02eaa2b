"""The engine NLL as a torch.autograd.Function: forward value and backward gradient against the oracle, and
a torch optimiser reaching the MIGRAD minimum."""
import numpy as np
import pytest

import goofit_gb300 as gf
from goofit_gb300 import workloads as W
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_forward_and_backward_match_oracle():
    from goofit_gb300.torch_nll import free_parameters, nll
    wl = W.make_c2(20_000, seed=7)
    pdf = wl.pdf
    x = free_parameters(pdf).requires_grad_(True)
    v = nll(pdf, x, precision="fp64")
    v.backward()
    nodes, params, obs = pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    pv = np.array([p.value for p in params])
    free = [i for i, p in enumerate(params) if not p.fixed]
    assert float(v) == pytest.approx(O.nll(nodes, olist, pv, wl.data.to_numpy()), rel=1e-10)
    fd = O.fd_grad(nodes, olist, pv, wl.data.to_numpy(), free, h=1e-6)
    np.testing.assert_allclose(x.grad.numpy(), fd, rtol=1e-5, atol=1e-2)


def test_torch_optimiser_reaches_the_migrad_minimum():
    from goofit_gb300.torch_nll import free_parameters, nll
    wl = W.make_c1(50_000, seed=3)
    fm = gf.FitManager(wl.pdf, precision="fp64", tolerance=0.01)
    fm.verbosity = 0
    r = fm.fit()
    best = wl.variables["alpha"].value
    sigma = wl.variables["alpha"].error
    wl.reset()
    x = free_parameters(wl.pdf).requires_grad_(True)
    opt = torch.optim.LBFGS([x], lr=1.0, max_iter=50, line_search_fn="strong_wolfe")

    def closure():
        opt.zero_grad()
        v = nll(wl.pdf, x, precision="fp64")
        v.backward()
        return v

    opt.step(closure)
    assert abs(float(x[0]) - best) < 0.01 * sigma
