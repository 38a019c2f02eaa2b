"""MINOS errors of FitManager (FitManagerMinuit2 with MnMinos, src/goofit/FitManagerMinuit2.cpp:58-80).

For the one-parameter exponential fit the MINOS points are where the FP64 oracle's NLL rises by
up = 0.5 above the minimum (within 0.01); for the composite model each MINOS point's profile (MIGRAD over
the other parameters with the parameter fixed) rises by 0.5 within 0.01, and the errors are close to the
parabolic ones (large samples: within 10%)."""
import numpy as np
import pytest

import goofit_gb300 as gf
from goofit_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _tree(pdf):
    nodes, params, obs = pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    return nodes, olist, params


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_minos_exponential_matches_the_oracle_profile(prec):
    wl = W.make_c1(100_000)
    fm = gf.FitManager(wl.pdf, precision=prec, tolerance=0.01)
    fm.verbosity = 0
    fm.setMinos()
    r = fm.fit()
    assert r.valid
    alpha = wl.variables["alpha"]
    lo_err, up_err = alpha.minos_error
    assert lo_err < 0 < up_err
    nodes, olist, params = _tree(wl.pdf)
    x = wl.data.to_numpy()
    best = np.array([v.value for v in params])
    f0 = O.nll(nodes, olist, best, x)
    ia = [v.name for v in params].index("alpha")
    for d in (lo_err, up_err):
        p = best.copy()
        p[ia] += d
        assert abs(O.nll(nodes, olist, p, x) - f0 - 0.5) < 0.01, d
        assert abs(abs(d) - alpha.error) < 0.05 * alpha.error


def test_minos_composite_profile_rises_by_up():
    wl = W.make_c2(200_000)
    fm = gf.FitManager(wl.pdf, precision="fp64", tolerance=0.01)
    fm.verbosity = 0
    fm.setMinos()
    r = fm.fit()
    assert r.valid
    assert set(fm.minos_errors) == {k for k, v in wl.variables.items() if not v.fixed}
    nodes, olist, params = _tree(wl.pdf)
    names = [v.name for v in params]
    eng, _ = wl.pdf._engine_for(wl.pdf.data, "fp64")
    best = np.array([v.value for v in params])
    err = np.array([v.error for v in params])
    lo = np.array([v.lowerlimit for v in params])
    hi = np.array([v.upperlimit for v in params])
    fixed = np.array([1 if v.fixed else 0 for v in params], np.int32)
    limited = np.array([0 if (v.fixed or v.lowerlimit == v.upperlimit) else 1 for v in params], np.int32)
    for name, (dlo, dup) in fm.minos_errors.items():
        i = names.index(name)
        assert dlo < 0 < dup
        assert abs(-dlo - err[i]) < 0.1 * err[i] and abs(dup - err[i]) < 0.1 * err[i], name
        fx = fixed.copy()
        fx[i] = 1
        for d in (dlo, dup):
            x = best.copy()
            x[i] += d
            rr = eng.fit(x, err, lo, hi, limited, fx, tolerance=0.01)
            assert abs(rr.fmin - r.fmin - 0.5) < 0.01, (name, d)
