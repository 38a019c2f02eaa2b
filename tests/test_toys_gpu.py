"""Batched toy fits (C4 shape): one engine holds many datasets of uneven size, every MIGRAD round is one
batched graph launch, and each toy's result must equal its single fit and, for a sample, the FP64 oracle
fit within 0.01 sigma."""
import numpy as np
import pytest

import goofit_gb300 as gf
from goofit_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _setup(study, prec):
    nodes, params, obs = study.pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    mask = [0 if v.fixed else 1 for v in params]
    eng = gf.Engine(prec)
    eng.set_tree(nodes, olist, len(params), mask)
    eng.set_num_toys(len(study.datas))
    for t, d in enumerate(study.datas):
        eng.upload(d, toy=t)
    return eng, nodes, olist, params


def _limits(params):
    err = np.array([v.error for v in params])
    lo = np.array([v.lowerlimit for v in params])
    hi = np.array([v.upperlimit for v in params])
    fixed = np.array([1 if v.fixed else 0 for v in params], np.int32)
    limited = np.array([0 if v.fixed else 1 for v in params], np.int32)
    return err, lo, hi, limited, fixed


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_batched_fits_match_single_and_oracle(prec):
    study = W.make_c4(n_toys=12, mean_events=6000, lo=5000, hi=60000, seed=7)
    eng, nodes, olist, params = _setup(study, prec)
    x0 = np.array([study.start.get(v.name, v.value) for v in params])
    err, lo, hi, limited, fixed = _limits(params)
    X0 = np.tile(x0, (len(study.datas), 1))
    res = eng.fit_batch(X0, err, lo, hi, limited, fixed, tolerance=0.001)
    assert all(r.valid for r in res)
    free = [i for i, f in enumerate(fixed) if not f]
    for t in (0, 5, 11):
        single = eng.fit(x0, err, lo, hi, limited, fixed, tolerance=0.001, toy=t)
        for i in free:
            assert abs(res[t].values[i] - single.values[i]) < 0.01 * single.errors[i]
    for t in (0, 7):
        m = gf.Minimizer(x0, err, lo, hi, limited, fixed, tolerance=0.001)
        ro = m.minimize(lambda p: O.nll(nodes, olist, p, study.datas[t]))
        assert ro.valid
        for i in free:
            assert abs(res[t].values[i] - ro.values[i]) < 0.01 * ro.errors[i], (t, params[i].name)
            assert res[t].errors[i] == pytest.approx(ro.errors[i], rel=0.02)


def test_batched_nll_equals_per_toy_oracle():
    study = W.make_c4(n_toys=64, mean_events=5000, seed=3)
    eng, nodes, olist, params = _setup(study, "mixed")
    pv = np.array([v.value for v in params])
    P = np.tile(pv, (64, 1))
    nll = eng.nll_batch(P)
    for t in range(0, 64, 9):
        assert nll[t] == pytest.approx(O.nll(nodes, olist, pv, study.datas[t]), rel=1e-6)
