"""GenerateSig of the amplitude PDFs (Amp3Body::GenerateSig, src/PDFs/physics/Amp3Body.cu:430-547;
Amp4Body::GenerateSig, src/PDFs/physics/Amp4Body.cu:560-677): shapes and kinematics of the returned
events, weights = the amplitude density from the FP64 engine, and accepted events distributed like an
independent accept-reject sample of the same density (means within 5 standard errors)."""
import numpy as np
import pytest

from goofit_gb300 import phasespace
from goofit_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _m2(a, b):
    q = a + b
    return q[:, 3] ** 2 - np.sum(q[:, :3] ** 2, axis=1)


def _same_mean(x, y):
    se = np.sqrt(x.var() / len(x) + y.var() / len(y))
    return abs(x.mean() - y.mean()) < 5 * se


def test_amp3body_generate_sig():
    pdf = W.c3_model(300)[0]
    parts, var, w, f = pdf.GenerateSig(200_000, seed=7)
    assert len(parts) == 3 and all(p.shape == (200_000, 4) for p in parts)
    m12, m23, m13 = var
    np.testing.assert_allclose(m12, _m2(parts[0], parts[1]), rtol=1e-12)
    np.testing.assert_allclose(m23, _m2(parts[1], parts[2]), rtol=1e-12)
    np.testing.assert_allclose(m13, _m2(parts[0], parts[2]), rtol=1e-12)
    # momentum balance in the parent frame and the Dalitz-plot identity m12 + m13 + m23 = M^2 + sum m_i^2
    tot = parts[0] + parts[1] + parts[2]
    np.testing.assert_allclose(tot[:, :3], 0, atol=1e-12)
    d = pdf.getDecayInfo()
    np.testing.assert_allclose(m12 + m13 + m23, d.motherMass ** 2 + d.daug1Mass ** 2 + d.daug2Mass ** 2 +
                               d.daug3Mass ** 2, rtol=1e-10)
    assert np.all(w >= 0) and 0.01 < f.mean() < 0.9
    ref = W.c3_generate(pdf, int(f.sum()), seed=8, batch=500_000)
    assert _same_mean(m12[f], ref[0]) and _same_mean(m13[f], ref[1])
    # the same seed gives the same events
    a = pdf.GenerateSig(5000, seed=11)
    b = pdf.GenerateSig(5000, seed=11)
    np.testing.assert_array_equal(a[1][0], b[1][0])
    np.testing.assert_array_equal(a[3], b[3])


def test_amp4body_generate_sig():
    pdf = W.c5_model(20_000)[0]
    parts, var, w, f = pdf.GenerateSig(100_000, seed=3)
    assert len(parts) == 4 and len(var) == 5 and w.shape == (100_000,) and f.dtype == bool
    v5 = phasespace.dim5(np.stack(parts, axis=1))
    for a, b in zip(var, v5):
        np.testing.assert_array_equal(a, b)
    assert np.all(w >= 0) and 0.005 < f.mean() < 0.9
    ref = W.c5_generate(pdf, int(f.sum()), seed=4, batch=400_000)
    for i in (0, 1, 2):
        assert _same_mean(var[i][f], ref[i]), i
