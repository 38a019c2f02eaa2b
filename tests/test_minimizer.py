"""The project MIGRAD (ask/tell C ABI) on analytic test functions."""
import math

import numpy as np
import pytest

import goofit_gb300 as gf


def test_quadratic_minimum_and_errors():
    # f = 0.5 (x-a)^T H (x-a); with up = 0.5 the covariance is H^-1
    H = np.array([[4.0, 1.0, 0.0], [1.0, 3.0, 0.5], [0.0, 0.5, 2.0]])
    a = np.array([1.0, -2.0, 0.5])
    f = lambda x: 0.5 * (x - a) @ H @ (x - a)
    g = lambda x: H @ (x - a)
    for use_grad in (False, True):
        m = gf.Minimizer([0.0, 0.0, 0.0], [1.0, 1.0, 1.0], use_grad=use_grad, tolerance=1e-4)
        r = m.minimize(f, g)
        assert r.valid
        # MIGRAD stops once EDM < 0.002 tol up: the distance to the minimum is <= sqrt(2 EDM) sigma
        sig = np.sqrt(np.diag(np.linalg.inv(H)))
        assert np.all(np.abs(r.values - a) <= 3 * np.sqrt(2 * 0.002 * 1e-4 * 0.5) * sig + 1e-9)
        np.testing.assert_allclose(m.covariance(), np.linalg.inv(H), rtol=1e-4, atol=1e-8)
        np.testing.assert_allclose(r.errors, np.sqrt(np.diag(np.linalg.inv(H))), rtol=1e-4)


def test_rosenbrock():
    f = lambda x: 100 * (x[1] - x[0] ** 2) ** 2 + (1 - x[0]) ** 2
    g = lambda x: np.array([-400 * x[0] * (x[1] - x[0] ** 2) - 2 * (1 - x[0]), 200 * (x[1] - x[0] ** 2)])
    for use_grad in (False, True):
        m = gf.Minimizer([-1.2, 1.0], [0.1, 0.1], use_grad=use_grad, tolerance=1e-3, maxfcn=5000)
        r = m.minimize(f, g)
        assert r.valid
        np.testing.assert_allclose(r.values, [1.0, 1.0], atol=2e-3)


def test_limits_and_fixed():
    f = lambda x: (x[0] - 3.0) ** 2 + (x[1] + 1.0) ** 2 + (x[2] - 5.0) ** 2
    m = gf.Minimizer([0.5, 0.0, 2.0], [0.1, 0.1, 0.1], lo=[0.0, -10, 0], hi=[2.0, 10, 0], limited=[1, 1, 0],
                     fixed=[0, 0, 1], tolerance=1e-3)
    r = m.minimize(f)
    # bounded at the upper limit, fixed parameter untouched
    assert r.values[0] == pytest.approx(2.0, abs=1e-3)
    assert r.values[1] == pytest.approx(-1.0, abs=2e-3)  # sqrt(2 edmval) sigma
    assert r.values[2] == 2.0


def test_lower_and_upper_single_limits():
    f = lambda x: (x[0] + 2.0) ** 2 + (x[1] - 4.0) ** 2
    m = gf.Minimizer([1.0, 0.0], [0.1, 0.1], lo=[0.0, 0.0], hi=[0.0, 1.0], limited=[2, 3], tolerance=1e-3)
    r = m.minimize(f)
    assert r.values[0] == pytest.approx(0.0, abs=1e-3)
    assert r.values[1] == pytest.approx(1.0, abs=1e-3)


def test_nan_values_are_backed_off():
    # a function that is undefined beyond x > 2 (NaN) still converges to its minimum at 1.5
    f = lambda x: float("nan") if x[0] > 2 else (x[0] - 1.5) ** 2
    m = gf.Minimizer([0.0], [3.0], tolerance=1e-3)
    r = m.minimize(f)
    assert r.values[0] == pytest.approx(1.5, abs=1e-4)


def test_call_limit_is_reported():
    f = lambda x: 100 * (x[1] - x[0] ** 2) ** 2 + (1 - x[0]) ** 2
    m = gf.Minimizer([-1.2, 1.0], [0.1, 0.1], maxfcn=20)
    r = m.minimize(f)
    assert r.call_limit and not r.valid
