"""Trees and seeded events of the combination-PDF tests (tests/test_combine_gpu.py on the GPU against the
oracle, tests/test_reference_build.py on the CPU against the reference's own code)."""
import numpy as np

import goofit_gb300 as gf


def prod_separate():
    x = gf.Observable("x", -5.0, 5.0)
    y = gf.Observable("y", 0.0, 10.0)
    g = gf.GaussianPdf("gx", x, gf.Variable("mx", 0.2, 0.01, -1, 1), gf.Variable("sx", 1.1, 0.01, 0.1, 3))
    e = gf.ExpPdf("ey", y, gf.Variable("ay", -0.4, 0.01, -2, -0.01))
    rng = np.random.default_rng(41)
    n = 100_000
    xs = np.clip(rng.normal(0.2, 1.1, n), -4.99, 4.99)
    ys = -np.log(1 - rng.random(n) * (1 - np.exp(-0.4 * 10))) / 0.4
    return gf.ProdPdf("prod", [g, e]), np.vstack([xs, ys])


def prod_overlap():
    x = gf.Observable("x", -5.0, 5.0)
    x.setNumBins(2000)
    g = gf.GaussianPdf("gx", x, gf.Variable("mx", 0.2, 0.01, -1, 1), gf.Variable("sx", 1.4, 0.01, 0.1, 3))
    e = gf.ExpPdf("ex", x, gf.Variable("ax", -0.15, 0.01, -2, 2))
    rng = np.random.default_rng(42)
    xs = rng.uniform(-4.99, 4.99, 50_000)
    return gf.ProdPdf("prod", [g, e]), xs.reshape(1, -1)


def extended_add():
    x = gf.Observable("x", 0.0, 10.0)
    e = gf.ExpPdf("e", x, gf.Variable("a", -0.5, 0.01, -3, -0.01))
    g = gf.GaussianPdf("g", x, gf.Variable("m", 4.0, 0.01, 1, 8), gf.Variable("s", 0.7, 0.01, 0.1, 3))
    n1, n2 = gf.Variable("n_e", 30_000.0, 10, 0, 1e6), gf.Variable("n_g", 20_000.0, 10, 0, 1e6)
    rng = np.random.default_rng(43)
    xe = -np.log(1 - rng.random(30_000) * (1 - np.exp(-5))) / 0.5
    xg = np.clip(rng.normal(4.0, 0.7, 20_000), 0.01, 9.99)
    return gf.AddPdf("ext", [n1, n2], [e, g]), np.concatenate([xe, xg]).reshape(1, -1), (n1, n2)
