"""The FP64 restatement (oracle/oracle.cpp) against the reference's own likelihood code, compiled for the
CPU from the reference's sources (oracle/ref/Makefile, Thrust's OMP backend, project-written shims for the
reference's empty submodules): the same NLL, at 1e-12 relative, for the benchmark configurations' trees on
the same events and parameter points.

* C1 ExpPdf (analytic normalisation).
* C2 Add(Convolution(Exp, Gauss), flat Poly) on a 10,000-bin numeric normalisation, at the truth and at
  shifted alpha, mu and sigma (the convolution table values and its grid sum).
* ProdPdf of factors on separate observables (analytic norms) and on a shared one (numeric norm), and
  an extended AddPdf (the yields' term of AddPdf::calculateNLL).
* C3 Amp3Body with the eight relativistic Breit-Wigner resonances, at the coefficients of the workload and
  with every coefficient, mass and width shifted (cached waves and the 64 integrals rebuilt by the
  reference).
* C5 Amp4Body with the six decay chains on the same flat phase-space normalisation events (given to the
  reference as 4-vectors, to the restatement as its five variables), one parameter shifted at a time and
  all together.
* Dim5: the reference's own 4-vectors -> (m12, m34, cos12, cos34, phi) against the restatement's (1e-12),
  and on the reference's golden vectors (tests/simple/VectorsTest.cu) within the test's 1e-5.

Skipped where the reference sources are absent.  Each reference tree is built in a fresh process.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import combine_trees as CT
from goofit_gb300 import phasespace as PS
from goofit_gb300 import workloads as W
from oracle import oracle as O
from oracle import ref as R

pytestmark = pytest.mark.skipif(not R.available(), reason="reference sources not present")

RTOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _ref_built():
    R.build()


def tree(pdf):
    nodes, params, obs = pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    return nodes, olist, params


def test_c1_exp_matches_reference():
    wl = W.make_c1(100_000, seed=1)
    nodes, olist, params = tree(wl.pdf)
    x = wl.data.to_numpy()
    P = np.array([-0.3, -0.7, -1.1])
    ref = R.isolated("exp_nll", x[0], 0.0, 10.0, P)
    for a, r in zip(P, ref):
        assert O.nll(nodes, olist, [a], x) == pytest.approx(r, rel=RTOL)


def test_c2_composite_matches_reference():
    wl = W.make_c2(200_000, seed=2)
    nodes, olist, params = tree(wl.pdf)
    x = wl.data.to_numpy()
    names = [v.name for v in params]
    order = ["fsig", "alpha", "mu", "sigma", "c0"]
    pts = np.array([[0.7, -1 / 1.5, 0.0, 0.3, 1.0], [0.65, -0.6, 0.05, 0.35, 1.0], [0.72, -0.75, -0.08, 0.26, 1.0]])
    ref = R.isolated("c2_nll", x[0], -5.0, 10.0, 10_000, W.C2_CONV_RANGE, pts)
    for pt, r in zip(pts, ref):
        pv = np.array([pt[order.index(n)] for n in names])
        assert O.nll(nodes, olist, pv, x) == pytest.approx(r, rel=RTOL)
        assert O.nll(nodes, olist, pv, x, brute_force=True) == pytest.approx(r, rel=RTOL)


def _pv(pdf, values):
    return np.array([values[v.name] for v in pdf._flatten()[1]])


def test_prodpdf_and_extended_addpdf_match_reference():
    # separate observables
    pdf, cols = CT.prod_separate()
    nodes, olist, params = tree(pdf)
    pts = np.array([[0.2, 1.1, -0.4], [0.25, 1.0, -0.45]])
    ref = R.isolated("prod_nll", cols[0], cols[1], pts)
    for pt, r in zip(pts, ref):
        pv = _pv(pdf, dict(zip(["mx", "sx", "ay"], pt)))
        assert O.nll(nodes, olist, pv, cols) == pytest.approx(r, rel=RTOL)
    # shared observable: numeric normalisation of the product
    pdf, cols = CT.prod_overlap()
    nodes, olist, params = tree(pdf)
    pts = np.array([[0.2, 1.4, -0.15], [0.1, 1.3, -0.2]])
    ref = R.isolated("prod_overlap_nll", cols[0], 2000, pts)
    for pt, r in zip(pts, ref):
        pv = _pv(pdf, dict(zip(["mx", "sx", "ax"], pt)))
        assert O.nll(nodes, olist, pv, cols) == pytest.approx(r, rel=RTOL)
    # extended AddPdf
    pdf, cols, _ = CT.extended_add()
    nodes, olist, params = tree(pdf)
    pts = np.array([[-0.5, 4.0, 0.7, 30_000.0, 20_000.0], [-0.45, 4.1, 0.75, 31_000.0, 18_500.0]])
    ref = R.isolated("extadd_nll", cols[0], pts)
    for pt, r in zip(pts, ref):
        pv = _pv(pdf, dict(zip(["a", "m", "s", "n_e", "n_g"], pt)))
        assert O.nll(nodes, olist, pv, cols) == pytest.approx(r, rel=RTOL)


def _dalitz_points(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        a, b = rng.uniform(0, 3, 2)
        if O.in_dalitz(a, b, W.C3_M, W.C3_MK, W.C3_MPI, W.C3_MPI0):
            out.append((a, b))
    p = np.array(out).T
    return np.vstack([p, np.arange(n, dtype=np.float64)[None, :]])


@pytest.mark.parametrize("bins", [300, 1500])
def test_c3_amp3body_matches_reference(bins):
    pdf = W.c3_model(bins)[0]
    nodes, olist, params = tree(pdf)
    cols = _dalitz_points(2000, 5)
    names = [v.name for v in params]

    def vec(pv):
        d = dict(zip(names, pv))
        return np.concatenate([[d[f"{nm}_amp_real"], d[f"{nm}_amp_imag"], d[f"{nm}_mass"], d[f"{nm}_width"]]
                               for nm, *_ in W.C3_RESONANCES])

    pv = np.array([v.value for v in params])
    pv2 = pv.copy()
    shift = [i for i, n in enumerate(names) if n.endswith(("_amp_real", "_amp_imag", "_mass", "_width"))]
    pv2[shift] *= 1 + 0.03 * np.random.default_rng(6).standard_normal(len(shift))
    spin = [s for _, _, _, s, _ in W.C3_RESONANCES]
    cyc = [int(p) for *_, p in W.C3_RESONANCES]
    dec = [W.C3_M, W.C3_MK, W.C3_MPI, W.C3_MPI0, 1.5, 5.0]
    ref = R.isolated("amp3_nll", cols[0], cols[1], bins, dec, spin, cyc, np.stack([vec(pv), vec(pv2)]))
    for p, r in zip((pv, pv2), ref):
        assert O.nll(nodes, olist, p, cols) == pytest.approx(r, rel=RTOL)


C5_LS = ["rho_mass", "rho_width", "Kst_mass", "Kst_width", "K1_mass", "K1_width", "a1_mass", "a1_width", "f0_mass",
         "f0_width"]
C5_CHAINS = ["K*rho_S", "K*rho_P", "K*rho_D", "K1rho", "a1rho", "K*f0"]


@pytest.fixture(scope="module")
def c5():
    nn = 20_000
    pdf = W.c5_model(nn, norm_seed=55)[0]
    nodes, olist, params = tree(pdf)
    # the 4-vectors behind the Amp4Body's normalisation events (the same generator stream)
    p4 = PS.generate(W.C5_M, W.C5_MASSES, nn, np.random.Generator(np.random.PCG64(55)))
    assert np.array_equal(PS.dim5(p4), pdf.norm_events)
    ev = PS.dim5(PS.generate(W.C5_M, W.C5_MASSES, 3000, np.random.Generator(np.random.PCG64(99))))
    cols = np.vstack([ev, np.arange(3000, dtype=np.float64)[None, :]])
    return pdf, nodes, olist, params, p4[..., [3, 0, 1, 2]], cols


def test_c5_amp4body_matches_reference(c5):
    pdf, nodes, olist, params, p4, cols = c5
    names = [v.name for v in params]

    def vec(pv):
        d = dict(zip(names, pv))
        return np.array([d[k] for k in C5_LS] + sum([[d[f"{c}_re"], d[f"{c}_im"]] for c in C5_CHAINS], []))

    pv = np.array([v.value for v in params])
    pts = [pv]
    for k in ("rho_width", "K1_mass", "a1_width", "f0_mass", "K*rho_P_re", "a1rho_im"):
        p = pv.copy()
        p[names.index(k)] *= 1.03
        pts.append(p)
    # everything the harness takes at once (line shapes and coefficients; the efficiency stays constant)
    p = pv.copy()
    idx = [names.index(k) for k in C5_LS] + [names.index(f"{c}_{s}") for c in C5_CHAINS for s in ("re", "im")]
    p[idx] *= 1 + 0.02 * np.random.default_rng(4).standard_normal(len(idx))
    pts.append(p)
    O.set_amp4_norm_events(pdf.norm_events)
    # one reference tree per point: every point's caches and normalisation built from scratch
    for pt in pts:
        r = R.isolated("amp4_nll", cols[:5], [W.C5_M] + list(W.C5_MASSES), p4, vec(pt)[None, :])[0]
        assert O.nll(nodes, olist, pt, cols) == pytest.approx(r, rel=RTOL)


def test_dim5_matches_reference():
    p4 = PS.generate(W.C5_M, W.C5_MASSES, 2000, np.random.Generator(np.random.PCG64(7)))
    ref = R.isolated("dim5", p4[..., [3, 0, 1, 2]])
    np.testing.assert_allclose(PS.dim5(p4), ref, rtol=0, atol=1e-12)


def test_reference_dim5_on_its_golden_vectors():
    g = json.loads((Path(__file__).parent / "golden" / "dim5_vectors.json").read_text())
    ev = np.array(g["events"]).reshape(-1, 4, 4)  # (px, py, pz, E) per daughter
    ref = R.isolated("dim5", ev[..., [3, 0, 1, 2]]).T
    ans = np.array(g["answers"])
    # Catch2 Approx(...).epsilon(1e-5): relative to the larger magnitude
    assert np.all(np.abs(ref - ans) <= g["epsilon"] * np.maximum(np.abs(ref), np.abs(ans)))
