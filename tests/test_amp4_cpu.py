"""4-body kinematics without a GPU: the Dim5 variables against the reference's known answers
(tests/simple/VectorsTest.cu:10-86, fixture made by tests/golden/make_dim5_vectors.py), get4Vecs as their
inverse, the flatness of the phase-space generator, and the Amp4Body tree checks."""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

import goofit_gb300 as gf
from goofit_gb300 import _abi as A
from goofit_gb300 import phasespace as PS
from goofit_gb300 import workloads as W
from oracle import oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden" / "dim5_vectors.json"


def test_dim5_matches_reference_known_answers():
    g = json.loads(GOLDEN.read_text())
    ev = np.array(g["events"]).reshape(10, 4, 4)
    got = PS.dim5(ev)
    ans = np.array(g["answers"]).T
    # Catch2 Approx(...).epsilon(1e-5): relative to the larger magnitude
    assert np.all(np.abs(got - ans) <= g["epsilon"] * np.maximum(np.abs(got), np.abs(ans)))


def test_get4vecs_inverts_dim5():
    masses = [W.C5_M] + W.C5_MASSES
    v = PS.norm_events(W.C5_M, W.C5_MASSES, 500, 3)
    for i in range(500):
        P = O.get4vecs(v[:, i], masses)
        assert np.abs(P.sum(axis=0)[:3]).max() < 1e-12
        assert P.sum(axis=0)[3] == pytest.approx(W.C5_M, abs=1e-12)
        back = PS.dim5(P[None])[:, 0]
        np.testing.assert_allclose(back, v[:, i], atol=1e-11)


def test_phase_space_angles_are_flat():
    v = PS.norm_events(W.C5_M, W.C5_MASSES, 200_000, 9)
    for k, (lo, hi) in zip((2, 3, 4), ((-1, 1), (-1, 1), (-np.pi, np.pi))):
        h, _ = np.histogram(v[k], bins=20, range=(lo, hi))
        expected = len(v[k]) / 20
        chi2 = np.sum((h - expected) ** 2 / expected)
        assert chi2 < 60, (k, chi2)  # 19 degrees of freedom


def _tree(pdf):
    nodes, params, obs = pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    nd = pdf._nondiff_all()
    mask = [0 if (v.fixed or id(v) in nd) else 1 for v in params]
    return nodes, olist, params, mask


@pytest.mark.parametrize("prec", [A.GF_MIXED, A.GF_FP64])
def test_amp4body_kernels_compile_for_sm103a(prec):
    pdf = W.c5_model(1000)[0]
    nodes, olist, params, mask = _tree(pdf)
    L = A.lib()
    nl = A.NodeList(nodes)
    obs = A.observables_array(olist)
    marr, mp = A.i32(mask)
    n = C.c_int64()
    assert L.gf_compile_tree(nl.arr, nl.n, obs, len(olist), len(params), mp, prec, C.byref(n)) == 0, \
        L.gf_last_error(None)


def test_amp4body_lineshape_parameters_get_derivative_columns():
    """Floated line-shape masses and widths have analytic derivatives (dual numbers through the line shapes,
    single precision in the mixed engine); the efficiency's parameters do not."""
    pdf, _, _, ls = W.c5_model(1000, float_lineshapes=True)
    nodes, olist, params, mask = _tree(pdf)
    assert sum(mask) == 20
    L = A.lib()
    nl = A.NodeList(nodes)
    obs = A.observables_array(olist)
    marr, mp = A.i32(mask)
    n = C.c_int64()
    assert L.gf_generated_source(nl.arr, nl.n, obs, len(olist), len(params), mp, A.GF_MIXED, None, 0, C.byref(n)) == 0
    buf = C.create_string_buffer(n.value + 1)
    L.gf_generated_source(nl.arr, nl.n, obs, len(olist), len(params), mp, A.GF_MIXED, buf, n.value + 1, C.byref(n))
    src = buf.value.decode()
    assert "gf_lineshape_t<GfDualF>" in src and "gf_ampn" in src
    full = [0 if v.fixed else 1 for v in params]
    for i, v in enumerate(params):
        if v.name == "constantOne":
            full[i] = 1
    marr, mp = A.i32(full)
    rc = L.gf_generated_source(nl.arr, nl.n, obs, len(olist), len(params), mp, A.GF_MIXED, None, 0, C.byref(n))
    assert rc == A.GF_ERR_BAD_TREE and b"efficiency" in L.gf_last_error(None)


def _source(nodes, olist, params, mask, prec):
    L = A.lib()
    nl = A.NodeList(nodes)
    obs = A.observables_array(olist)
    marr, mp = A.i32(mask)
    n = C.c_int64()
    assert L.gf_generated_source(nl.arr, nl.n, obs, len(olist), len(params), mp, prec, None, 0, C.byref(n)) == 0
    buf = C.create_string_buffer(n.value + 1)
    L.gf_generated_source(nl.arr, nl.n, obs, len(olist), len(params), mp, prec, buf, n.value + 1, C.byref(n))
    return buf.value.decode()


def c3_floated(bins):
    """The C3 Amp3Body with the masses and widths of its first two resonances floated."""
    pdf = W.c3_model(bins)[0]
    names = [nm for nm, *_ in W.C3_RESONANCES[:2]]
    for v in pdf.getParameters():
        if any(v.name in (f"{nm}_mass", f"{nm}_width") for nm in names):
            v.fixed = False
            v.error = 0.01 * v.value
            v.lowerlimit, v.upperlimit = 0.5 * v.value, 1.5 * v.value
    return pdf


@pytest.mark.parametrize("prec", [A.GF_MIXED, A.GF_FP64])
@pytest.mark.parametrize("model", ["c5", "c3"])
def test_recompute_mode_kernels_compile_for_sm103a(prec, model):
    """With floated line-shape (C5) or resonance (C3) parameters the tree also gets the recompute-mode kernels:
    a gradient event kernel that calls the amplitude functions per event and an integral kernel that
    evaluates them per normalisation point; both compile for sm_103a."""
    pdf = W.c5_model(1000, float_lineshapes=True)[0] if model == "c5" else c3_floated(300)
    nodes, olist, params, mask = _tree(pdf)
    src = _source(nodes, olist, params, mask, prec)
    assert "gf_evt_gr(" in src and "gf_gramr(" in src
    body = src[src.index("gf_evt_gr("):]
    assert "gf_ampv_0(xd0_0[ij]" in body[:body.index("extern \"C\"") if "extern \"C\"" in body else len(body)]
    L = A.lib()
    nl = A.NodeList(nodes)
    obs = A.observables_array(olist)
    marr, mp = A.i32(mask)
    n = C.c_int64()
    assert L.gf_compile_tree(nl.arr, nl.n, obs, len(olist), len(params), mp, prec, C.byref(n)) == 0, \
        L.gf_last_error(None)
    # without floated amplitude-shape parameters there is nothing to recompute
    fixed = [0 if (v.fixed or v.name.endswith(("_mass", "_width"))) else m for v, m in zip(params, mask)]
    assert "gf_evt_gr(" not in _source(nodes, olist, params, fixed, prec)
