"""C-ABI boundary checks that need no GPU: the library loads, exports every
entry point include/gfengine.h declares, validates trees, and compiles the
generated kernels of the benchmark trees for sm_103a."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import goofit_gb300 as gf
from goofit_gb300 import _abi as A
from goofit_gb300 import workloads as W

HEADER = Path(__file__).resolve().parent.parent / "include" / "gfengine.h"


def declared_symbols():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gf_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = A.lib()
    syms = declared_symbols()
    assert len(syms) >= 25
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    bound = {name for name, _, _ in A.SIGNATURES}
    assert set(syms) <= bound, set(syms) - bound


def test_version_string():
    assert b"sm_103a" in A.lib().gf_version()


def _tree(pdf):
    nodes, params, obs = pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    nd = pdf._nondiff_all()
    mask = [0 if (v.fixed or id(v) in nd) else 1 for v in params]
    return nodes, olist, params, mask


@pytest.mark.parametrize("batch", [False, True])
@pytest.mark.parametrize("prec", [A.GF_MIXED, A.GF_FP64])
@pytest.mark.parametrize("which", ["c1", "c2", "c3"])
def test_generated_kernels_compile_for_sm103a(which, prec, batch):
    """NVRTC compiles the kernels of every workload tree for sm_103a, in the one-toy and the toy-batch
    shapes (different table, grid and event kernels), without a device."""
    if which == "c3":
        pdf = W.c3_model(1500)[0]
    else:
        pdf = (W.make_c1(1000) if which == "c1" else W.make_c2(2000)).pdf
    nodes, olist, params, mask = _tree(pdf)
    nl = A.NodeList(nodes)
    obs = A.observables_array(olist)
    marr, mp = A.i32(mask)
    n = C.c_int64()
    L = A.lib()
    rc = L.gf_generated_source(nl.arr, nl.n, obs, len(olist), len(params), mp, prec, None, 0, C.byref(n))
    assert rc == 0 and n.value > 1000
    compile_tree = L.gf_compile_tree_batch if batch else L.gf_compile_tree
    rc = compile_tree(nl.arr, nl.n, obs, len(olist), len(params), mp, prec, C.byref(n))
    assert rc == 0, L.gf_last_error(None)
    assert n.value > 10000


def test_bad_trees_are_rejected():
    L = A.lib()
    obs = A.observables_array([(0.0, 1.0, 10, 0)])
    cases = [
        [dict(op=A.GF_OP_EXP, params=[0, 1], obs=[0])],                        # wrong arity
        [dict(op=A.GF_OP_ADD, params=[0], obs=[0], children=[0, 1])],         # child before parent
        [dict(op=99, obs=[0])],                                              # unknown operator
        [dict(op=A.GF_OP_EXP, params=[5], obs=[0])],                          # parameter out of range
        [dict(op=A.GF_OP_EXP, params=[0], obs=[0], flags=A.GF_FLAG_COMMON_NORM)],
        [dict(op=A.GF_OP_RES_RBW, params=[0, 1], consts=[3, 0, 1], obs=[])],  # spin 3
        [dict(op=A.GF_OP_MULTIPOLYNOMIAL, params=[0], consts=[1], obs=[0])],   # too few coefficients
    ]
    for nodes in cases:
        nl = A.NodeList(nodes)
        n = C.c_int64()
        rc = L.gf_generated_source(nl.arr, nl.n, obs, 1, 2, None, A.GF_MIXED, None, 0, C.byref(n))
        assert rc == A.GF_ERR_BAD_TREE, nodes


def test_engine_without_device_reports_no_device():
    from tests.conftest import have_gpu
    if have_gpu():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    rc = A.lib().gf_engine_create(C.byref(h), 0, A.GF_MIXED)
    assert rc == A.GF_ERR_NO_DEVICE
    with pytest.raises(A.EngineError):
        gf.Engine("mixed")


def test_amp3body_tree_checks():
    """Amp3Body trees: the efficiency's parameters have no analytic derivative (the resonances' do), and the
    normalisation bins inside the kinematic boundary are found by the FP64 boundary test."""
    from oracle import oracle as O
    pdf = W.c3_model(60)[0]
    nodes, olist, params, mask = _tree(pdf)
    L = A.lib()
    nl = A.NodeList(nodes)
    obs = A.observables_array(olist)
    n = C.c_int64()
    full = [0 if v.fixed else 1 for v in params]
    for v in params:
        if v.name in ("rho770_mass", "constantOne"):
            v.fixed = False
    full = [0 if v.fixed else 1 for v in params]
    marr, mp = A.i32(full)
    rc = L.gf_generated_source(nl.arr, nl.n, obs, len(olist), len(params), mp, A.GF_MIXED, None, 0, C.byref(n))
    assert rc == A.GF_ERR_BAD_TREE and b"efficiency" in L.gf_last_error(None)
    full = [0 if (v.fixed or v.name == "constantOne") else 1 for v in params]
    marr, mp = A.i32(full)
    assert L.gf_generated_source(nl.arr, nl.n, obs, len(olist), len(params), mp, A.GF_MIXED, None, 0, C.byref(n)) == 0
    for v in params:
        if v.name in ("rho770_mass", "constantOne"):
            v.fixed = True
    # the generated normalisation pass loops over exactly the in-Dalitz bins of a 60 x 60 grid
    marr, mp = A.i32(mask)
    rc = L.gf_generated_source(nl.arr, nl.n, obs, len(olist), len(params), mp, A.GF_FP64, None, 0, C.byref(n))
    buf = C.create_string_buffer(n.value + 1)
    L.gf_generated_source(nl.arr, nl.n, obs, len(olist), len(params), mp, A.GF_FP64, buf, n.value + 1, C.byref(n))
    src = buf.value.decode()
    inside = sum(O.in_dalitz(3.0 / 60 * (a + 0.5), 3.0 / 60 * (b + 0.5), W.C3_M, W.C3_MK, W.C3_MPI, W.C3_MPI0)
                 for a in range(60) for b in range(60))
    assert 0 < inside < 3600
    assert f"const i64 npts = {inside}LL," in src
