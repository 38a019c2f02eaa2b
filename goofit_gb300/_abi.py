"""ctypes binding of the engine's C ABI (include/gfengine.h).

The shared library is built in-tree by ``goofit_gb300.build`` and must be
present: nothing in this package falls back to a CPU implementation.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "lib" / "libgfengine.so"

# gf_status
GF_OK = 0
GF_ERR_INVALID = 1
GF_ERR_CUDA = 2
GF_ERR_COMPILE = 3
GF_ERR_NAN_NORM = 4
GF_ERR_NONPOS_NORM = 5
GF_ERR_ZERO_NLL = 6
GF_ERR_OOM = 7
GF_ERR_TIMEOUT = 8
GF_ERR_BAD_TREE = 9
GF_ERR_STATE = 10
GF_ERR_NO_DEVICE = 11

GF_FP64 = 0
GF_MIXED = 1

GF_OP_EXP = 1
GF_OP_EXP_OFFSET = 2
GF_OP_EXP_POLY = 3
GF_OP_EXP_POLY_OFFSET = 4
GF_OP_GAUSSIAN = 5
GF_OP_POLYNOMIAL = 6
GF_OP_POLYNOMIAL_OFFSET = 7
GF_OP_ADD = 8
GF_OP_ADD_EXT = 9
GF_OP_PROD = 10
GF_OP_CONVOLUTION = 11
GF_OP_AMP3BODY = 12
GF_OP_AMP4BODY = 13
GF_OP_MULTIPOLYNOMIAL = 14
GF_OP_RES_RBW = 20
GF_OP_RES_NONRES = 21
GF_OP_AMPLITUDE = 15
GF_OP_LS_RBW = 22
GF_OP_LS_SBW = 23
GF_OP_SPINFACTOR = 24

GF_FLAG_COMMON_NORM = 1
GF_FLAG_SEPARATE_NORM = 2

GF_METRIC_EVAL = 0
GF_METRIC_NLL = 1
GF_METRIC_PROB = 2
GF_AMP_AUTO = 0
GF_AMP_STORE = 1
GF_AMP_RECOMPUTE = 2
GF_FIT_UNBINNED_NLL = 0
GF_FIT_BINNED_NLL = 1
GF_FIT_BINNED_ERROR = 2
GF_FIT_BINNED_CHISQ = 3

_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)


class gf_node(C.Structure):
    _fields_ = [
        ("op", C.c_int32),
        ("flags", C.c_int32),
        ("n_params", C.c_int32),
        ("n_consts", C.c_int32),
        ("n_obs", C.c_int32),
        ("n_children", C.c_int32),
        ("params", _i32p),
        ("consts", _f64p),
        ("obs", _i32p),
        ("children", _i32p),
        ("integration_bins", C.c_int32),
        ("reserved", C.c_int32),
    ]


class gf_observable(C.Structure):
    _fields_ = [("lo", C.c_double), ("hi", C.c_double), ("nbins", C.c_int32), ("is_event_number", C.c_int32)]


class gf_fit_result(C.Structure):
    _fields_ = [
        ("fmin", C.c_double),
        ("edm", C.c_double),
        ("nfcn", C.c_int32),
        ("ngrad", C.c_int32),
        ("valid", C.c_int32),
        ("above_max_edm", C.c_int32),
        ("call_limit", C.c_int32),
        ("has_covariance", C.c_int32),
        ("hesse_failed", C.c_int32),
        ("made_posdef", C.c_int32),
        ("n_iter", C.c_int32),
        ("reserved", C.c_int32),
    ]


class gf_fit_options(C.Structure):
    _fields_ = [
        ("err", _f64p),
        ("lo", _f64p),
        ("hi", _f64p),
        ("limited", _i32p),
        ("fixed", _i32p),
        ("up", C.c_double),
        ("tolerance", C.c_double),
        ("strategy", C.c_int32),
        ("maxfcn", C.c_int32),
        ("use_grad", C.c_int32),
        ("reserved", C.c_int32),
        ("fnoise_rel", C.c_double),
        ("cov", _f64p),
    ]


# (name, restype, argtypes) for every entry point declared in include/gfengine.h
_vp = C.c_void_p
SIGNATURES = [
    ("gf_engine_create", C.c_int, [C.POINTER(_vp), C.c_int, C.c_int]),
    ("gf_engine_destroy", C.c_int, [_vp]),
    ("gf_last_error", C.c_char_p, [_vp]),
    ("gf_version", C.c_char_p, []),
    ("gf_set_tree", C.c_int, [_vp, C.POINTER(gf_node), C.c_int, C.POINTER(gf_observable), C.c_int, C.c_int, _i32p]),
    ("gf_set_num_toys", C.c_int, [_vp, C.c_int]),
    ("gf_upload_events", C.c_int, [_vp, C.c_int, _f64p, C.c_int64]),
    ("gf_set_params", C.c_int, [_vp, C.c_int, _f64p, C.c_int]),
    ("gf_nll", C.c_int, [_vp, C.c_int, _f64p]),
    ("gf_nll_grad", C.c_int, [_vp, C.c_int, _f64p, _f64p]),
    ("gf_nll_batch", C.c_int, [_vp, C.c_int, _f64p, _i32p, _f64p, _f64p]),
    ("gf_num_grad", C.c_int, [_vp]),
    ("gf_num_params", C.c_int, [_vp]),
    ("gf_num_toys", C.c_int, [_vp]),
    ("gf_grad_params", C.c_int, [_vp, _i32p, C.c_int]),
    ("gf_normalize", C.c_int, [_vp, C.c_int, _f64p, _f64p]),
    ("gf_eval_events", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _f64p, C.c_int64]),
    ("gf_amp3_integrals", C.c_int, [_vp, C.c_int, C.c_int, _f64p, C.c_int]),
    ("gf_amp3_cached_wave", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _f64p, C.c_int64]),
    ("gf_set_norm_events", C.c_int, [_vp, C.c_int, _f64p, C.c_int64]),
    ("gf_set_fit_metric", C.c_int, [_vp, C.c_int]),
    ("gf_last_timing", C.c_int, [_vp, _f64p, _f64p]),
    ("gf_launches_per_eval", C.c_int, [_vp, C.c_int]),
    ("gf_event_chunk", C.c_int64, [_vp]),
    ("gf_set_wait_limit", C.c_int, [_vp, C.c_uint64]),
    ("gf_set_gram_wait_limit", C.c_int, [_vp, C.c_uint64]),
    ("gf_set_amp_mode", C.c_int, [_vp, C.c_int, C.c_int64]),
    ("gf_amp_recomputing", C.c_int, [_vp]),
    ("gf_amp_store_bytes", C.c_int64, [_vp]),
    ("gf_tune_shapes", C.c_int, [_vp]),
    ("gf_get_shapes", C.c_int, [_vp, _i32p, _i32p, _i32p]),
    ("gf_time_kernels", C.c_int, [_vp, C.c_int, C.c_int, _f64p, _f64p, _f64p]),
    ("gf_minimizer_create", C.c_int, [C.POINTER(_vp), C.c_int, _f64p, _f64p, _f64p, _f64p, _i32p, _i32p,
                                      C.c_double, C.c_int, C.c_double, C.c_int, C.c_int, C.c_double]),
    ("gf_minimizer_ask", C.c_int, [_vp, _f64p, _i32p]),
    ("gf_minimizer_tell", C.c_int, [_vp, C.c_double, _f64p]),
    ("gf_minimizer_result", C.c_int, [_vp, C.POINTER(gf_fit_result), _f64p, _f64p, _f64p]),
    ("gf_minimizer_destroy", C.c_int, [_vp]),
    ("gf_fit", C.c_int, [_vp, C.c_int, C.POINTER(gf_fit_options), _f64p, _f64p, _f64p, C.POINTER(gf_fit_result)]),
    ("gf_fit_batch", C.c_int, [_vp, C.c_int, C.POINTER(gf_fit_options), _f64p, _f64p, _f64p,
                               C.POINTER(gf_fit_result)]),
    ("gf_nll_exp_noalloc", C.c_int, [C.c_void_p, C.c_int64, C.c_double, C.c_double, C.c_double, C.c_void_p,
                                     C.c_void_p]),
    ("gf_noalloc_last_error", C.c_char_p, []),
    ("gf_generated_source", C.c_int, [C.POINTER(gf_node), C.c_int, C.POINTER(gf_observable), C.c_int, C.c_int,
                                      _i32p, C.c_int, C.c_char_p, C.c_int64, C.POINTER(C.c_int64)]),
    ("gf_compile_tree", C.c_int, [C.POINTER(gf_node), C.c_int, C.POINTER(gf_observable), C.c_int, C.c_int,
                                  _i32p, C.c_int, C.POINTER(C.c_int64)]),
    ("gf_compile_tree_batch", C.c_int, [C.POINTER(gf_node), C.c_int, C.POINTER(gf_observable), C.c_int, C.c_int,
                                        _i32p, C.c_int, C.POINTER(C.c_int64)]),
]

_lib = None


class EngineError(RuntimeError):
    """Raised for a non-zero gf_status (mirrors GooFit::GeneralError)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[gf_status {code}] {msg}")
        self.code = code


def lib() -> C.CDLL:
    """Loads libgfengine.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "or `python -m goofit_gb300.build`")
        L = C.CDLL(str(LIB_PATH))
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(code: int, eng=None) -> None:
    if code != GF_OK:
        msg = lib().gf_last_error(eng)
        raise EngineError(code, msg.decode() if msg else "")


def f64(a):
    import numpy as np
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_f64p)


def i32(a):
    import numpy as np
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(_i32p)


class NodeList:
    """Owns the arrays a gf_node list points into."""

    def __init__(self, nodes: list[dict]):
        self._keep = []
        self.arr = (gf_node * len(nodes))()
        for i, n in enumerate(nodes):
            g = self.arr[i]
            g.op = n["op"]
            g.flags = n.get("flags", 0)
            for key, field, conv in (("params", "params", i32), ("consts", "consts", f64),
                                     ("obs", "obs", i32), ("children", "children", i32)):
                vals = n.get(key, [])
                a, p = conv(vals if len(vals) else [0])
                self._keep.append(a)
                setattr(g, field, p)
                setattr(g, "n_" + key, len(vals))
            g.integration_bins = n.get("integration_bins", 0)
        self.n = len(nodes)


def observables_array(obs: list[tuple]) -> C.Array:
    arr = (gf_observable * len(obs))()
    for i, (lo, hi, nb, ev) in enumerate(obs):
        arr[i].lo, arr[i].hi, arr[i].nbins, arr[i].is_event_number = lo, hi, nb, ev
    return arr
