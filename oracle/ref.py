"""ctypes wrapper of the reference's own likelihood code compiled for the CPU (oracle/_ref/libgoofit_ref.so).

TEST INFRASTRUCTURE ONLY: tests/test_reference_build.py uses it to pin the FP64 restatement
(oracle/oracle.cpp) to the reference's arithmetic; the engine never loads it.

`oracle/ref/Makefile` builds the library from the reference's sources where they lie (GooFit's
src/PDFs/..., src/goofit/..., compiled as C++ with Thrust's OMP backend), with project-written shim
headers for the reference's empty submodules and generated headers (oracle/ref/shim/), link stand-ins for
the Minuit2 fit path and a harness of C entry points (oracle/ref/harness.cpp).  The sources exist only
where the reference checkout is (GOOFIT_REFERENCE, default /root/reference); elsewhere `available()` is
False.

The reference keeps one PDF tree in process-global tables that only grow, so every configuration is built
and evaluated in a fresh spawned process (`isolated`), at all requested parameter points in one go.
"""
from __future__ import annotations

import ctypes as C
import multiprocessing as mp
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_ref" / "libgoofit_ref.so"
REFERENCE = Path(os.environ.get("GOOFIT_REFERENCE", "/root/reference"))
_f64p = C.POINTER(C.c_double)
_i32p = C.POINTER(C.c_int)


def available() -> bool:
    """The reference sources are present (the library can be built here)."""
    return (REFERENCE / "src" / "PDFs" / "GooPdf.cu").exists()


def build() -> Path:
    subprocess.run(["make", "-s", f"-j{min(16, os.cpu_count() or 4)}", "-C", str(HERE / "ref"), f"REF={REFERENCE}"],
                   check=True)
    return LIB


def _lib() -> C.CDLL:
    L = C.CDLL(str(LIB))
    L.ref_last_error.restype = C.c_char_p
    return L


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _check(L, rc):
    if rc:
        raise RuntimeError("reference build: " + L.ref_last_error().decode())


def _exp_nll(x, lo, hi, P):
    L = _lib()
    x, P = _d(x), _d(P)
    out = np.zeros(len(P))
    _check(L, L.ref_exp_nll(x.ctypes.data_as(_f64p), C.c_long(len(x)), C.c_double(lo), C.c_double(hi),
                            P.ctypes.data_as(_f64p), len(P), out.ctypes.data_as(_f64p)))
    return out


def _c2_nll(x, xlo, xhi, bins, conv, P):
    L = _lib()
    x, conv, P = _d(x), _d(conv), _d(P).reshape(-1, 5)
    out = np.zeros(len(P))
    _check(L, L.ref_c2_nll(x.ctypes.data_as(_f64p), C.c_long(len(x)), C.c_double(xlo), C.c_double(xhi), int(bins),
                           conv.ctypes.data_as(_f64p), P.ctypes.data_as(_f64p), len(P), out.ctypes.data_as(_f64p)))
    return out


def _prod_nll(xs, ys, P):
    L = _lib()
    xs, ys, P = _d(xs), _d(ys), _d(P).reshape(-1, 3)
    out = np.zeros(len(P))
    _check(L, L.ref_prod_nll(xs.ctypes.data_as(_f64p), ys.ctypes.data_as(_f64p), C.c_long(len(xs)),
                             P.ctypes.data_as(_f64p), len(P), out.ctypes.data_as(_f64p)))
    return out


def _prod_overlap_nll(xs, bins, P):
    L = _lib()
    xs, P = _d(xs), _d(P).reshape(-1, 3)
    out = np.zeros(len(P))
    _check(L, L.ref_prod_overlap_nll(xs.ctypes.data_as(_f64p), C.c_long(len(xs)), int(bins), P.ctypes.data_as(_f64p),
                                     len(P), out.ctypes.data_as(_f64p)))
    return out


def _extadd_nll(xs, P):
    L = _lib()
    xs, P = _d(xs), _d(P).reshape(-1, 5)
    out = np.zeros(len(P))
    _check(L, L.ref_extadd_nll(xs.ctypes.data_as(_f64p), C.c_long(len(xs)), P.ctypes.data_as(_f64p), len(P),
                               out.ctypes.data_as(_f64p)))
    return out


def _amp3_nll(m12, m13, bins, dec, spin, cyc, P):
    L = _lib()
    m12, m13, dec = _d(m12), _d(m13), _d(dec)
    spin = np.ascontiguousarray(spin, dtype=np.int32)
    cyc = np.ascontiguousarray(cyc, dtype=np.int32)
    nres = len(spin)
    P = _d(P).reshape(-1, 4 * nres)
    out = np.zeros(len(P))
    _check(L, L.ref_amp3_nll(m12.ctypes.data_as(_f64p), m13.ctypes.data_as(_f64p), C.c_long(len(m12)), int(bins),
                             dec.ctypes.data_as(_f64p), nres, spin.ctypes.data_as(_i32p), cyc.ctypes.data_as(_i32p),
                             P.ctypes.data_as(_f64p), len(P), out.ctypes.data_as(_f64p)))
    return out


def _amp4_nll(ev5, masses, norm_p4, P):
    L = _lib()
    ev5, masses = _d(ev5).reshape(5, -1), _d(masses)
    norm_p4 = _d(norm_p4).reshape(-1, 4, 4)
    P = _d(P).reshape(-1, 22)
    out = np.zeros(len(P))
    _check(L, L.ref_amp4_nll(ev5.ctypes.data_as(_f64p), C.c_long(ev5.shape[1]), masses.ctypes.data_as(_f64p),
                             norm_p4.ctypes.data_as(_f64p), C.c_long(norm_p4.shape[0]), P.ctypes.data_as(_f64p),
                             len(P), out.ctypes.data_as(_f64p)))
    return out


def _dim5(p4):
    L = _lib()
    p4 = _d(p4).reshape(-1, 4, 4)
    out = np.zeros((5, p4.shape[0]))
    _check(L, L.ref_dim5(p4.ctypes.data_as(_f64p), C.c_long(p4.shape[0]), out.ctypes.data_as(_f64p)))
    return out


def _run(q, fn, args):
    try:
        q.put(("ok", globals()[fn](*args)))
    except Exception as e:  # reported in the parent
        q.put(("err", repr(e)))


def isolated(fn: str, *args, timeout: float = 600.0):
    """Runs one of the entry points above (by name: exp_nll, c2_nll, prod_nll, prod_overlap_nll, extadd_nll,
    amp3_nll, amp4_nll, dim5) in a fresh
    spawned process and returns its result."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=_run, args=(q, "_" + fn, args))
    p.start()
    try:
        status, val = q.get(timeout=timeout)
    finally:
        p.join(30)
    if status != "ok":
        raise RuntimeError(val)
    return val
