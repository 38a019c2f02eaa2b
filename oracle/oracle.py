"""ctypes wrapper of the FP64 CPU oracle (oracle/oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by bench.py's CPU-baseline leg
and by __graft_entry__.smoke() as the checker; the engine never uses it.
The library is built by `make -C oracle` into oracle/_build/.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

from goofit_gb300 import _abi as A

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists() or LIB.stat().st_mtime < max((HERE / f).stat().st_mtime for f in ("oracle.cpp", "amp4.h")):
            build()
        L = C.CDLL(str(LIB))
        f64p, i32p = C.POINTER(C.c_double), C.POINTER(C.c_int32)
        L.oracle_evaluate.argtypes = [C.POINTER(A.gf_node), C.c_int, C.POINTER(A.gf_observable), C.c_int, f64p,
                                      C.c_int, f64p, C.c_int64, C.c_int, C.c_int, C.c_int, f64p, f64p, f64p]
        L.oracle_evaluate.restype = C.c_int
        L.oracle_nll.argtypes = [C.POINTER(A.gf_node), C.c_int, C.POINTER(A.gf_observable), C.c_int, f64p, C.c_int,
                                 f64p, C.c_int64, C.c_int, f64p]
        L.oracle_nll.restype = C.c_int
        L.oracle_last_error.restype = C.c_char_p
        L.oracle_mt19937_exponential.argtypes = [C.c_uint32, C.c_double, C.c_int64, f64p]
        L.oracle_num_threads.restype = C.c_int
        L.oracle_amp3_integrals.argtypes = [C.POINTER(A.gf_node), C.c_int, C.POINTER(A.gf_observable), C.c_int,
                                            f64p, C.c_int, C.c_int, f64p]
        L.oracle_amp3_integrals.restype = C.c_int
        L.oracle_amp3_resonance.argtypes = [C.POINTER(A.gf_node), C.c_int, C.POINTER(A.gf_observable), C.c_int,
                                            f64p, C.c_int, C.c_int, C.c_int, f64p, f64p, C.c_int64, f64p]
        L.oracle_amp3_resonance.restype = C.c_int
        L.oracle_binned.argtypes = [C.POINTER(A.gf_node), C.c_int, C.POINTER(A.gf_observable), C.c_int, f64p,
                                    C.c_int, f64p, C.c_int64, C.c_int, f64p]
        L.oracle_binned.restype = C.c_int
        L.oracle_set_amp4_norm_events.argtypes = [f64p, C.c_int64]
        L.oracle_amp4_gram.argtypes = [C.POINTER(A.gf_node), C.c_int, C.POINTER(A.gf_observable), C.c_int, f64p,
                                       C.c_int, C.c_int, f64p]
        L.oracle_amp4_gram.restype = C.c_int
        L.oracle_amp4_amplitudes.argtypes = [C.POINTER(A.gf_node), C.c_int, C.POINTER(A.gf_observable), C.c_int,
                                             f64p, C.c_int, C.c_int, f64p, C.c_int64, f64p]
        L.oracle_amp4_amplitudes.restype = C.c_int
        L.oracle_get4vecs.argtypes = [f64p, f64p, f64p]
        L.oracle_in_dalitz.argtypes = [C.c_double] * 6
        L.oracle_in_dalitz.restype = C.c_int
        _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


def _prep(nodes, observables, params, soa):
    nl = A.NodeList(nodes)
    obs = A.observables_array(observables)
    p, pp = A.f64(params)
    s = np.ascontiguousarray(np.asarray(soa, dtype=np.float64).reshape(len(observables), -1))
    return nl, obs, p, pp, s


def nll(nodes, observables, params, soa, brute_force: bool = False) -> float:
    """GooPdf::calculateNLL restated in FP64 (root = node 0)."""
    L = lib()
    nl, obs, p, pp, s = _prep(nodes, observables, params, soa)
    out = C.c_double()
    rc = L.oracle_nll(nl.arr, nl.n, obs, len(observables), pp, len(p), s.ctypes.data_as(C.POINTER(C.c_double)),
                      s.shape[1], 1 if brute_force else 0, C.byref(out))
    if rc:
        raise OracleError(L.oracle_last_error().decode())
    return out.value


def evaluate(nodes, observables, params, soa, metric: int = A.GF_METRIC_PROB, root: int = 0,
             brute_force: bool = False):
    """Per-event metric values plus every node's normalize() integral and factor."""
    L = lib()
    nl, obs, p, pp, s = _prep(nodes, observables, params, soa)
    n = s.shape[1]
    out = np.zeros(max(n, 1))
    I = np.zeros(nl.n)
    N = np.zeros(nl.n)
    f64p = C.POINTER(C.c_double)
    rc = L.oracle_evaluate(nl.arr, nl.n, obs, len(observables), pp, len(p), s.ctypes.data_as(f64p), n, root,
                           metric, 1 if brute_force else 0, out.ctypes.data_as(f64p), I.ctypes.data_as(f64p),
                           N.ctypes.data_as(f64p))
    if rc:
        raise OracleError(L.oracle_last_error().decode())
    return out[:n], I, N


def fd_grad(nodes, observables, params, soa, indices, h: float = 1e-5) -> np.ndarray:
    """Central finite differences of the oracle NLL (step h relative to max(1, |p|))."""
    p0 = np.asarray(params, dtype=np.float64)
    g = np.zeros(len(indices))
    for j, i in enumerate(indices):
        step = h * max(1.0, abs(p0[i]))
        pp, pm = p0.copy(), p0.copy()
        pp[i] += step
        pm[i] -= step
        g[j] = (nll(nodes, observables, pp, soa) - nll(nodes, observables, pm, soa)) / (2 * step)
    return g


def minimum_offset_sigma(nodes, observables, params, soa, cov, free, h: float = 1e-5) -> np.ndarray:
    """Distance, per free parameter and in units of its error, from `params` to the oracle's own NLL
    minimum: one Newton step -V g with g the oracle's central-difference gradient at `params` and V the
    fit's covariance (for an NLL with up = 0.5, V is the inverse Hessian).  Exact for a quadratic NLL, so a
    fitted point within 0.01 sigma of the oracle's minimum gives values below 0.01 here."""
    free = list(free)
    g = fd_grad(nodes, observables, params, soa, free, h=h)
    V = np.asarray(cov, dtype=np.float64)[np.ix_(free, free)]
    step = V @ g
    return np.abs(step) / np.sqrt(np.diag(V))


def mt19937_exponential(seed: int, lam: float, n: int) -> np.ndarray:
    """std::mt19937(seed) + std::exponential_distribution<>(lam) draws."""
    out = np.zeros(n)
    lib().oracle_mt19937_exponential(seed, lam, n, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def num_threads() -> int:
    return lib().oracle_num_threads()


def amp3_integrals(nodes, observables, params, node: int, n_res: int) -> np.ndarray:
    """Amp3Body integrals I_ij (n x n complex, before the bin size factor) of `node`."""
    nl, obs, p, pp, _ = _prep(nodes, observables, params, np.zeros((len(observables), 1)))
    out = np.zeros(2 * n_res * n_res)
    rc = lib().oracle_amp3_integrals(nl.arr, nl.n, obs, len(observables), pp, len(p), node,
                                     out.ctypes.data_as(C.POINTER(C.c_double)))
    if rc:
        raise OracleError(lib().oracle_last_error().decode())
    return (out[0::2] + 1j * out[1::2]).reshape(n_res, n_res)


def amp3_resonance(nodes, observables, params, node: int, res: int, m12, m13) -> np.ndarray:
    """Amplitude of resonance node `res` of Amp3Body `node` at the given points (zero outside the plot)."""
    nl, obs, p, pp, _ = _prep(nodes, observables, params, np.zeros((len(observables), 1)))
    a = np.ascontiguousarray(m12, dtype=np.float64)
    b = np.ascontiguousarray(m13, dtype=np.float64)
    out = np.zeros(2 * len(a))
    f64p = C.POINTER(C.c_double)
    rc = lib().oracle_amp3_resonance(nl.arr, nl.n, obs, len(observables), pp, len(p), node, res,
                                     a.ctypes.data_as(f64p), b.ctypes.data_as(f64p), len(a), out.ctypes.data_as(f64p))
    if rc:
        raise OracleError(lib().oracle_last_error().decode())
    return out[0::2] + 1j * out[1::2]


def in_dalitz(m12: float, m13: float, M: float, d1: float, d2: float, d3: float) -> bool:
    return bool(lib().oracle_in_dalitz(m12, m13, M, d1, d2, d3))


def set_amp4_norm_events(soa5) -> None:
    """Flat phase-space normalisation events (5, n) used by every later Amp4Body normalisation."""
    a = np.ascontiguousarray(soa5, dtype=np.float64)
    lib().oracle_set_amp4_norm_events(a.ctypes.data_as(C.POINTER(C.c_double)), a.shape[1])


def amp4_gram(nodes, observables, params, node: int, n_amp: int) -> np.ndarray:
    """G_ab = sum over the normalisation events of A_a conj(A_b) of Amp4Body `node`."""
    nl, obs, p, pp, _ = _prep(nodes, observables, params, np.zeros((len(observables), 1)))
    out = np.zeros(2 * n_amp * n_amp)
    rc = lib().oracle_amp4_gram(nl.arr, nl.n, obs, len(observables), pp, len(p), node,
                                out.ctypes.data_as(C.POINTER(C.c_double)))
    if rc:
        raise OracleError(lib().oracle_last_error().decode())
    return (out[0::2] + 1j * out[1::2]).reshape(n_amp, n_amp)


def amp4_amplitudes(nodes, observables, params, node: int, n_amp: int, soa5) -> np.ndarray:
    """Amplitudes (n, n_amp) complex of Amp4Body `node` at the points soa5 (5, n)."""
    nl, obs, p, pp, _ = _prep(nodes, observables, params, np.zeros((len(observables), 1)))
    v = np.ascontiguousarray(soa5, dtype=np.float64)
    n = v.shape[1]
    out = np.zeros(2 * n * n_amp)
    f64p = C.POINTER(C.c_double)
    rc = lib().oracle_amp4_amplitudes(nl.arr, nl.n, obs, len(observables), pp, len(p), node, v.ctypes.data_as(f64p), n,
                                      out.ctypes.data_as(f64p))
    if rc:
        raise OracleError(lib().oracle_last_error().decode())
    return (out[0::2] + 1j * out[1::2]).reshape(n, n_amp)


def get4vecs(v5, masses5) -> np.ndarray:
    """get4Vecs at one point: (4, 4) daughter 4-vectors (x, y, z, E)."""
    f64p = C.POINTER(C.c_double)
    a = np.ascontiguousarray(v5, dtype=np.float64)
    m = np.ascontiguousarray(masses5, dtype=np.float64)
    out = np.zeros(16)
    lib().oracle_get4vecs(a.ctypes.data_as(f64p), m.ctypes.data_as(f64p), out.ctypes.data_as(f64p))
    return out.reshape(4, 4)


def binned(nodes, observables, params, soa, metric: int) -> float:
    """A binned fit's objective; soa = bin centres of the observables, contents, volumes (or errors)."""
    obs_all = list(observables) + [(-1e300, 1e300, 1, 0), (-1e300, 1e300, 1, 0)]
    nl, obs, p, pp, s = _prep(nodes, obs_all, params, soa)
    out = C.c_double()
    rc = lib().oracle_binned(nl.arr, nl.n, obs, len(obs_all), pp, len(p), s.ctypes.data_as(C.POINTER(C.c_double)),
                             s.shape[1], metric, C.byref(out))
    if rc:
        raise OracleError(lib().oracle_last_error().decode())
    return out.value
