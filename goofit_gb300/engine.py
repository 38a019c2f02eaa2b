"""Object wrapper over the engine C ABI (include/gfengine.h).

`Engine` owns one gf_engine handle: a PDF tree (node list), its datasets
("toys") resident in HBM and the generated kernels.  `Minimizer` exposes the
ask/tell minimiser.  Everything here calls libgfengine.so; there is no CPU
path.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _abi as A

PRECISIONS = {"fp64": A.GF_FP64, "mixed": A.GF_MIXED}


@dataclass
class FitResult:
    """Outcome of one MIGRAD fit (the FunctionMinimum fields the reference reads)."""
    values: np.ndarray
    errors: np.ndarray
    fmin: float
    edm: float
    nfcn: int
    ngrad: int
    valid: bool
    above_max_edm: bool
    call_limit: bool
    has_covariance: bool
    hesse_failed: bool
    made_posdef: bool
    n_iter: int
    covariance: np.ndarray | None = None  # external covariance of the final Hesse (n x n), when requested

    @staticmethod
    def from_c(r: A.gf_fit_result, x, e, cov=None) -> "FitResult":
        return FitResult(np.array(x, dtype=float), np.array(e, dtype=float), r.fmin, r.edm, r.nfcn, r.ngrad,
                         bool(r.valid), bool(r.above_max_edm), bool(r.call_limit), bool(r.has_covariance),
                         bool(r.hesse_failed), bool(r.made_posdef), r.n_iter, cov)

    # Minuit2::FunctionMinimum spellings used by GooFit users
    def IsValid(self) -> bool:
        return self.valid

    def Fval(self) -> float:
        return self.fmin

    def Edm(self) -> float:
        return self.edm

    def NFcn(self) -> int:
        return self.nfcn


def _fit_options(n, err, lo, hi, limited, fixed, up, tolerance, strategy, maxfcn, use_grad, fnoise_rel=0.0):
    keep = []

    def f(a):
        arr, p = A.f64(a)
        keep.append(arr)
        return p

    def i(a):
        arr, p = A.i32(a)
        keep.append(arr)
        return p

    o = A.gf_fit_options()
    o.err = f(err)
    o.lo = f(lo)
    o.hi = f(hi)
    o.limited = i(limited)
    o.fixed = i(fixed)
    o.up = up
    o.tolerance = tolerance
    o.strategy = strategy
    o.maxfcn = maxfcn
    o.use_grad = 1 if use_grad else 0
    o.fnoise_rel = fnoise_rel
    return o, keep


class Engine:
    """One likelihood engine on one GPU."""

    def __init__(self, precision: str = "mixed", device: int = 0):
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {list(PRECISIONS)}")
        self.precision = precision
        self._h = C.c_void_p()
        self._L = A.lib()
        A.check(self._L.gf_engine_create(C.byref(self._h), device, PRECISIONS[precision]))
        self.n_params = 0
        self.n_grad = 0
        self.grad_params: list[int] = []
        self.n_obs = 0
        self.n_toys = 1
        self._n_events: dict[int, int] = {}

    def close(self) -> None:
        if self._h:
            self._L.gf_engine_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int) -> None:
        A.check(rc, self._h)

    # ---- tree / data ----
    def set_fit_metric(self, metric: int) -> None:
        """GF_FIT_UNBINNED_NLL (default) or a binned metric; before set_tree."""
        self._check(self._L.gf_set_fit_metric(self._h, metric))
        self.fit_metric = metric

    def set_tree(self, nodes: list[dict], observables: list[tuple], n_params: int, grad_mask=None) -> None:
        self._nodes = A.NodeList(nodes)
        self._obs = A.observables_array(observables)
        mask = np.zeros(max(n_params, 1), dtype=np.int32) if grad_mask is None else np.asarray(grad_mask, np.int32)
        marr, mp = A.i32(mask)
        self._check(self._L.gf_set_tree(self._h, self._nodes.arr, self._nodes.n, self._obs, len(observables),
                                        n_params, mp))
        self.n_params = n_params
        # binned metrics carry two more rows: bin contents and volumes (or errors)
        self.n_obs = len(observables) + (2 if getattr(self, "fit_metric", 0) else 0)
        self.n_grad = self._L.gf_num_grad(self._h)
        buf = (C.c_int32 * max(1, self.n_grad))()
        self._L.gf_grad_params(self._h, buf, self.n_grad)
        self.grad_params = [buf[i] for i in range(self.n_grad)]
        self.n_toys = 1
        self._n_events = {}

    def set_num_toys(self, n: int) -> None:
        self._check(self._L.gf_set_num_toys(self._h, n))
        self.n_toys = n
        self._n_events = {}

    def upload(self, soa: np.ndarray, toy: int = 0) -> None:
        """soa: (n_obs, n_events) float64 array (or 1-D for one observable)."""
        a = np.asarray(soa, dtype=np.float64)
        if a.ndim == 1:
            a = a.reshape(1, -1)
        if a.shape[0] != self.n_obs:
            raise ValueError(f"expected {self.n_obs} observable rows, got {a.shape[0]}")
        arr, p = A.f64(a)
        self._check(self._L.gf_upload_events(self._h, toy, p, a.shape[1]))
        self._n_events[toy] = a.shape[1]

    # ---- evaluation ----
    def set_params(self, params, toy: int = 0) -> None:
        arr, p = A.f64(params)
        self._check(self._L.gf_set_params(self._h, toy, p, len(arr)))

    def nll(self, params=None, toy: int = 0) -> float:
        if params is not None:
            self.set_params(params, toy)
        out = C.c_double()
        self._check(self._L.gf_nll(self._h, toy, C.byref(out)))
        return out.value

    def nll_grad(self, params=None, toy: int = 0) -> tuple[float, np.ndarray]:
        if params is not None:
            self.set_params(params, toy)
        out = C.c_double()
        g = np.zeros(max(1, self.n_grad))
        self._check(self._L.gf_nll_grad(self._h, toy, C.byref(out), g.ctypes.data_as(A._f64p)))
        return out.value, g[: self.n_grad]

    def nll_batch(self, P: np.ndarray, active=None, grad: bool = False):
        P = np.ascontiguousarray(P, dtype=np.float64).reshape(self.n_toys, self.n_params)
        nll = np.zeros(self.n_toys)
        G = np.zeros((self.n_toys, max(1, self.n_grad))) if grad else None
        act = None if active is None else np.ascontiguousarray(active, dtype=np.int32)
        rc = self._L.gf_nll_batch(self._h, self.n_toys, P.ctypes.data_as(A._f64p),
                                  None if act is None else act.ctypes.data_as(A._i32p),
                                  nll.ctypes.data_as(A._f64p), None if G is None else G.ctypes.data_as(A._f64p))
        self._check(rc)
        return (nll, G[:, : self.n_grad]) if grad else nll

    def normalize(self, toy: int = 0) -> tuple[np.ndarray, np.ndarray]:
        n = self._nodes.n
        I = np.zeros(n)
        N = np.zeros(n)
        self._check(self._L.gf_normalize(self._h, toy, I.ctypes.data_as(A._f64p), N.ctypes.data_as(A._f64p)))
        return I, N

    def eval_events(self, metric: int = A.GF_METRIC_PROB, toy: int = 0) -> np.ndarray:
        n = self._n_events.get(toy, 0)
        out = np.zeros(max(1, n))
        self._check(self._L.gf_eval_events(self._h, toy, 0, metric, out.ctypes.data_as(A._f64p), n))
        return out[:n]

    def set_norm_events(self, node: int, soa5: np.ndarray) -> None:
        """Flat phase-space normalisation events (5, n) of Amp4Body node `node`."""
        a = np.ascontiguousarray(soa5, dtype=np.float64)
        self._check(self._L.gf_set_norm_events(self._h, node, a.ctypes.data_as(A._f64p), a.shape[1]))

    def amp3_integrals(self, node: int, n_res: int, toy: int = 0) -> np.ndarray:
        """Amp3Body normalisation integrals I_ij (n x n complex) at the toy's current parameters."""
        out = np.zeros(2 * n_res * n_res)
        self._check(self._L.gf_amp3_integrals(self._h, toy, node, out.ctypes.data_as(A._f64p), len(out)))
        return (out[0::2] + 1j * out[1::2]).reshape(n_res, n_res)

    def amp3_cached_wave(self, node: int, res: int, toy: int = 0) -> np.ndarray:
        """Cached amplitude of resonance `res` for every event of the toy (complex128)."""
        n = self._n_events.get(toy, 0)
        out = np.zeros(max(2, 2 * n))
        self._check(self._L.gf_amp3_cached_wave(self._h, toy, node, res, out.ctypes.data_as(A._f64p), n))
        return out[0:2 * n:2] + 1j * out[1:2 * n:2]

    def last_timing(self) -> tuple[float, float]:
        a, b = C.c_double(), C.c_double()
        self._L.gf_last_timing(self._h, C.byref(a), C.byref(b))
        return a.value, b.value

    def time_kernels(self, grad: bool = True, toy: int = 0) -> tuple[float, float, float]:
        """(conv, grid, event) kernel times in ms, each launched alone with CUDA events."""
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        self._check(self._L.gf_time_kernels(self._h, toy, 1 if grad else 0, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def launches_per_eval(self, grad: bool = True) -> int:
        return self._L.gf_launches_per_eval(self._h, 1 if grad else 0)

    def set_wait_limit(self, ns: int) -> None:
        """Longest device-side wait at the one-launch evaluation's grid barrier (ns; 0: the default 1 s)."""
        self._check(self._L.gf_set_wait_limit(self._h, int(ns)))

    def set_gram_wait_limit(self, ns: int) -> None:
        """Longest wait of each pipeline stage of the tensor-core Gram kernel (ns; 0: the default 2 s)."""
        self._check(self._L.gf_set_gram_wait_limit(self._h, int(ns)))

    def set_amp_mode(self, mode: str, budget_bytes: int = 0) -> None:
        """Amplitude derivatives 'store'd per event and normalisation point, 'recompute'd where they are used,
        or 'auto' (recompute when storing would take more than budget_bytes; 0: a quarter of the free device
        memory).  Before the first upload."""
        m = {"auto": A.GF_AMP_AUTO, "store": A.GF_AMP_STORE, "recompute": A.GF_AMP_RECOMPUTE}[mode]
        self._check(self._L.gf_set_amp_mode(self._h, m, int(budget_bytes)))

    def amp_recomputing(self) -> int | None:
        """True / False once decided (the first upload after set_tree), None before."""
        r = int(self._L.gf_amp_recomputing(self._h))
        return None if r < 0 else bool(r)

    def amp_store_bytes(self) -> int:
        """Device bytes the store mode keeps for amplitude derivatives and normalisation points."""
        return int(self._L.gf_amp_store_bytes(self._h))

    def tune_shapes(self) -> dict:
        """Runs the launch-shape autotuner (table k-tiles, grid bins per CTA, Gram slice width) on the uploaded
        events and returns the shapes in use."""
        self._check(self._L.gf_tune_shapes(self._h))
        return self.shapes()

    def shapes(self) -> dict:
        kp, bpb, w = C.c_int32(), C.c_int32(), C.c_int32()
        self._check(self._L.gf_get_shapes(self._h, C.byref(kp), C.byref(bpb), C.byref(w)))
        return {"conv_kp": kp.value, "grid_bins_per_cta": bpb.value, "gram_slice_width": w.value,
                "event_chunk": self.event_chunk()}

    def event_chunk(self) -> int:
        """Events per chunk of the event pass (after the autotuner, once an evaluation has run)."""
        return int(self._L.gf_event_chunk(self._h))

    # ---- fits ----
    def default_fnoise(self, n_events: int | None = None) -> float:
        """Relative rounding noise of the NLL in the mixed path.  FP32 per-event terms summed into
        compensated pairs leave a random rounding of about 1e-7 * sqrt(n) absolute, 1e-7 / sqrt(n)
        relative; the line search treats changes below 15 times that as ties (clamped to [1e-9, 2e-8])."""
        if self.precision != "mixed":
            return 0.0
        n = n_events if n_events else max(self._n_events.values(), default=1)
        return float(min(2e-8, max(1e-9, 1.5e-6 / math.sqrt(max(1, n)))))

    def fit(self, x0, err, lo, hi, limited, fixed, *, up=0.5, tolerance=0.1, strategy=1, maxfcn=0,
            use_grad=True, toy: int = 0, fnoise_rel=None) -> FitResult:
        n = self.n_params
        fn = self.default_fnoise(self._n_events.get(toy)) if fnoise_rel is None else fnoise_rel
        o, keep = _fit_options(n, err, lo, hi, limited, fixed, up, tolerance, strategy, maxfcn, use_grad, fn)
        xa, xp = A.f64(x0)
        x = np.zeros(n)
        e = np.zeros(n)
        cov = np.zeros((n, n))
        o.cov = cov.ctypes.data_as(A._f64p)
        r = A.gf_fit_result()
        self._check(self._L.gf_fit(self._h, toy, C.byref(o), xp, x.ctypes.data_as(A._f64p),
                                   e.ctypes.data_as(A._f64p), C.byref(r)))
        return FitResult.from_c(r, x, e, cov)

    def fit_batch(self, X0, err, lo, hi, limited, fixed, *, up=0.5, tolerance=0.1, strategy=1, maxfcn=0,
                  use_grad=True, fnoise_rel=None) -> list[FitResult]:
        n = self.n_params
        T = self.n_toys
        # one tolerance for the batch: that of the smallest toy
        fn = self.default_fnoise(min(self._n_events.values(), default=1)) if fnoise_rel is None else fnoise_rel
        o, keep = _fit_options(n, err, lo, hi, limited, fixed, up, tolerance, strategy, maxfcn, use_grad, fn)
        X0 = np.ascontiguousarray(X0, dtype=np.float64).reshape(T, n)
        X = np.zeros((T, n))
        E = np.zeros((T, n))
        COV = np.zeros((T, n, n))
        o.cov = COV.ctypes.data_as(A._f64p)
        R = (A.gf_fit_result * T)()
        self._check(self._L.gf_fit_batch(self._h, T, C.byref(o), X0.ctypes.data_as(A._f64p),
                                         X.ctypes.data_as(A._f64p), E.ctypes.data_as(A._f64p), R))
        return [FitResult.from_c(R[t], X[t], E[t], COV[t]) for t in range(T)]


class Minimizer:
    """Ask/tell MIGRAD (same code the native fit loop uses)."""

    def __init__(self, x0, err, lo=None, hi=None, limited=None, fixed=None, *, up=0.5, strategy=1, tolerance=0.1,
                 maxfcn=0, use_grad=False, fnoise_rel=0.0):
        n = len(x0)
        self.n = n
        self._L = A.lib()
        self._h = C.c_void_p()
        z = np.zeros(n)
        arrs = [A.f64(x0), A.f64(err), A.f64(z if lo is None else lo), A.f64(z if hi is None else hi),
                A.i32(np.zeros(n, np.int32) if limited is None else limited),
                A.i32(np.zeros(n, np.int32) if fixed is None else fixed)]
        self._keep = [a for a, _ in arrs]
        A.check(self._L.gf_minimizer_create(C.byref(self._h), n, *[p for _, p in arrs], up, strategy, tolerance,
                                            maxfcn, 1 if use_grad else 0, fnoise_rel))

    def minimize(self, fcn, grad=None) -> FitResult:
        """fcn(x) -> float; grad(x) -> array (needed if use_grad)."""
        x = np.zeros(self.n)
        need = C.c_int32()
        while self._L.gf_minimizer_ask(self._h, x.ctypes.data_as(A._f64p), C.byref(need)) == 1:
            f = float(fcn(x.copy()))
            if need.value:
                g = np.ascontiguousarray(grad(x.copy()), dtype=np.float64)
                self._L.gf_minimizer_tell(self._h, f, g.ctypes.data_as(A._f64p))
            else:
                self._L.gf_minimizer_tell(self._h, f, None)
        return self.result()

    def result(self) -> FitResult:
        r = A.gf_fit_result()
        x = np.zeros(self.n)
        e = np.zeros(self.n)
        self._L.gf_minimizer_result(self._h, C.byref(r), x.ctypes.data_as(A._f64p), e.ctypes.data_as(A._f64p), None)
        return FitResult.from_c(r, x, e)

    def covariance(self) -> np.ndarray:
        r = A.gf_fit_result()
        cov = np.zeros((self.n, self.n))
        self._L.gf_minimizer_result(self._h, C.byref(r), None, None, cov.ctypes.data_as(A._f64p))
        return cov

    def __del__(self):
        try:
            if self._h:
                self._L.gf_minimizer_destroy(self._h)
        except Exception:
            pass
