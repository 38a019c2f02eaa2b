"""Benchmark of the fit path on the composite 1-D workload (2,000,000 events), with --config c1/c3/c4/c5
legs for the other configurations.

Workload (default, C2): AddPdf(fsig; ConvolutionPdf(ExpPdf(alpha), GaussianPdf(mu, sigma)), flat
PolynomialPdf) on x in [-5, 10], tau = 1.5, mu = 0, sigma = 0.3, background fraction 0.3, 10,000-bin
numeric normalisation, 2e6 seeded synthetic events (accept-reject on the model density).

A step is one FCN call of MIGRAD on the whole dataset: the NLL and its analytic gradient with
respect to the four floated parameters, i.e. 2e6 event-NLL evaluations.  `value` is event-NLL
evaluations per second with the events resident in HBM; the L2 cache (129 MB) is flushed with a
256 MB write before every timed step because the event columns (16 MB) would otherwise stay in L2.
`e2e` repeats the step through the C ABI with host buffers: the FP64 events are copied from pinned
host memory and converted on the device every step, and the NLL/gradient are read back.

`fit` runs MIGRAD at tolerance 0.01 three ways on the same data: mixed precision + analytic gradient,
FP64 + analytic gradient (the precision change alone) and FP64 + numerical gradient (the reference's
plain path); `parity` compares the mixed fit with the FP64 fit and, outside any timed region, with the
FP64 oracle (NLL at the minimum, and the distance to the oracle's own minimum in units of sigma).

--impl reference times the reference algorithm on the host cores instead: the FP64 restatement of
GooFit's OMP path (brute-force convolution per event, numeric normalisation), on a bounded sample.

--gpus N (under torchrun) runs N independent replicas (the fit path does not shard in this
configuration); value is the sum over ranks of events / max step time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "MIGRAD fit wall-time & event-NLL evals/s: mixed-prec vs FP64 on GB300 at 1e-6 rel NLL"
# DRAM bytes of one gf_evt_g launch over 2e6 events, from one ncu capture (profiles/gf_evt_g_c2_composite_2e6.md)
EVT_DRAM_BYTES_PER_LAUNCH = 8_055_040
EVT_DRAM_EVENTS = 2_000_000
# DRAM bytes of one gf_evt_g launch of the amplitude workloads (profiles/gf_evt_g_amp3_amp4_c3_c5.md):
# C3 over 5e5 events, C5 over 3e5 events
EVT_DRAM_BYTES_AMP = {"c3": (32_034_048, 500_000), "c5": (14_432_256, 300_000)}
# DRAM bytes of one gf_fcn_g launch (the one-launch FCN) over 2e6 events, from one ncu capture
# (profiles/gf_fcn_g_c2_composite_2e6.md)
FCN_DRAM_BYTES = 8_084_736
FCN_DRAM_SOURCE = "ncu dram__bytes_read.sum + dram__bytes_write.sum, profiles/gf_fcn_g_c2_composite_2e6.md"
N_EVENTS = 2_000_000
WORKLOAD = "c2: AddPdf(0.7 Conv(Exp tau=1.5, Gauss mu=0 sigma=0.3) + 0.3 flat Poly), x in [-5,10], 2e6 events"


def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0), "src": "measured"}
    return {"hbm_gbs": 6800.0, "src": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def barrier_max(value: float, world: int, device: str | None) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args) -> dict:
    """The reference algorithm (oracle port, brute-force convolution) on all host cores."""
    import numpy as np

    from goofit_gb300 import workloads as W
    from oracle import oracle as O

    sample = args.ref_sample
    wl = W.make_c2(sample, seed=2)
    nodes, params, obs = wl.pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    pv = np.array([v.value for v in params])
    data = wl.data.to_numpy()
    for _ in range(args.warmup):
        O.nll(nodes, olist, pv, data, brute_force=True)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.nll(nodes, olist, pv, data, brute_force=True)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * sum(times) / len(times)
    value = sample / (ms / 1e3)
    cores = O.num_threads()
    return {
        "metric": METRIC, "value": value, "unit": "event-NLL evals/s", "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample_events": sample, "l2": "n/a (host)"},
        "cpu_baseline": {"value": value, "unit": "event-NLL evals/s", "cores": cores, "kind": "port",
                         "sample": f"{sample} events of the 2e6-event workload, one NLL per step "
                                   "(FP64 restatement of the reference OMP path, brute-force convolution)"},
        "e2e": {"value": value, "unit": "event-NLL evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def cpu_baseline(sample: int, reps: int = 2) -> dict:
    import numpy as np

    from goofit_gb300 import workloads as W
    from oracle import oracle as O
    wl = W.make_c2(sample, seed=2)
    nodes, params, obs = wl.pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    pv = np.array([v.value for v in params])
    data = wl.data.to_numpy()
    O.nll(nodes, olist, pv, data, brute_force=True)
    t0 = time.perf_counter()
    for _ in range(reps):
        O.nll(nodes, olist, pv, data, brute_force=True)
    dt = (time.perf_counter() - t0) / reps
    return {"value": sample / dt, "unit": "event-NLL evals/s", "cores": O.num_threads(), "kind": "port",
            "sample": f"{sample} events, {reps} NLL evaluations (FP64 restatement of the reference OMP path, "
                      "brute-force convolution per event)"}


def fit_report(wl, nodes, olist, params, free, norm=None, tolerance: float = 0.01) -> dict:
    """MIGRAD on the workload three ways (mixed + analytic, FP64 + analytic, FP64 + numerical gradient) at
    the given tolerance, then the parity of the mixed fit against the FP64 fit and the FP64 oracle (the
    oracle as checker, after the timed fits)."""
    import numpy as np

    import goofit_gb300 as gf
    from oracle import oracle as O

    fits, cov = {}, None
    for label, prec, grad in (("mixed_analytic", "mixed", "analytic"), ("fp64_analytic", "fp64", "analytic"),
                              ("fp64_numerical", "fp64", "numerical")):
        # the engine of this precision evaluates once before the timed fit (layout, event-chunk autotuner,
        # captured graphs, amplitude caches: one-time costs of a data set, not of the fit)
        wl.reset()
        eng, _ = wl.pdf._engine_for(wl.data, prec)
        p0 = np.array([v.value for v in params])
        eng.nll(p0)
        eng.nll_grad(p0)
        wl.reset()
        fm = gf.FitManager(wl.pdf, precision=prec, gradient=grad, tolerance=tolerance)
        fm.verbosity = 0
        r = fm.fit()
        fits[label] = {"wall_s": fm.wall_seconds, "nfcn": r.nfcn, "valid": r.valid, "fmin": r.fmin, "edm": r.edm,
                       "values": {params[i].name: params[i].value for i in free},
                       "errors": {params[i].name: params[i].error for i in free}}
        if label == "mixed_analytic":
            cov = fm.covariance
            xm = np.array([v.value for v in params])
    m, a, n = fits["mixed_analytic"], fits["fp64_analytic"], fits["fp64_numerical"]
    fits["tolerance"] = tolerance
    fits["speedup_wall"] = n["wall_s"] / m["wall_s"]
    fits["speedup_wall_precision_only"] = a["wall_s"] / m["wall_s"]
    data = wl.data.to_numpy()
    if norm is not None:
        O.set_amp4_norm_events(norm)
    ref = O.nll(nodes, olist, xm, data)
    off = O.minimum_offset_sigma(nodes, olist, xm, data, cov, free)
    parity = {
        "mixed_vs_fp64_rel_dnll": abs(m["fmin"] - a["fmin"]) / abs(a["fmin"]),
        "mixed_vs_fp64_max_dsigma": max(abs(m["values"][k] - a["values"][k]) / a["errors"][k] for k in m["values"]),
        "oracle_rel_nll": abs(m["fmin"] - ref) / abs(ref),
        "oracle_max_dsigma": float(np.max(off)),
        "oracle": "FP64 CPU restatement of the reference algorithm; distance to its minimum = one Newton step "
                  "with its central-difference gradient and the mixed fit's covariance",
    }
    return {"fit": fits, "parity": parity}


def fcn_wall_us(call, n: int = 50) -> float:
    """Median host wall time of one FCN call (warm, no L2 flush, no clock sampler running)."""
    import numpy as np
    for _ in range(3):
        call()
    t = []
    for _ in range(n):
        t0 = time.perf_counter()
        call()
        t.append(time.perf_counter() - t0)
    return float(np.median(t) * 1e6)


def run_engine(args) -> dict | None:
    import ctypes as C

    import numpy as np
    import torch

    import goofit_gb300 as gf
    from goofit_gb300 import _abi as A
    from goofit_gb300 import workloads as W

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dev = f"cuda:{local}"
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device(dev))

    wl = W.make_c2(N_EVENTS, seed=2 + rank)
    nodes, params, obs = wl.pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    mask = [0 if v.fixed else 1 for v in params]
    pv = np.array([v.value for v in params])
    eng = gf.Engine(args.precision, device=local)
    eng.set_tree(nodes, olist, len(params), mask)
    host = torch.empty((1, N_EVENTS), dtype=torch.float64, pin_memory=True)
    host.numpy()[:] = wl.data.to_numpy()
    hp = C.cast(host.data_ptr(), C.POINTER(C.c_double))
    L = A.lib()
    A.check(L.gf_upload_events(eng._h, 0, hp, N_EVENTS), eng._h)
    eng._n_events[0] = N_EVENTS
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step():
        return eng.nll_grad(pv)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    def timed(sampler: bool):
        dev_ms = []
        clk = ClockSampler(local) if sampler else None
        if clk:
            clk.__enter__()
        try:
            if world > 1:
                import torch.distributed as dist
                dist.barrier()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                flush.zero_()
                torch.cuda.synchronize()
                step()
                dev_ms.append(eng.last_timing()[0])
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
        finally:
            if clk:
                clk.__exit__(None, None, None)
        return dev_ms, wall, clk

    dev_ms, wall, clk = timed(True)
    ms = float(np.mean(dev_ms))
    ms = barrier_max(ms, world, dev)
    value = world * N_EVENTS / (ms / 1e3)
    # the same loop without the nvidia-smi sampler, and the FCN call alone (host wall, warm)
    _, wall_nosampler, _ = timed(False)
    fcn_us = fcn_wall_us(step)

    launches = eng.launches_per_eval(True)
    one_launch = launches == 1
    # the three-launch chain's kernels, each launched alone (CUDA events on the engine's stream, L2 flushed)
    kt = []
    for _ in range(max(args.steps, 5)):
        flush.zero_()
        torch.cuda.synchronize()
        kt.append(eng.time_kernels(True))
    kt = np.mean(np.array(kt), axis=0)

    # end to end through the C ABI with host buffers
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        A.check(L.gf_upload_events(eng._h, 0, hp, N_EVENTS), eng._h)
        eng.nll_grad(pv)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            e2e_ms.append(1e3 * dt)
    e2e = barrier_max(float(np.mean(e2e_ms)), world, dev)

    # roofline of the dominant kernel.  One launch per FCN (gf_fcn_g): the whole step is that kernel, timed
    # by the CUDA events around it; three launches: the event kernel launched alone.  Algorithmic bytes = the
    # int32 bin offset of every event (the flat polynomial needs no x; the convolution needs x only through
    # its bin offset); the tables stay on chip.
    bytes_per_event = 4
    kern_ms = ms if one_launch else float(kt[2])
    peaks = load_peaks()
    achieved = N_EVENTS * bytes_per_event / (kern_ms / 1e3) / 1e9
    traffic = FCN_DRAM_BYTES if one_launch else EVT_DRAM_BYTES_PER_LAUNCH * N_EVENTS / EVT_DRAM_EVENTS
    traffic_src = (FCN_DRAM_SOURCE if one_launch else
                   "ncu dram__bytes_read.sum + dram__bytes_write.sum, profiles/gf_evt_g_c2_composite_2e6.md")

    rep = {}
    if rank == 0 and not args.no_fit:
        free = [i for i, m in enumerate(mask) if m]
        rep = fit_report(wl, nodes, olist, params, free, tolerance=args.fit_tolerance)

    if rank != 0:
        return None
    cpu = cpu_baseline(args.cpu_sample) if not args.no_cpu else None
    line = {
        "metric": METRIC, "value": value, "unit": "event-NLL evals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32-events/f64-reductions" if args.precision == "mixed" else "f64",
        "data": "synthetic (seeded accept-reject on the model density)",
        "config": {"workload": WORKLOAD, "events": N_EVENTS, "precision": args.precision,
                   "step": "one FCN call: NLL + analytic gradient (4 floated parameters)",
                   "kernels_per_step": launches,
                   "l2": "flushed (256 MB write) before every timed step",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "event_chunk": eng.event_chunk(), "event_chunk_autotuned": os.environ.get("GF_AUTOTUNE", "1") != "0"},
        "e2e": {"value": world * N_EVENTS / (e2e / 1e3), "unit": "event-NLL evals/s",
                "h2d_bytes_per_step": N_EVENTS * 8 + len(params) * 8, "d2h_bytes_per_step": (2 + eng.n_grad) * 8,
                "ms_per_step": e2e},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "traffic": traffic, "traffic_source": traffic_src,
                     "kernel": "gf_fcn_g" if one_launch else "gf_evt_g",
                     "kernel_ms": kern_ms, "bytes_per_event": bytes_per_event, "peak_source": peaks["src"],
                     "three_launch_kernels_alone_ms": {"gf_conv_g": float(kt[0]), "gf_grid_g": float(kt[1]),
                                                       "gf_evt_g": float(kt[2])}},
        "cpu_baseline": cpu,
        "gpu_launches": launches * args.steps,
        "clocks": clk.summary(),
        "wall_ms_per_step": 1e3 * wall / args.steps,
        "wall_ms_per_step_without_clock_sampler": 1e3 * wall_nosampler / args.steps,
        "fcn_wall_us": fcn_us,
        "wall_note": "wall_ms_per_step is the host time of the timed loop per step: the 256 MB L2 flush, two "
                     "device synchronisations and the FCN call, with nvidia-smi sampling clocks alongside; "
                     "fcn_wall_us is one FCN call alone (host wall, warm)",
    }
    line.update(rep)
    return line


def run_toys(args) -> dict:
    """C4: lockstep MIGRAD fits of n toys of the composite model, one batched graph launch per round."""
    import ctypes as C

    import numpy as np
    import torch

    import goofit_gb300 as gf
    from goofit_gb300 import _abi as A
    from goofit_gb300 import workloads as W
    from oracle import oracle as O

    torch.cuda.set_device(0)
    study = W.make_c4(n_toys=args.toys, seed=4)
    nodes, params, obs = study.pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    mask = [0 if v.fixed else 1 for v in params]
    names = [v.name for v in params]
    x0 = np.array([study.start.get(v.name, v.value) for v in params])
    err = np.array([v.error for v in params])
    lo = np.array([v.lowerlimit for v in params])
    hi = np.array([v.upperlimit for v in params])
    fixed = np.array([1 if v.fixed else 0 for v in params], np.int32)
    limited = np.array([0 if v.fixed else 1 for v in params], np.int32)
    free = [i for i in range(len(params)) if not fixed[i]]
    counts = [int(d.shape[1]) for d in study.datas]
    n_events = int(sum(counts))
    tol = args.fit_tolerance
    # the toys' FP64 events in one page-locked host block (the e2e leg uploads them from there every step)
    host = torch.empty(n_events, dtype=torch.float64, pin_memory=True)
    off = np.cumsum([0] + counts)
    for t, d in enumerate(study.datas):
        host.numpy()[off[t]:off[t + 1]] = d[0]
    base = host.data_ptr()
    L = A.lib()
    out = {"metric": METRIC, "config": {"workload": f"c4: {args.toys} toys of the composite model, Poisson(20000) "
                                                    "events clipped to [5000, 60000], +-10% jittered truths",
                                        "events_total": n_events}}
    res_by = {}
    clk = None
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda:0")
    for label, prec, grad in (("mixed_analytic", "mixed", True), ("fp64_analytic", "fp64", True),
                              ("fp64_numerical", "fp64", False)):
        eng = gf.Engine(prec)
        eng.set_tree(nodes, olist, len(params), mask)
        eng.set_num_toys(args.toys)
        for t in range(args.toys):
            A.check(L.gf_upload_events(eng._h, t, C.cast(base + 8 * int(off[t]), C.POINTER(C.c_double)), counts[t]),
                    eng._h)
            eng._n_events[t] = counts[t]
        P = np.tile(x0, (args.toys, 1))
        eng.nll_batch(P, grad=True)
        # launch shapes (table k-tiles; the event chunk is tuned at the first evaluation), once per process
        t_tune = time.perf_counter()
        shapes = eng.tune_shapes()
        tune_s = time.perf_counter() - t_tune
        for _ in range(3):
            eng.nll_batch(P, grad=True)
        shapes["event_chunk"] = eng.event_chunk()
        torch.cuda.synchronize()
        rt = []
        for _ in range(10):
            flush.zero_()
            torch.cuda.synchronize()
            eng.nll_batch(P, grad=True)
            rt.append(eng.last_timing()[0])
        rtw = []
        for _ in range(10):
            eng.nll_batch(P, grad=True)
            rtw.append(eng.last_timing()[0])
        X0 = np.tile(x0, (args.toys, 1))
        if label == "mixed_analytic":
            clk = ClockSampler(0)
            clk.__enter__()
        t0 = time.perf_counter()
        res = eng.fit_batch(X0, err, lo, hi, limited, fixed, tolerance=tol, use_grad=grad)
        wall = time.perf_counter() - t0
        if label == "mixed_analytic":
            clk.__exit__(None, None, None)
            kt = []
            for _ in range(5):
                flush.zero_()
                torch.cuda.synchronize()
                kt.append(eng.time_kernels(True, -1))
            kt = np.mean(np.array(kt), axis=0)
            launches_round = eng.launches_per_eval(True)
            # end to end through the C ABI: every toy's events uploaded from page-locked host memory, then the
            # whole lockstep fit; the fitted values and errors are read back
            e2e_s = []
            for _ in range(2):
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                for t in range(args.toys):
                    A.check(L.gf_upload_events(eng._h, t, C.cast(base + 8 * int(off[t]), C.POINTER(C.c_double)),
                                               counts[t]), eng._h)
                eng.fit_batch(X0, err, lo, hi, limited, fixed, tolerance=tol, use_grad=grad)
                e2e_s.append(time.perf_counter() - t1)
        vals = np.array([r.values for r in res])
        errs = np.array([r.errors for r in res])
        pulls = {}
        for i in free:
            truth = np.array([tr[names[i]] for tr in study.truths])
            pl = (vals[:, i] - truth) / np.where(errs[:, i] > 0, errs[:, i], np.nan)
            pulls[names[i]] = {"mean": float(np.nanmean(pl)), "std": float(np.nanstd(pl))}
        out[label] = {"fit_wall_s": wall, "fits_per_s": args.toys / wall,
                      "valid": int(sum(r.valid for r in res)), "mean_nfcn": float(np.mean([r.nfcn for r in res])),
                      "max_nfcn": int(max(r.nfcn for r in res)),
                      "invalid_reasons": {"call_limit": int(sum(r.call_limit for r in res)),
                                          "above_max_edm": int(sum(r.above_max_edm for r in res)),
                                          "no_covariance": int(sum(not r.has_covariance for r in res))},
                      "round_ms_with_grad": float(np.mean(rt)),
                      "event_nll_evals_per_s": n_events / (np.mean(rt) / 1e3), "pulls": pulls,
                      "shapes": shapes, "shape_tuning_s": tune_s,
                      "round_ms_with_grad_warm_l2": float(np.mean(rtw))}
        if label == "mixed_analytic":
            # per lockstep round of the fit (one batched evaluation; rounds = the most FCNs of any toy): wall
            # time, and the part of it beyond a gradient round's device time (host MIGRAD steps, launch,
            # synchronisation; a lower bound, value-only rounds being shorter) - what keeping the whole fit in
            # one persistent launch could remove
            rounds = int(max(r.nfcn for r in res))
            out[label].update({"rounds": rounds, "round_wall_ms": 1e3 * wall / rounds,
                               "round_host_and_launch_ms": 1e3 * wall / rounds - float(np.mean(rtw))})
        res_by[label] = res
        eng.close()
    m = out["mixed_analytic"]
    rm, ra = res_by["mixed_analytic"], res_by["fp64_analytic"]
    dsig = max(abs(a.values[i] - b.values[i]) / b.errors[i] for a, b in zip(rm, ra) for i in free)
    # the oracle as checker (after the timed fits): NLL at the fitted minima and distance to the oracle's own
    # minima for a sample of toys
    sample = list(range(0, args.toys, max(1, args.toys // 16)))
    orel, ooff = 0.0, 0.0
    for t in sample:
        ref = O.nll(nodes, olist, rm[t].values, study.datas[t])
        orel = max(orel, abs(rm[t].fmin - ref) / abs(ref))
        ooff = max(ooff, float(np.max(O.minimum_offset_sigma(nodes, olist, rm[t].values, study.datas[t],
                                                              rm[t].covariance, free, h=1e-6))))
    out["parity"] = {"mixed_vs_fp64_max_dsigma": dsig, "toys_compared": args.toys,
                     "oracle_rel_nll": orel, "oracle_max_dsigma": ooff, "oracle_toys": len(sample)}
    out["speedup_wall"] = out["fp64_numerical"]["fit_wall_s"] / m["fit_wall_s"]
    out["speedup_wall_precision_only"] = out["fp64_analytic"]["fit_wall_s"] / m["fit_wall_s"]
    # CPU baseline: MIGRAD fits of a few toys with the oracle NLL (numerical gradient) on the host cores
    cpu = None
    if not args.no_cpu:
        t0 = time.perf_counter()
        nfit = 4
        for t in range(nfit):
            mz = gf.Minimizer(x0, err, lo, hi, limited, fixed, tolerance=tol)
            mz.minimize(lambda p, d=study.datas[t]: O.nll(nodes, olist, p, d))
        dt = time.perf_counter() - t0
        cpu = {"value": nfit / dt, "unit": "fits/s", "cores": O.num_threads(), "kind": "port",
               "sample": f"{nfit} toys fitted with MIGRAD (numerical gradient) on the FP64 restatement"}
    # roofline of the event kernel (batch shape) over all toys: 4 bytes (bin offset) per event; the table
    # kernel, issue-bound on FP32 arithmetic, is reported beside it as a share of the round
    peaks = load_peaks()
    evt_ms = float(kt[2])
    achieved = n_events * 4 / (evt_ms / 1e3) / 1e9
    rounds = int(max(r.nfcn for r in rm))
    out.update({"value": m["fits_per_s"], "unit": "fits/s", "n_gpus": 1, "steps": args.toys, "warmup": 3,
                "ms_per_step": 1e3 * m["fit_wall_s"] / args.toys, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32-events/f64-reductions",
                "data": "synthetic (seeded accept-reject per toy)",
                "e2e": {"value": args.toys / float(np.mean(e2e_s)), "unit": "fits/s",
                        "h2d_bytes_per_step": n_events * 8 // args.toys,
                        "d2h_bytes_per_step": 2 * len(params) * 8,
                        "note": "a step is one toy's fit; every toy's FP64 events are uploaded from page-locked "
                                "host memory before the lockstep fit, inside the timed region"},
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                             "frac": achieved / peaks["hbm_gbs"], "traffic": None, "kernel": "gf_evt_g (batch)",
                             "kernel_ms": evt_ms, "bytes_per_event": 4, "peak_source": peaks["src"],
                             "round_kernels_alone_ms": {"gf_conv_g": float(kt[0]), "gf_grid_g": float(kt[1]),
                                                        "gf_evt_g": evt_ms},
                             "note": "the convolution-table kernel dominates the round; it is bound by the issue "
                                     "rate of its FP32 products and two-sum corrections, not by HBM"},
                "cpu_baseline": cpu,
                "gpu_launches": rounds * launches_round,
                "clocks": clk.summary() if clk else None})
    out["config"].update({"toys": args.toys, "precision": "mixed", "step": "one toy's MIGRAD fit (lockstep)",
                          "tuned_shapes": m["shapes"],
                          "fit_tolerance": tol, "parallelism": "single GPU",
                          "l2": "flushed before each timed round of round_ms_with_grad; the fits run back to back"})
    return out


def run_dalitz(args) -> dict:
    """C3: Amp3Body with 8 RBW resonances, 5e5 events, 1500 x 1500 normalisation bins; C5: Amp4Body with 6
    decay chains, 3e5 events, 2e6 normalisation events.  A step is one FCN (NLL + analytic gradient of the
    floated amplitude coefficients) with the amplitude caches and the integrals built (resonance / line-shape
    parameters fixed, as in the reference's amplitude fits); the one-time cache and integral build is timed
    separately."""
    import ctypes as C

    import numpy as np
    import torch

    import goofit_gb300 as gf
    from goofit_gb300 import _abi as A
    from goofit_gb300 import workloads as W

    torch.cuda.set_device(0)
    c5 = args.config == "c5"
    n = args.events or (300_000 if c5 else 500_000)
    t0 = time.perf_counter()
    wl = W.make_c5(n, 2_000_000, seed=5) if c5 else W.make_c3(n, seed=3)
    gen_s = time.perf_counter() - t0
    nodes, params, obs = wl.pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    nd = wl.pdf._nondiff_all()
    mask = [0 if (v.fixed or id(v) in nd) else 1 for v in params]
    names = [v.name for v in params]
    pv = np.array([v.value for v in params])
    cols = wl.data.to_numpy()
    eng = gf.Engine(args.precision)
    eng.set_tree(nodes, olist, len(params), mask)
    for i, p in enumerate(wl.pdf._flat_order):
        p._engine_setup(eng, i)
    host = torch.empty(cols.shape, dtype=torch.float64, pin_memory=True)
    host.numpy()[:] = cols
    hp = C.cast(host.data_ptr(), C.POINTER(C.c_double))
    L = A.lib()
    A.check(L.gf_upload_events(eng._h, 0, hp, n), eng._h)
    eng._n_events[0] = n
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda:0")

    # one-time build of the amplitude cache and the integrals (a resonance parameter changes)
    im = names.index("rho_mass" if c5 else "rho770_mass")
    build_ms = []
    for k in range(4):
        p = pv.copy()
        p[im] *= 1 + 1e-6 * (k + 1)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        eng.nll(p)
        build_ms.append(1e3 * (time.perf_counter() - t1))
    eng.nll(pv)

    for _ in range(args.warmup):
        eng.nll_grad(pv)
    torch.cuda.synchronize()
    dev_ms = []
    with ClockSampler(0) as clk:
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            eng.nll_grad(pv)
            dev_ms.append(eng.last_timing()[0])
        torch.cuda.synchronize()
        wall = time.perf_counter() - t1
    ms = float(np.mean(dev_ms))
    kt = []
    for _ in range(max(args.steps, 5)):
        flush.zero_()
        torch.cuda.synchronize()
        kt.append(eng.time_kernels(True))
    evt = float(np.mean(np.array(kt), axis=0)[2])
    # end to end through the C ABI with host buffers: upload (the cache rebuild follows) + one FCN
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        A.check(L.gf_upload_events(eng._h, 0, hp, n), eng._h)
        eng.nll_grad(pv)
        if i >= args.warmup:
            e2e_ms.append(1e3 * (time.perf_counter() - t1))
    e2e = float(np.mean(e2e_ms))

    # algorithmic bytes of the event pass: one complex amplitude per resonance / amplitude and event (R2)
    rbytes = 4 if args.precision == "mixed" else 8
    n_amp = 6 if c5 else 8
    bytes_per_event = n_amp * 2 * rbytes
    peaks = load_peaks()
    # one launch per FCN (gf_fcn_g): the step is that kernel; else the event kernel launched alone
    one_launch = eng.launches_per_eval(True) == 1
    kern = "gf_fcn_g" if one_launch else "gf_evt_g"
    kern_ms = ms if one_launch else evt
    achieved = n * bytes_per_event / (kern_ms / 1e3) / 1e9

    rep = {}
    if not args.no_fit:
        free = [i for i, m in enumerate(mask) if m]
        rep = fit_report(wl, nodes, olist, params, free, wl.pdf.norm_events if c5 else None, args.fit_tolerance)
    if c5 and not args.no_modes:
        rep["lineshapes_floated"] = c5_lineshape_modes(args, cols, max(args.steps, 5))
    cpu = None
    if not args.no_cpu:
        from oracle import oracle as O
        sample = min(n, 100_000)
        if c5:
            O.set_amp4_norm_events(wl.pdf.norm_events)
        O.nll(nodes, olist, pv, cols[:, :sample])
        t1 = time.perf_counter()
        O.nll(nodes, olist, pv, cols[:, :sample])
        dt = time.perf_counter() - t1
        # the restatement recomputes the normalisation integrals on every call; the reference caches them
        # while the resonance parameters stay put (Amp3Body.cu:263-330, Amp4Body.cu:405-418), so their time
        # is taken out of the per-FCN cost
        t1 = time.perf_counter()
        if c5:
            O.amp4_gram(nodes, olist, pv, 0, 6)
        else:
            O.amp3_integrals(nodes, olist, pv, 0, 8)
        dti = time.perf_counter() - t1
        integ = "the 2e6-event normalisation sums" if c5 else "the 1500 x 1500 integrals"
        cpu = {"value": sample / max(dt - dti, 1e-9), "unit": "event-NLL evals/s", "cores": O.num_threads(),
               "kind": "port",
               "sample": f"{sample} events, one NLL (FP64 restatement: amplitudes per event), minus the time of "
                         f"{integ} ({dti:.3f} s of {dt:.3f} s), which the reference caches between FCNs"}
    return {
        "metric": METRIC, "value": n / (ms / 1e3), "unit": "event-NLL evals/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32-events/f64-reductions" if args.precision == "mixed" else "f64",
        "data": f"synthetic (accept-reject on the model density, generated in {gen_s:.1f} s)",
        "config": {"workload": ("c5: Amp4Body 1.865 -> pi+ pi- K- pi+, 6 decay chains (BW/SBW), seeded coefficients, "
                                "2e6 flat phase-space normalisation events") if c5 else
                               ("c3: Amp3Body 1.865 -> 0.4937 + 0.13957 + 0.13498 GeV, 8 RBW, seeded coefficients, "
                                "1500x1500 normalisation bins"),
                   "events": n, "precision": args.precision,
                   "step": f"one FCN: NLL + analytic gradient of {int(sum(mask))} amplitude components, caches built",
                   "l2": "flushed (256 MB write) before every timed step", "parallelism": "single GPU",
                   "event_chunk": eng.event_chunk(), "event_chunk_autotuned": os.environ.get("GF_AUTOTUNE", "1") != "0"},
        "e2e": {"value": n / (e2e / 1e3), "unit": "event-NLL evals/s", "h2d_bytes_per_step": int(cols.nbytes),
                "d2h_bytes_per_step": (2 + eng.n_grad) * 8, "ms_per_step": e2e,
                "note": "includes the upload and the per-event amplitude columns it invalidates (the integrals "
                        "depend on parameters only and stay cached)"},
        "cache_and_integral_build_ms": float(np.median(build_ms)),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"],
                     "traffic": EVT_DRAM_BYTES_AMP[args.config][0] * n / EVT_DRAM_BYTES_AMP[args.config][1],
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, "
                                       "profiles/gf_evt_g_amp3_amp4_c3_c5.md (event pass of the same bytes)",
                     "kernel": kern, "kernel_ms": kern_ms, "event_kernel_alone_ms": evt,
                     "bytes_per_event": bytes_per_event, "peak_source": peaks["src"]},
        "cpu_baseline": cpu,
        "gpu_launches": eng.launches_per_eval(True) * args.steps,
        "clocks": clk.summary(),
        "wall_ms_per_step": 1e3 * wall / args.steps,
        **rep,
    }


def c5_lineshape_modes(args, cols, steps: int) -> dict:
    """C5 with the ten line-shape masses and widths floated (20 free parameters), in the two amplitude modes:
    'store' keeps dA/dt per event and per normalisation point, 'recompute' recomputes them in the gradient
    pass and in the integrals.  Per mode: one FCN (NLL + gradient) with the caches valid (device time, L2
    flushed), one FCN after a line-shape change (wall time: value columns and integrals rebuilt, then the
    FCN), and the device bytes the store mode keeps; and the largest gradient difference between the modes."""
    import numpy as np
    import torch

    import goofit_gb300 as gf
    from goofit_gb300 import workloads as W

    pdf = W.c5_model(2_000_000, float_lineshapes=True)[0]
    nodes, params, obs = pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    nd = pdf._nondiff_all()
    mask = [0 if (v.fixed or id(v) in nd) else 1 for v in params]
    names = [v.name for v in params]
    pv = np.array([v.value for v in params])
    im = names.index("rho_mass")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda:0")
    out, grads = {}, {}
    for mode in ("store", "recompute"):
        eng = gf.Engine(args.precision)
        eng.set_amp_mode(mode)
        eng.set_tree(nodes, olist, len(params), mask)
        eng.set_norm_events(0, pdf.norm_events)
        eng.upload(cols)
        for _ in range(max(3, args.warmup)):
            eng.nll_grad(pv)
        dev = []
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            eng.nll_grad(pv)
            dev.append(eng.last_timing()[0])
        reb = []
        for k in range(steps):
            p = pv.copy()
            p[im] *= 1 + 1e-6 * (k + 1)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            eng.nll_grad(p)
            reb.append(1e3 * (time.perf_counter() - t1))
        grads[mode] = eng.nll_grad(pv)[1]
        out[mode] = {"fcn_ms": float(np.mean(dev)), "fcn_after_lineshape_change_ms": float(np.median(reb)),
                     "recomputing": eng.amp_recomputing(),
                     "store_mode_bytes": eng.amp_store_bytes() if mode == "store" else 0}
        eng.close()
    gs, gr = grads["store"], grads["recompute"]
    out["grad_max_rel_diff"] = float(np.abs(gs - gr).max() / np.abs(gs).max())
    out["free_parameters"] = int(sum(mask))
    return out


def run_c1(args) -> dict:
    """C1: ExpPdf(x; alpha) on x in [0, 10], 1e5 events drawn from exp(-0.7 x), analytic normalisation, MIGRAD
    from alpha = -0.3.  A step is one FCN (NLL + dNLL/dalpha); the fits are compared with an FP64 oracle fit
    (MIGRAD on the restatement's NLL, numerical gradient), as the reference's test_exp.py compares alpha and
    its error."""
    import ctypes as C

    import numpy as np
    import torch

    import goofit_gb300 as gf
    from goofit_gb300 import _abi as A
    from goofit_gb300 import workloads as W
    from oracle import oracle as O

    torch.cuda.set_device(0)
    n = args.events or 100_000
    wl = W.make_c1(n, seed=1)
    nodes, params, obs = wl.pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    pv = np.array([v.value for v in params])
    eng = gf.Engine(args.precision)
    eng.set_tree(nodes, olist, len(params), [1])
    host = torch.empty((1, n), dtype=torch.float64, pin_memory=True)
    host.numpy()[:] = wl.data.to_numpy()
    hp = C.cast(host.data_ptr(), C.POINTER(C.c_double))
    L = A.lib()
    A.check(L.gf_upload_events(eng._h, 0, hp, n), eng._h)
    eng._n_events[0] = n
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda:0")
    for _ in range(args.warmup):
        eng.nll_grad(pv)
    torch.cuda.synchronize()
    dev_ms = []
    with ClockSampler(0) as clk:
        torch.cuda.synchronize()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            eng.nll_grad(pv)
            dev_ms.append(eng.last_timing()[0])
        torch.cuda.synchronize()
    ms = float(np.mean(dev_ms))
    fcn_us = fcn_wall_us(lambda: eng.nll_grad(pv))
    kt = []
    for _ in range(max(args.steps, 5)):
        flush.zero_()
        torch.cuda.synchronize()
        kt.append(eng.time_kernels(True))
    evt = float(np.mean(np.array(kt), axis=0)[2])
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        A.check(L.gf_upload_events(eng._h, 0, hp, n), eng._h)
        eng.nll_grad(pv)
        if i >= args.warmup:
            e2e_ms.append(1e3 * (time.perf_counter() - t1))
    e2e = float(np.mean(e2e_ms))
    bpe = 4 if args.precision == "mixed" else 8
    peaks = load_peaks()
    achieved = n * bpe / (evt / 1e3) / 1e9
    rep = {}
    if not args.no_fit:
        rep = fit_report(wl, nodes, olist, params, [0], tolerance=args.fit_tolerance)
        # the reference scenario's FP64 fit on the host: MIGRAD over the restatement's NLL
        data = wl.data.to_numpy()
        t1 = time.perf_counter()
        mz = gf.Minimizer([-0.3], [0.1], [-10.0], [10.0], np.array([1], np.int32), np.array([0], np.int32),
                          tolerance=args.fit_tolerance)
        ro = mz.minimize(lambda p: O.nll(nodes, olist, p, data))
        wall_o = time.perf_counter() - t1
        m = rep["fit"]["mixed_analytic"]
        rep["oracle_fit"] = {"alpha": float(ro.values[0]), "error": float(ro.errors[0]), "nfcn": ro.nfcn,
                             "wall_s": wall_o, "valid": ro.valid,
                             "mixed_dsigma": abs(m["values"]["alpha"] - ro.values[0]) / ro.errors[0],
                             "mixed_rel_error_diff": abs(m["errors"]["alpha"] - ro.errors[0]) / ro.errors[0]}
    cpu = None
    if not args.no_cpu:
        data = wl.data.to_numpy()
        O.nll(nodes, olist, pv, data)
        t1 = time.perf_counter()
        reps = 20
        for _ in range(reps):
            O.nll(nodes, olist, pv, data)
        dt = (time.perf_counter() - t1) / reps
        cpu = {"value": n / dt, "unit": "event-NLL evals/s", "cores": O.num_threads(), "kind": "port",
               "sample": f"all {n} events, {reps} NLL evaluations (FP64 restatement)"}
    line = {
        "metric": METRIC, "value": n / (ms / 1e3), "unit": "event-NLL evals/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32-events/f64-reductions" if args.precision == "mixed" else "f64",
        "data": "synthetic (inverse-CDF draws from exp(-0.7 x) on [0, 10])",
        "config": {"workload": f"c1: ExpPdf(x; alpha), x in [0, 10], {n} events, analytic normalisation",
                   "events": n, "precision": args.precision, "step": "one FCN: NLL + dNLL/dalpha",
                   "l2": "flushed (256 MB write) before every timed step", "parallelism": "single GPU"},
        "e2e": {"value": n / (e2e / 1e3), "unit": "event-NLL evals/s", "h2d_bytes_per_step": n * 8 + 8,
                "d2h_bytes_per_step": 4 * 8, "ms_per_step": e2e},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "traffic": None, "kernel": "gf_evt_g", "kernel_ms": evt,
                     "bytes_per_event": bpe, "peak_source": peaks["src"]},
        "cpu_baseline": cpu,
        "gpu_launches": eng.launches_per_eval(True) * args.steps,
        "clocks": clk.summary(),
        "fcn_wall_us": fcn_us,
    }
    line.update(rep)
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--cpu-sample", type=int, default=200_000)
    ap.add_argument("--ref-sample", type=int, default=100_000)
    ap.add_argument("--no-fit", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c3", "c4", "c5"])
    ap.add_argument("--no-modes", action="store_true",
                    help="c5: skip the floated-line-shape FCNs in the store and recompute amplitude modes")
    ap.add_argument("--fit-tolerance", type=float, default=0.01)
    ap.add_argument("--toys", type=int, default=1024)
    ap.add_argument("--events", type=int, default=0)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_setup()
    if args.config == "c4":
        print(json.dumps(run_toys(args)))
        return
    if args.config == "c1":
        print(json.dumps(run_c1(args)))
        return
    if args.config in ("c3", "c5"):
        print(json.dumps(run_dalitz(args)))
        return
    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference(args)))
        return
    line = run_engine(args)
    if line is not None:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
