"""Seeded synthetic workloads of the benchmark configurations.

No dataset is downloaded: every configuration is generated from a seed with
the shapes and sizes the configuration names.

C1  ExpPdf(x; alpha) on x in [0, 10], x ~ exp(-0.7 x) truncated (inverse CDF), alpha0 = -0.3.
C2  AddPdf(f_sig; ConvolutionPdf(ExpPdf(alpha), GaussianPdf(mu, sigma)), PolynomialPdf(c0)) on x in
    [-5, 10]; tau = 1.5 (alpha = -1/tau), mu = 0, sigma = 0.3, background fraction 0.3; events by
    accept-reject on the model's own density; 10,000-bin numeric normalisation.  The convolution's
    integration constants are (0, 10, 0.01): the exponential is a decay starting at t = 0, smeared by
    the resolution.  (With the default (-10, 10) range the exponential is not truncated inside the
    observable range, so mu and sigma would only rescale the normalisation and be unidentifiable.)
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import api as G


@dataclass
class Workload:
    name: str
    pdf: G.GooPdf
    data: G.UnbinnedDataSet
    truth: dict
    start: dict
    variables: dict = field(default_factory=dict)
    observables: list = field(default_factory=list)

    def reset(self) -> None:
        for k, v in self.start.items():
            self.variables[k].value = v


def c1_data(n: int, seed: int, slope: float = 0.7, lo: float = 0.0, hi: float = 10.0) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    u = rng.random(n)
    return -np.log(1.0 - u * (1.0 - np.exp(-slope * (hi - lo)))) / slope + lo


def make_c1(n: int = 100_000, seed: int = 1) -> Workload:
    x = G.Observable("x", 0.0, 10.0)
    alpha = G.Variable("alpha", -0.3, 0.1, -10.0, 10.0)
    pdf = G.ExpPdf("exppdf", x, alpha)
    data = G.UnbinnedDataSet(x)
    data.from_numpy(c1_data(n, seed).reshape(1, -1))
    pdf.setData(data)
    return Workload("c1-exp-1e5", pdf, data, {"alpha": -0.7}, {"alpha": -0.3}, {"alpha": alpha}, [x])


C2_CONV_RANGE = (0.0, 10.0, 0.01)


def _conv_table(alpha, mu, sigma, lo=C2_CONV_RANGE[0], hi=C2_CONV_RANGE[1], step=C2_CONV_RANGE[2], xlo=-5.0,
                xhi=10.0):
    """FP64 restatement of the ConvolutionPdf value per bin offset, for generating events only."""
    nM = int(np.floor((hi - lo) / step + 0.5))
    ic3, ic4 = lo - xhi, hi - xlo
    nR = int(np.floor((ic4 - ic3) / step + 0.5))
    tm = (hi - lo) / nM * (np.arange(nM) + 0.5) + lo
    tr = (ic4 - ic3) / nR * (np.arange(nR) + 0.5) + ic3
    M = np.exp(alpha * tm)
    R = np.exp(-0.5 * (tr - mu) ** 2 / sigma ** 2)
    off = int(xhi / step)
    lbo = lo / step - np.floor(lo / step)
    kmin = int(np.floor(xlo / step - lbo))
    kmax = int(np.floor(xhi / step - lbo))
    ks = np.arange(kmin, kmax + 1)
    full = np.correlate(R, M, mode="valid")  # full[j] = sum_m M[m] R[m + j]
    T = full[off - ks]
    return ks, T, lbo


def c2_data(n: int, seed: int, alpha=-1 / 1.5, mu=0.0, sigma=0.3, fsig=0.7, xlo=-5.0, xhi=10.0) -> np.ndarray:
    ks, T, lbo = _conv_table(alpha, mu, sigma, xlo=xlo, xhi=xhi)
    step = 0.01
    nb = 10_000
    centres = (xhi - xlo) / nb * (np.arange(nb) + 0.5) + xlo
    kc = np.floor(centres / step - lbo).astype(np.int64)
    Iconv = (xhi - xlo) / nb * T[kc - ks[0]].sum()
    dens = fsig * T / Iconv + (1 - fsig) / (xhi - xlo)
    pmax = dens.max() * 1.001
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    have = 0
    while have < n:
        m = int((n - have) * 1.3 * pmax * (xhi - xlo)) + 1024
        x = rng.uniform(xlo, xhi, m)
        k = np.floor(x / step - lbo).astype(np.int64)
        keep = rng.random(m) * pmax < dens[k - ks[0]]
        out.append(x[keep])
        have += int(keep.sum())
    return np.concatenate(out)[:n]


def make_c2(n: int = 2_000_000, seed: int = 2, truth: dict | None = None) -> Workload:
    tr = dict(alpha=-1 / 1.5, mu=0.0, sigma=0.3, fsig=0.7)
    if truth:
        tr.update(truth)
    x = G.Observable("x", -5.0, 10.0)
    x.setNumBins(10_000)
    alpha = G.Variable("alpha", -0.6, 0.05, -2.0, -0.1)
    mu = G.Variable("mu", 0.05, 0.02, -1.0, 1.0)
    sigma = G.Variable("sigma", 0.35, 0.02, 0.05, 1.0)
    c0 = G.Variable("c0", 1.0)  # a separately normalised flat polynomial's coefficient is degenerate: fixed
    fsig = G.Variable("fsig", 0.65, 0.02, 0.0, 1.0)
    model = G.ExpPdf("model", x, alpha)
    resol = G.GaussianPdf("resolution", x, mu, sigma)
    conv = G.ConvolutionPdf("signal", x, model, resol)
    conv.setIntegrationConstants(*C2_CONV_RANGE)
    bkg = G.PolynomialPdf("background", x, [c0], 0)
    pdf = G.AddPdf("total", fsig, conv, bkg)
    data = G.UnbinnedDataSet(x)
    data.from_numpy(c2_data(n, seed, tr["alpha"], tr["mu"], tr["sigma"], tr["fsig"]).reshape(1, -1))
    pdf.setData(data)
    start = {"alpha": -0.6, "mu": 0.05, "sigma": 0.35, "fsig": 0.65}
    return Workload("c2-conv-2e6", pdf, data, tr, start,
                    {"alpha": alpha, "mu": mu, "sigma": sigma, "c0": c0, "fsig": fsig}, [x])


@dataclass
class ToyStudy:
    name: str
    pdf: G.GooPdf
    variables: dict
    truths: list  # per toy: dict of generation parameters
    datas: list   # per toy: (1, n) float64 arrays
    start: dict


def make_c4(n_toys: int = 1024, mean_events: float = 20_000, lo: int = 5_000, hi: int = 60_000,
            seed: int = 4) -> ToyStudy:
    """C4: toys of the C2 model; Poisson(mean) event counts clipped to [lo, hi]; each toy's generation
    parameters jittered uniformly by +-10% around the C2 truth (mu jittered by +-0.1 sigma_res)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    base = make_c2(16, seed=0)
    counts = np.clip(rng.poisson(mean_events, n_toys), lo, hi)
    truths, datas = [], []
    for t in range(n_toys):
        j = rng.uniform(-0.1, 0.1, 4)
        tr = dict(alpha=(-1 / 1.5) * (1 + j[0]), mu=0.3 * j[1], sigma=0.3 * (1 + j[2]), fsig=0.7 * (1 + j[3]))
        truths.append(tr)
        datas.append(c2_data(int(counts[t]), seed=10_000 + seed * 100_000 + t, alpha=tr["alpha"], mu=tr["mu"],
                             sigma=tr["sigma"], fsig=tr["fsig"]).reshape(1, -1))
    return ToyStudy("c4-toys", base.pdf, base.variables, truths, datas, dict(base.start))
