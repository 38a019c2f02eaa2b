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
C3  Amp3Body for a 1.865 GeV parent to daughters of 0.4937 (K), 0.13957 (pi) and 0.13498 (pi0) GeV with 8
    relativistic Breit-Wigners (masses/widths 0.775/0.149, 0.892/0.050, 1.414/0.232, 1.425/0.270,
    0.980/0.050, 1.465/0.400, 1.720/0.250, 1.275/0.185; spins 0-2); seeded coefficients with magnitude
    U[0.1, 2] and phase U[0, 2 pi) (the first one fixed: the overall scale and phase are not measurable);
    m12 = m^2(K pi), m13 = m^2(K pi0) on [0, 3] GeV^2 with 1500 x 1500 normalisation bins; constant
    efficiency; 5e5 events by accept-reject on the model density evaluated by the FP64 engine (needs a GPU).
C5  Amp4Body for a 1.865 GeV parent to (pi+, pi-, K-, pi+) with masses (0.13957, 0.13957, 0.4937, 0.13957)
    GeV (the daughter order of the reference's DP4 example); observables (m12, m34, cos12, cos34, phi,
    eventNumber); 6 Bose-symmetrised decay chains with BW/SBW line shapes (masses 0.5-1.5 GeV, widths
    0.05-0.4 GeV): K*rho in S, P and D wave (vector-vector), K1(1270) -> rho K and a1(1260) -> rho pi
    (axial-vector + pseudoscalar), K* f0(500) (vector + scalar); seeded coefficients with magnitude
    U[0.1, 2] and phase U[0, 2 pi) (the first fixed); 2,000,000 flat phase-space normalisation events;
    300,000 events by accept-reject on the model density evaluated by the FP64 engine (needs a GPU).
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


# parent and daughter masses (GeV) and the resonance set of the C3 configuration
C3_M, C3_MK, C3_MPI, C3_MPI0 = 1.865, 0.4937, 0.13957, 0.13498
C3_RESONANCES = [
    # name, mass, width, spin, daughter pair
    ("rho770", 0.775, 0.149, 1, G.PAIR_23),
    ("kst892", 0.892, 0.050, 1, G.PAIR_12),
    ("kst1410", 1.414, 0.232, 1, G.PAIR_13),
    ("k0st1430", 1.425, 0.270, 0, G.PAIR_12),
    ("f0_980", 0.980, 0.050, 0, G.PAIR_23),
    ("rho1450", 1.465, 0.400, 1, G.PAIR_23),
    ("rho1700", 1.720, 0.250, 1, G.PAIR_23),
    ("f2_1270", 1.275, 0.185, 2, G.PAIR_23),
]


def c3_coefficients(n_res: int = 8, seed: int = 3) -> list[complex]:
    rng = np.random.Generator(np.random.PCG64(seed))
    mag = rng.uniform(0.1, 2.0, n_res)
    ph = rng.uniform(0.0, 2 * np.pi, n_res)
    return [complex(m * np.cos(p), m * np.sin(p)) for m, p in zip(mag, ph)]


def c3_model(bins: int = 1500, n_res: int = 8, coef_seed: int = 3):
    """The C3 Amp3Body tree (no data attached); returns (pdf, variables, observables)."""
    m12 = G.Observable("m12", 0.0, 3.0)
    m13 = G.Observable("m13", 0.0, 3.0)
    m12.setNumBins(bins)
    m13.setNumBins(bins)
    evt = G.EventNumber("eventNumber")
    d = G.DecayInfo3()
    d.motherMass, d.daug1Mass, d.daug2Mass, d.daug3Mass = C3_M, C3_MK, C3_MPI, C3_MPI0
    d.meson_radius, d.mother_meson_radius = 1.5, 5.0
    variables = {}
    coefs = c3_coefficients(n_res, coef_seed)
    for k, (name, mass, width, spin, pair) in enumerate(C3_RESONANCES[:n_res]):
        re, im, free = coefs[k].real, coefs[k].imag, k > 0
        if free:
            ar = G.Variable(f"{name}_amp_real", re, 0.001, 0, 0)
            ai = G.Variable(f"{name}_amp_imag", im, 0.001, 0, 0)
            variables[ar.name], variables[ai.name] = ar, ai
        else:
            ar, ai = G.Variable(f"{name}_amp_real", re), G.Variable(f"{name}_amp_imag", im)
        m = G.Variable(f"{name}_mass", mass)
        w = G.Variable(f"{name}_width", width)
        d.add_resonance(G.RBW(name, ar, ai, m, w, spin, int(pair)))
    eff = G.PolynomialPdf("constantEff", [m12, m13], [G.Variable("constantOne", 1)],
                          [G.Variable("constantZero0", 0), G.Variable("constantZero1", 0)], 0)
    pdf = G.Amp3Body("signalPDF", m12, m13, evt, d, eff)
    return pdf, variables, [m12, m13, evt]


def c3_generate(pdf, n: int, seed: int, batch: int = 4_000_000) -> np.ndarray:
    """Accept-reject sample of the Amp3Body density: uniform candidates in the (m12, m13) box, weights from
    the FP64 engine's per-event values.  Returns a (3, n) array [m12, m13, eventNumber]."""
    from .engine import Engine
    from . import _abi as A
    rng = np.random.Generator(np.random.PCG64(seed))
    nodes, params, obs = pdf._flatten()
    eng = Engine("fp64")
    eng.set_tree(nodes, [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs],
                 len(params), [0] * len(params))
    pv = np.array([v.value for v in params])
    lo, hi = obs[0].lowerlimit, obs[0].upperlimit
    out12, out13, vmax, have = [], [], None, 0
    while have < n:
        c = np.empty((3, batch))
        c[0] = rng.uniform(lo, hi, batch)
        c[1] = rng.uniform(obs[1].lowerlimit, obs[1].upperlimit, batch)
        c[2] = np.arange(batch, dtype=np.float64)
        eng.upload(c)
        eng.set_params(pv)
        v = eng.eval_events(A.GF_METRIC_EVAL)
        if vmax is None:
            vmax = 1.2 * float(v.max())
        vmax = max(vmax, float(v.max()))
        keep = rng.random(batch) * vmax < v
        out12.append(c[0][keep])
        out13.append(c[1][keep])
        have += int(keep.sum())
    m12 = np.concatenate(out12)[:n]
    m13 = np.concatenate(out13)[:n]
    return np.vstack([m12, m13, np.arange(n, dtype=np.float64)])


def make_c3(n: int = 500_000, seed: int = 3, bins: int = 1500, n_res: int = 8, data: np.ndarray | None = None) -> Workload:
    pdf, variables, obs = c3_model(bins, n_res)
    truth = {k: v.value for k, v in variables.items()}
    cols = data if data is not None else c3_generate(pdf, n, seed)
    ds = G.UnbinnedDataSet(obs)
    ds.from_numpy(cols)
    pdf.setData(ds)
    # start 5% away from the truth
    start = {k: v * 1.05 for k, v in truth.items()}
    return Workload(f"c3-amp3body-{n}", pdf, ds, truth, start, variables, obs)


C5_M = 1.865
C5_MASSES = [0.13957, 0.13957, 0.4937, 0.13957]


def c5_model(n_norm: int = 2_000_000, coef_seed: int = 5, norm_seed: int = 55, float_lineshapes: bool = False):
    """The C5 Amp4Body tree (no data attached); returns (pdf, variables, observables, lineshape variables)."""
    m12 = G.Observable("m12", 0, 3)
    m34 = G.Observable("m34", 0, 3)
    c12 = G.Observable("cos12", -1, 1)
    c34 = G.Observable("cos34", -1, 1)
    phi = G.Observable("phi", -3.5, 3.5)
    evt = G.EventNumber("eventNumber")
    obs = [m12, m34, c12, c34, phi, evt]
    d = G.DecayInfo4()
    d.particle_masses = [C5_M] + C5_MASSES
    d.meson_radius = 1.5

    def var(name, v):
        return G.Variable(name, v, 0.01 * v, 0.5 * v, 1.5 * v) if float_lineshapes else G.Variable(name, v)

    ls_vars = {k: var(k, v) for k, v in [("rho_mass", 0.775), ("rho_width", 0.149), ("Kst_mass", 0.892),
                                           ("Kst_width", 0.050), ("K1_mass", 1.272), ("K1_width", 0.090),
                                           ("a1_mass", 1.230), ("a1_width", 0.400), ("f0_mass", 0.500),
                                           ("f0_width", 0.400)]}
    V = ls_vars
    RBW, SBW, SF = G.Lineshapes.RBW, G.Lineshapes.SBW, G.SpinFactor
    P = G.DP4Pair

    def krho():
        return [RBW("rho(770)", V["rho_mass"], V["rho_width"], 1, P.M_12),
                RBW("K*(892)", V["Kst_mass"], V["Kst_width"], 1, P.M_34),
                RBW("rho(770)", V["rho_mass"], V["rho_width"], 1, P.M_24),
                RBW("K*(892)", V["Kst_mass"], V["Kst_width"], 1, P.M_13)]

    def sf(kind, a, b):
        return [SF("SF", kind, C5_M, *a), SF("SF", kind, C5_M, *b)]

    S4 = G.SF_4Body
    chains = [
        ("K*rho_S", krho(), sf(S4.DtoV1V2_V1toP1P2_V2toP3P4_S, (0, 1, 2, 3), (3, 1, 2, 0))),
        ("K*rho_P", krho(), sf(S4.DtoV1V2_V1toP1P2_V2toP3P4_P, (0, 1, 2, 3), (3, 1, 2, 0))),
        ("K*rho_D", krho(), sf(S4.DtoV1V2_V1toP1P2_V2toP3P4_D, (0, 1, 2, 3), (3, 1, 2, 0))),
        ("K1rho", [SBW("K1(1270)", V["K1_mass"], V["K1_width"], 0, P.M_12_3),
                   RBW("rho(770)", V["rho_mass"], V["rho_width"], 1, P.M_12),
                   SBW("K1(1270)", V["K1_mass"], V["K1_width"], 0, P.M_24_3),
                   RBW("rho(770)", V["rho_mass"], V["rho_width"], 1, P.M_24)],
         sf(S4.DtoAP1_AtoVP2_VtoP3P4, (3, 2, 0, 1), (0, 2, 3, 1))),
        ("a1rho", [SBW("a1(1260)", V["a1_mass"], V["a1_width"], 0, P.M_12_4),
                   RBW("rho(770)", V["rho_mass"], V["rho_width"], 1, P.M_12),
                   SBW("a1(1260)", V["a1_mass"], V["a1_width"], 0, P.M_24_1),
                   RBW("rho(770)", V["rho_mass"], V["rho_width"], 1, P.M_24)],
         sf(S4.DtoAP1_AtoVP2_VtoP3P4, (2, 3, 0, 1), (2, 0, 3, 1))),
        ("K*f0", [RBW("K*(892)", V["Kst_mass"], V["Kst_width"], 1, P.M_34),
                  RBW("f0(500)", V["f0_mass"], V["f0_width"], 0, P.M_12),
                  RBW("K*(892)", V["Kst_mass"], V["Kst_width"], 1, P.M_13),
                  RBW("f0(500)", V["f0_mass"], V["f0_width"], 0, P.M_24)],
         sf(S4.DtoVS_VtoP1P2_StoP3P4, (2, 3, 0, 1), (2, 0, 3, 1))),
    ]
    rng = np.random.Generator(np.random.PCG64(coef_seed))
    mag = rng.uniform(0.1, 2.0, len(chains))
    ph = rng.uniform(0.0, 2 * np.pi, len(chains))
    variables = {}
    for k, (name, ls, sfs) in enumerate(chains):
        re, im = mag[k] * np.cos(ph[k]), mag[k] * np.sin(ph[k])
        if k == 0:
            ar, ai = G.Variable(f"{name}_re", re), G.Variable(f"{name}_im", im)
        else:
            ar = G.Variable(f"{name}_re", re, 0.01, 0, 0)
            ai = G.Variable(f"{name}_im", im, 0.01, 0, 0)
            variables[ar.name], variables[ai.name] = ar, ai
        d.amplitudes.append(G.Amplitude(name, ar, ai, ls, sfs, 2))
    eff = G.PolynomialPdf("constantEff", [m12, m34], [G.Variable("constantOne", 1)],
                          [G.Variable("constantZero0", 0), G.Variable("constantZero1", 0)], 0)
    pdf = G.Amp4Body("DK3pi", obs, d, eff, n_norm, norm_seed)
    return pdf, variables, obs, ls_vars


def c5_generate(pdf, n: int, seed: int, batch: int = 2_000_000) -> np.ndarray:
    """Accept-reject sample of the Amp4Body density over flat phase space; weights from the FP64 engine's
    per-event values.  Returns a (6, n) array [m12, m34, cos12, cos34, phi, eventNumber]."""
    from . import phasespace
    from .engine import Engine
    from . import _abi as A
    rng = np.random.Generator(np.random.PCG64(seed))
    nodes, params, obs = pdf._flatten()
    eng = Engine("fp64")
    eng.set_tree(nodes, [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs],
                 len(params), [0] * len(params))
    for i, p in enumerate(pdf._flat_order):
        p._engine_setup(eng, i)
    pv = np.array([v.value for v in params])
    masses = pdf.decayInfo.particle_masses
    out, vmax, have = [], None, 0
    while have < n:
        v5 = phasespace.dim5(phasespace.generate(masses[0], masses[1:], batch, rng))
        c = np.vstack([v5, np.arange(batch, dtype=np.float64)])
        eng.upload(c)
        eng.set_params(pv)
        w = eng.eval_events(A.GF_METRIC_EVAL)
        if vmax is None:
            vmax = 1.2 * float(w.max())
        vmax = max(vmax, float(w.max()))
        keep = rng.random(batch) * vmax < w
        out.append(v5[:, keep])
        have += int(keep.sum())
    v = np.concatenate(out, axis=1)[:, :n]
    return np.vstack([v, np.arange(n, dtype=np.float64)])


def make_c5(n: int = 300_000, n_norm: int = 2_000_000, seed: int = 5, data: np.ndarray | None = None,
            float_lineshapes: bool = False) -> Workload:
    pdf, variables, obs, ls_vars = c5_model(n_norm, float_lineshapes=float_lineshapes)
    if float_lineshapes:
        variables.update(ls_vars)
    truth = {k: v.value for k, v in variables.items()}
    cols = data if data is not None else c5_generate(pdf, n, seed)
    ds = G.UnbinnedDataSet(obs)
    ds.from_numpy(cols)
    pdf.setData(ds)
    start = {k: v * 1.05 for k, v in truth.items()}
    return Workload(f"c5-amp4body-{n}", pdf, ds, truth, start, variables, obs)
