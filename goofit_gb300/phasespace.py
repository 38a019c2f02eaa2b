"""Flat n-body phase space and the 4-body kinematic variables.

Replaces, for the fit path, the MCBooster pieces the reference calls: `PhaseSpace::Generate` +
`Unweight` (the normalisation events of Amp4Body, src/PDFs/physics/Amp4Body.cu:243-290) and the Dim5
functor (include/goofit/PDFs/physics/detail/Dim5.h:19-111) that turns four daughter 4-vectors into
(m12, m34, cos12, cos34, phi).

Generation: the invariant masses of the nested subsystems (1 2), (1 2 3), ... are drawn uniformly between
their kinematic limits, the event weight is the product of the two-body break-up momenta, and events
are kept with probability weight / max weight (unweighting against the largest weight of the batch, as
MCBooster's Unweight does), which leaves them distributed as flat phase space.  Momenta follow from
isotropic two-body decays in each subsystem rest frame, boosted back to the parent frame.

Vector conventions of Dim5 (MCBooster's Vector4R, from EvtGen): `p * q` is the Minkowski product,
`dot`, `cross` and `d3mag` act on the 3-vector parts.  Arrays hold (px, py, pz, E) in the last axis.
"""
from __future__ import annotations

import numpy as np


def _pdk(a, b, c):
    """Two-body break-up momentum of a -> b c."""
    x = (a - b - c) * (a + b + c) * (a - b + c) * (a + b - c)
    return np.sqrt(np.maximum(x, 0.0)) / (2.0 * a)


def _boost(p, beta):
    """Boost 4-vectors p (..., 4) by velocity beta (..., 3)."""
    b2 = np.sum(beta * beta, axis=-1)
    gamma = 1.0 / np.sqrt(1.0 - b2)
    bp = np.sum(beta * p[..., :3], axis=-1)
    g2 = np.where(b2 > 0, (gamma - 1.0) / np.where(b2 > 0, b2, 1.0), 0.0)
    out = np.empty_like(p)
    out[..., :3] = p[..., :3] + (g2 * bp)[..., None] * beta + (gamma * p[..., 3])[..., None] * beta
    out[..., 3] = gamma * (p[..., 3] + bp)
    return out


def _isotropic(rng, n):
    cost = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2 * np.pi, n)
    sint = np.sqrt(1.0 - cost * cost)
    return np.stack([sint * np.cos(phi), sint * np.sin(phi), cost], axis=-1)


def generate(M: float, masses, n: int, rng: np.random.Generator, batch: int = 1_000_000) -> np.ndarray:
    """n flat phase-space events of M -> masses (the parent at rest): array (n, k, 4)."""
    masses = np.asarray(masses, dtype=np.float64)
    k = len(masses)
    if k < 2 or M <= masses.sum():
        raise ValueError("phase space is empty")
    out, have = [], 0
    tecm = M - masses.sum()
    cum = np.cumsum(masses)
    while have < n:
        m = int(min(batch, max(10_000, 4 * (n - have))))
        r = np.sort(rng.random((m, k - 2)), axis=1) if k > 2 else np.zeros((m, 0))
        # invariant masses of the subsystems (1..j), j = 2..k; the last one is M
        inv = np.empty((m, k))
        inv[:, 0] = masses[0]
        for j in range(1, k - 1):
            inv[:, j] = cum[j] + r[:, j - 1] * tecm
        inv[:, k - 1] = M
        pd = np.empty((m, k - 1))
        for j in range(1, k):
            pd[:, j - 1] = _pdk(inv[:, j], inv[:, j - 1], masses[j])
        w = np.prod(pd, axis=1)
        keep = rng.random(m) * w.max() < w
        inv, pd = inv[keep], pd[keep]
        mk = len(inv)
        if mk == 0:
            continue
        # decay chain from the inside out: subsystem j (mass inv[j]) -> subsystem j-1 + particle j
        p = np.zeros((mk, k, 4))
        d = _isotropic(rng, mk) * pd[:, 0:1]
        p[:, 0, :3] = d
        p[:, 0, 3] = np.sqrt(masses[0] ** 2 + np.sum(d * d, axis=1))
        p[:, 1, :3] = -d
        p[:, 1, 3] = np.sqrt(masses[1] ** 2 + np.sum(d * d, axis=1))
        for j in range(2, k):
            # subsystem (0..j-1) recoils against particle j in the rest frame of subsystem (0..j)
            u = _isotropic(rng, mk) * pd[:, j - 1:j]
            esub = np.sqrt(inv[:, j - 1] ** 2 + np.sum(u * u, axis=1))
            beta = u / esub[:, None]
            p[:, :j] = _boost(p[:, :j], beta[:, None, :])
            p[:, j, :3] = -u
            p[:, j, 3] = np.sqrt(masses[j] ** 2 + np.sum(u * u, axis=1))
        out.append(p)
        have += mk
    return np.concatenate(out)[:n]


# ---- Dim5 ----
def _mdot(a, b):
    return a[..., 3] * b[..., 3] - np.sum(a[..., :3] * b[..., :3], axis=-1)


def _dot3(a, b):
    return np.sum(a[..., :3] * b[..., :3], axis=-1)


def _cross3(a, b):
    c = np.zeros_like(a)
    c[..., :3] = np.cross(a[..., :3], b[..., :3])
    return c


def _d3mag(a):
    return np.sqrt(_dot3(a, a))


def _cos_hel(p, q, d):
    pd, pq, qd = _mdot(p, d), _mdot(p, q), _mdot(q, d)
    mp2, mq2, md2 = _mdot(p, p), _mdot(q, q), _mdot(d, d)
    return (pd * mq2 - pq * qd) / np.sqrt((pq * pq - mq2 * mp2) * (qd * qd - mq2 * md2))


def _phi(d1, d2, h1, h2):
    # the angle between the decay planes (d1, d2) and (h1, h2), signed by the (h1 + h2) direction
    d1n = d1 / _d3mag(d1)[..., None]
    d2n = d2 / _d3mag(d2)[..., None]
    h1n = h1 / _d3mag(h1)[..., None]
    h2n = h2 / _d3mag(h2)[..., None]
    h12 = h1 + h2
    h12n = h12 * (1.0 / _d3mag(h12))[..., None]
    n1 = _cross3(d1n, d2n)
    n2 = _cross3(h1n, h2n)
    n1 = n1 * (1.0 / _d3mag(n1))[..., None]
    n2 = n2 * (1.0 / _d3mag(n2))[..., None]
    n3 = _cross3(n1, n2)
    cp = _dot3(n1, n2)
    sp = _dot3(n3, h12n)
    phi = np.arccos(cp)
    return np.where(sp < 0, -phi, phi)


def dim5(p: np.ndarray) -> np.ndarray:
    """(n, 4, 4) daughter 4-vectors (px, py, pz, E) -> (5, n): m12, m34, cos12, cos34, phi."""
    p0, p1, p2, p3 = p[:, 0], p[:, 1], p[:, 2], p[:, 3]
    pm = p0 + p1 + p2 + p3
    p01 = p0 + p1
    p23 = p2 + p3
    return np.vstack([np.sqrt(_mdot(p01, p01)), np.sqrt(_mdot(p23, p23)), _cos_hel(pm, p01, p0),
                      _cos_hel(pm, p23, p2), _phi(p0, p1, p2, p3)])


def norm_events(M: float, masses, n: int, seed: int) -> np.ndarray:
    """n flat phase-space events of the 4-body decay as the (5, n) Amp4Body variables."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return dim5(generate(M, masses, n, rng))
