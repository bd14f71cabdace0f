"""Seeded synthetic planetary systems of the benchmark configurations.

No public dataset is involved: every configuration is a seeded draw from the
distributions below, built with ElementsIC(t0 = 0, H = N fully nested,
elements), elements rows (m, P, t0_transit, e cos w, e sin w, I, Omega) and a
star row (M*, 0, ..., 0).

  plain_3body   N=3, M*=1, m ~ U(3e-6, 3e-5), P = (10.0, 20.1),
                e ~ U(0, 0.05), w, t0 uniform over the orbit, I = pi/2,
                Omega = 0; h = P1/20 = 0.5, tmax = 1000 -> 2000 steps
  batch_3body   4096 Gaussian perturbations (1e-4 relative on masses,
                periods, e cos w, e sin w, t0) of one plain_3body draw
  batch_8body   1024 x N=8, M*=0.09, m ~ U(1e-6, 1.5e-5),
                P = (1.5, 2.4, 4.0, 6.1, 9.2, 12.4, 18.8)(1 + 1e-3 N(0,1)),
                e ~ U(0, 0.01), I = pi/2; h = 0.06, tmax = 1600
  batch_uneven  N ~ U{2..10}, P log-uniform 1..100 d sorted and
                redrawn until adjacent pairs are separated by more than
                HILL_DELTA mutual Hill radii, m log-uniform 1e-6..1e-4,
                e ~ U(0, 0.1), I = pi/2 + N(0, 0.01), Omega = 0,
                h = min(P)/20, tmax log-uniform 100..4000
"""
import math

import numpy as np

from .ics import ElementsIC

HILL_DELTA = 8.0
GNEWT = 39.4845 / (365.242 * 365.242)


def _ecc_pair(rng, emax, size=None):
    e = rng.uniform(0.0, emax, size)
    e = np.maximum(e, 1e-6)  # the element Jacobian has 1/e terms: keep e > 0
    w = rng.uniform(0.0, 2 * math.pi, size)
    return e * np.cos(w), e * np.sin(w)


def plain_3body(seed=0):
    """One 3-body system near 2:1 resonance.  Returns (elements, h, tmax)."""
    rng = np.random.default_rng(seed)
    el = np.zeros((3, 7))
    el[0, 0] = 1.0
    periods = (10.0, 20.1)
    for q, P in enumerate(periods):
        ec, es = _ecc_pair(rng, 0.05)
        el[q + 1] = [rng.uniform(3e-6, 3e-5), P, rng.uniform(0.0, P), ec, es, math.pi / 2, 0.0]
    return el, 0.5, 1000.0


def batch_3body(nsys=4096, seed=0):
    """nsys perturbations of one plain_3body draw.  Returns (list of elements, h, tmax)."""
    base, h, tmax = plain_3body(seed)
    rng = np.random.default_rng(seed + 1)
    out = []
    for _ in range(nsys):
        el = base.copy()
        for col in (0, 1, 2, 3, 4):  # m, P, t0, ecosw, esinw
            el[1:, col] = base[1:, col] * (1.0 + 1e-4 * rng.standard_normal(2))
        out.append(el)
    return out, h, tmax


def batch_8body(nsys=1024, seed=0):
    """nsys 8-body TRAPPIST-like systems.  Returns (list of elements, h, tmax)."""
    rng = np.random.default_rng(seed + 2)
    P0 = np.array([1.5, 2.4, 4.0, 6.1, 9.2, 12.4, 18.8])
    out = []
    for _ in range(nsys):
        el = np.zeros((8, 7))
        el[0, 0] = 0.09
        P = P0 * (1.0 + 1e-3 * rng.standard_normal(7))
        ec, es = _ecc_pair(rng, 0.01, 7)
        el[1:, 0] = rng.uniform(1e-6, 1.5e-5, 7)
        el[1:, 1] = P
        el[1:, 2] = rng.uniform(0.0, P)
        el[1:, 3] = ec
        el[1:, 4] = es
        el[1:, 5] = math.pi / 2
        out.append(el)
    return out, 0.06, 1600.0


def _hill_ok(P, m, mstar):
    a = np.cbrt(GNEWT * mstar * P * P / (4 * math.pi * math.pi))
    for q in range(len(P) - 1):
        rh = 0.5 * (a[q] + a[q + 1]) * np.cbrt((m[q] + m[q + 1]) / (3.0 * mstar))
        if (a[q + 1] - a[q]) / rh <= HILL_DELTA:
            return False
    return True


def batch_uneven(nsys=2048, seed=0, nmin=2, nmax=10):
    """Mixed body counts and durations.  Returns (list of elements, list of h, list of tmax)."""
    rng = np.random.default_rng(seed + 3)
    els, hs, tmaxs = [], [], []
    for _ in range(nsys):
        n = int(rng.integers(nmin, nmax + 1))
        npl = n - 1
        while True:
            P = np.sort(np.exp(rng.uniform(math.log(1.0), math.log(100.0), npl)))
            m = np.exp(rng.uniform(math.log(1e-6), math.log(1e-4), npl))
            if _hill_ok(P, m, 1.0):
                break
        el = np.zeros((n, 7))
        el[0, 0] = 1.0
        ec, es = _ecc_pair(rng, 0.1, npl)
        el[1:, 0] = m
        el[1:, 1] = P
        el[1:, 2] = rng.uniform(0.0, P)
        el[1:, 3] = ec
        el[1:, 4] = es
        el[1:, 5] = math.pi / 2 + 0.01 * rng.standard_normal(npl)
        els.append(el)
        hs.append(float(P.min() / 20.0))
        tmaxs.append(float(math.exp(rng.uniform(math.log(100.0), math.log(4000.0)))))
    return els, hs, tmaxs


def ic_of(el, t0=0.0):
    return ElementsIC(t0, el.shape[0], el)
