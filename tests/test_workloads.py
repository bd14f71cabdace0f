"""The seeded benchmark workloads: shapes, step counts, determinism and the
stability rule of the uneven batch (CPU only)."""
import math

import numpy as np

from nbg import workloads as W


def steps(h, tmax):
    return int(round(tmax / h))


def test_plain_3body_shape_and_steps():
    el, h, tmax = W.plain_3body(0)
    assert el.shape == (3, 7) and el[0, 0] == 1.0 and np.all(el[0, 1:] == 0.0)
    assert tuple(el[1:, 1]) == (10.0, 20.1)
    assert np.all((el[1:, 0] >= 3e-6) & (el[1:, 0] <= 3e-5))
    e = np.hypot(el[1:, 3], el[1:, 4])
    assert np.all((e > 0.0) & (e <= 0.05))  # e > 0: the element Jacobian has 1/e terms
    assert np.all(el[1:, 5] == math.pi / 2) and np.all(el[1:, 6] == 0.0)
    assert steps(h, tmax) == 2000


def test_batch_3body_is_a_perturbed_copy():
    base, _, _ = W.plain_3body(0)
    els, h, tmax = W.batch_3body(64, seed=0)
    assert len(els) == 64 and steps(h, tmax) == 2000
    for el in els:
        assert el.shape == (3, 7)
        rel = np.abs(el[1:, :5] / base[1:, :5] - 1.0)
        assert np.all(rel < 1e-3) and np.any(rel > 0.0)  # Gaussian 1e-4 perturbations
        assert np.array_equal(el[:, 5:], base[:, 5:]) and np.array_equal(el[0], base[0])


def test_batch_8body_shape_and_steps():
    els, h, tmax = W.batch_8body(16)
    assert steps(h, tmax) == 26667
    P0 = np.array([1.5, 2.4, 4.0, 6.1, 9.2, 12.4, 18.8])
    for el in els:
        assert el.shape == (8, 7) and el[0, 0] == 0.09
        assert np.all(np.abs(el[1:, 1] / P0 - 1.0) < 1e-2)
        assert np.all((el[1:, 0] >= 1e-6) & (el[1:, 0] <= 1.5e-5))
        assert np.all(np.hypot(el[1:, 3], el[1:, 4]) <= 0.01)


def test_batch_uneven_ranges_and_hill_separation():
    els, hs, tmaxs = W.batch_uneven(200, seed=0)
    ns = [el.shape[0] for el in els]
    assert min(ns) >= 2 and max(ns) <= 10 and len(set(ns)) == 9
    for el, h, tmax in zip(els, hs, tmaxs):
        P, m = el[1:, 1], el[1:, 0]
        assert np.all(np.diff(P) > 0.0) and P[0] >= 1.0 and P[-1] <= 100.0
        assert np.all((m >= 1e-6) & (m <= 1e-4))
        assert W._hill_ok(P, m, 1.0)
        assert h == P.min() / 20.0 and 100.0 <= tmax <= 4000.0
        assert 20 <= steps(h, tmax) <= 80000


def test_workloads_are_deterministic():
    a = W.batch_uneven(20, seed=7)
    b = W.batch_uneven(20, seed=7)
    assert all(np.array_equal(x, y) for x, y in zip(a[0], b[0])) and a[1:] == b[1:]
    c = W.batch_uneven(20, seed=8)
    assert not all(x.shape == y.shape and np.array_equal(x, y) for x, y in zip(a[0], c[0]))
