"""Full-size properties on the GPU at the benchmark workload's size.

At 4096 systems x 2000 steps the oracle would take minutes, so the whole
batch is checked through size-independent properties, and a sample of
systems against the oracle:
  * determinism: two runs are bitwise identical;
  * grad = false gives bitwise the transit times of grad = true;
  * the AHL21 map is symplectic in (x, v) for fixed masses, so the (x, v)
    block of jac_step has determinant 1 (Liouville) up to rounding;
  * every status word is clean and every output finite;
  * a sample of systems matches the oracle.
"""
import numpy as np
import pytest

import nbg
import oracle_lib as O
import parity as P
from conftest import has_gpu
from nbg import workloads as W

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not has_gpu(), reason="needs a CUDA GPU")]


@pytest.fixture(scope="module")
def c1_batch():
    els, h, tmax = W.batch_3body(4096, seed=0)
    states = [nbg.State(W.ic_of(el)) for el in els]
    timings = [nbg.TransitTiming(tmax, W.ic_of(el)) for el in els[:1]] * len(els)
    ntt = timings[0].ntt

    def run(grad):
        b = nbg.Batch([3] * len(els), 0, h, tmax, ntt, grad)
        for q, s in enumerate(states):
            b.set_system(q, s)
        b.run()
        return b

    return els, h, tmax, states, run


def test_deterministic_and_grad_free_times(c1_batch):
    els, h, tmax, states, run = c1_batch
    b1 = run(True)
    b2 = run(True)
    b0 = run(False)
    for k in ("x", "v", "tt", "count", "jac_step", "dtdq0", "dtdelements"):
        assert np.array_equal(b1.arrays[k], b2.arrays[k]), k
    assert np.array_equal(b1.arrays["tt"], b0.arrays["tt"])
    assert np.array_equal(b1.arrays["x"], b0.arrays["x"])
    # NONFINITE / NTT_OVERFLOW must not occur; a transit Newton search that stops at
    # ITMAX = 20 without an exact repeat is allowed (the reference continues
    # silently) but must stay rare.
    bad = nbg._lib.NBG_STATUS_NONFINITE | nbg._lib.NBG_STATUS_NTT_OVERFLOW
    assert np.all((b1.status & bad) == 0)
    itmax = int(np.count_nonzero(b1.status & nbg._lib.NBG_STATUS_NEWTON_ITMAX))
    transits = int(b1.arrays["count"].sum())
    assert itmax <= transits // 1000, (itmax, transits)
    for k in ("x", "v", "tt", "jac_step", "dtdq0", "dtdelements"):
        assert np.all(np.isfinite(b1.arrays[k])), k
    # symplectic (x, v) block: det = 1
    n, M = 3, 21
    rows = [7 * b + r for b in range(n) for r in range(6)]
    worst = 0.0
    for q in range(0, len(els), 37):
        J = b1.view("jac_step", q).reshape((M, M), order="F")
        d = np.linalg.det(J[np.ix_(rows, rows)])
        worst = max(worst, abs(d - 1.0))
    assert worst < 1e-8, worst
    # sample against the oracle
    for q in (0, 1000, 4095):
        s = states[q]
        so = O.OState(s.x, s.v, s.m, jac_init=s.jac_init)
        to = O.OTiming(3, int(b1.ntt[q]), 0)
        O.integrate_transits(so, to, h, tmax)
        cnt = b1.view("count", q)
        P.check_counts(cnt, to.count)
        ntt = int(b1.ntt[q])
        P.check_tt(b1.view("tt", q).reshape((3, ntt), order="F"), to.tt, to.count, tmax)
        P.check_transit_derivs(b1.view("dtdq0", q).reshape((3, ntt, 7, 3), order="F"), to.dtdq0, to.count)
        P.check_transit_derivs(b1.view("dtdelements", q).reshape((3, ntt, 7, 3), order="F"), to.dtdelements,
                               to.count, "dtdelements", to.dtdq0, so.jac_init)


def test_c2_shape_batch():
    """The 8-body workload's full batch (1024 systems, h = 0.06) over a
    shortened span (tmax = 120 days, 2000 steps): determinism, bitwise
    grad-free transit times, symplectic (x, v) block, clean status, and a
    sample of systems against the oracle."""
    els, h, _ = W.batch_8body(1024, seed=0)
    tmax = 120.0
    n, M = 8, 56
    states = [nbg.State(W.ic_of(el)) for el in els]
    ntt = nbg.TransitTiming(tmax, W.ic_of(els[0])).ntt + 2

    def run(grad):
        b = nbg.Batch([n] * len(els), 0, h, tmax, ntt, grad)
        for q, s in enumerate(states):
            b.set_system(q, s)
        b.run()
        return b

    b1, b2, b0 = run(True), run(True), run(False)
    for k in ("x", "v", "tt", "count", "jac_step", "dtdq0"):
        assert np.array_equal(b1.arrays[k], b2.arrays[k]), k
    assert np.array_equal(b1.arrays["tt"], b0.arrays["tt"])
    bad = nbg._lib.NBG_STATUS_NONFINITE | nbg._lib.NBG_STATUS_NTT_OVERFLOW
    assert np.all((b1.status & bad) == 0)
    transits = int(b1.arrays["count"].sum())
    assert transits > 1024 * 7 * 5
    itmax = int(np.count_nonzero(b1.status & nbg._lib.NBG_STATUS_NEWTON_ITMAX))
    assert itmax <= max(1, transits // 1000), (itmax, transits)
    rows = [7 * b + r for b in range(n) for r in range(6)]
    worst = 0.0
    for q in range(0, len(els), 97):
        J = b1.view("jac_step", q).reshape((M, M), order="F")
        worst = max(worst, abs(np.linalg.det(J[np.ix_(rows, rows)]) - 1.0))
    assert worst < 1e-8, worst
    for q in (0, 1023):
        s = states[q]
        so = O.OState(s.x, s.v, s.m, jac_init=s.jac_init)
        to = O.OTiming(n, ntt, 0)
        O.integrate_transits(so, to, h, tmax)
        P.check_counts(b1.view("count", q), to.count)
        P.check_tt(b1.view("tt", q).reshape((n, ntt), order="F"), to.tt, to.count, tmax)
        P.check_transit_derivs(b1.view("dtdq0", q).reshape((n, ntt, 7, n), order="F"), to.dtdq0, to.count)
        gs = type("S", (), {})()
        gs.x = b1.view("x", q).reshape((3, n), order="F")
        gs.v = b1.view("v", q).reshape((3, n), order="F")
        gs.jac_step = b1.view("jac_step", q).reshape((M, M), order="F")
        gs.dqdt = b1.view("dqdt", q)
        P.check_state(gs, so)
