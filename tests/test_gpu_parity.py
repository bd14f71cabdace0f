"""Parity of the CUDA path (libnbg_cuda through its C ABI) with the CPU oracle.

Every case runs the same seeded inputs through nbg_integrate_transits /
nbg_batch_integrate_transits and through the oracle's restatement of the
reference, and compares with the tolerances of tests/parity.py.
"""
import numpy as np
import pytest

import nbg
import oracle_lib as O
import parity as P
from conftest import has_gpu
from nbg import workloads as W

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not has_gpu(), reason="needs a CUDA GPU")]


def run_pair(el, h, tmax, grad=True, ti=1, t0=0.0, pair=None, H=None, masses=None):
    """(GPU state, GPU timing, oracle state, oracle timing) for one system."""
    ic = nbg.ElementsIC(t0, el.shape[0] if H is None else H, el)
    s = nbg.State(ic)
    if pair is not None:
        s.pair[...] = pair
    if masses is not None:
        s.m[...] = masses
    tt = nbg.TransitTiming(abs(tmax), ic, ti)
    x, v, jinit = s.x.copy(order="F"), s.v.copy(order="F"), s.jac_init.copy(order="F")
    nbg.Integrator(nbg.ahl21, h, t0, tmax)(s, tt, grad=grad)
    so = O.OState(x, v, ic.m if masses is None else masses, jac_init=jinit, t=t0, pair=pair)
    to = O.OTiming(ic.nbody, tt.ntt, ti - 1)
    O.integrate_transits(so, to, h, tmax, grad=grad)
    return s, tt, so, to


def compare(s, tt, so, to, tmax, grad=True):
    P.check_counts(tt.count, to.count)
    P.check_tt(tt.tt, to.tt, to.count, tmax)
    assert s.t[0] == so.t[0]
    P.check_state(s, so, check_jac=grad)
    if grad:
        P.check_transit_derivs(tt.dtdq0, to.dtdq0, to.count, "dtdq0")
        P.check_transit_derivs(tt.dtdelements, to.dtdelements, to.count, "dtdelements", to.dtdq0, so.jac_init)


def test_plain_3body_grad():
    """The plain single-system configuration: 3 bodies, h = 0.5, 2000 steps, ~150 transits."""
    el, h, tmax = W.plain_3body(0)
    s, tt, so, to = run_pair(el, h, tmax)
    assert to.count.sum() > 100
    compare(s, tt, so, to, tmax)


def test_grad_false_matches_grad_true_bitwise():
    """test/test_transit_timing.jl:97 and test/test_integrator.jl:184 on the GPU path."""
    el, h, tmax = W.plain_3body(3)
    ic = nbg.ElementsIC(0.0, 3, el)
    s1, s2 = nbg.State(ic), nbg.State(ic)
    t1, t2 = nbg.TransitTiming(tmax, ic), nbg.TransitTiming(tmax, ic)
    intr = nbg.Integrator(nbg.ahl21, h, 0.0, tmax)
    intr(s1, t1, grad=False)
    intr(s2, t2, grad=True)
    assert np.array_equal(t1.tt, t2.tt) and np.array_equal(t1.count, t2.count)
    assert np.array_equal(s1.x, s2.x) and np.array_equal(s1.v, s2.v)
    _, _, so, to = run_pair(el, h, tmax, grad=False)
    P.check_tt(t1.tt, to.tt, to.count, tmax)


@pytest.mark.parametrize("n", list(range(2, 11)))
def test_body_counts(n):
    """Every built body count against the oracle on a short integration."""
    els, hs, _ = W.batch_uneven(200, seed=n, nmin=n, nmax=n)
    el, h = els[0], hs[0]
    tmax = min(40.0, 200 * h)
    s, tt, so, to = run_pair(el, h, tmax)
    compare(s, tt, so, to, tmax)


def test_eight_body_trappist_like():
    els, h, _ = W.batch_8body(2, seed=5)
    tmax = 60.0
    s, tt, so, to = run_pair(els[0], h, tmax)
    assert to.count.sum() > 20
    compare(s, tt, so, to, tmax)


def test_kick_pairs():
    """pair[i,j] = true (kickfast! + phic!) for the planet pairs, Kepler for star-planet."""
    els, hs, _ = W.batch_uneven(50, seed=11, nmin=4, nmax=4)
    el, h = els[0], hs[0]
    pair = np.ones((4, 4), dtype=np.uint8)
    pair[0, :] = 0
    pair[:, 0] = 0
    s, tt, so, to = run_pair(el, h, 30.0, pair=pair)
    compare(s, tt, so, to, 30.0)


@pytest.mark.parametrize("ti", [2, 3])
def test_other_transited_body(ti):
    el, h, _ = W.plain_3body(4)
    s, tt, so, to = run_pair(el, h, 300.0, ti=ti)
    compare(s, tt, so, to, 300.0)


def test_backward_integration():
    """check_step (Integrator.jl:249-259): tmax < 0 integrates backward from s.t."""
    el, h, _ = W.plain_3body(5)
    s, tt, so, to = run_pair(el, h, -150.0)
    compare(s, tt, so, to, 150.0)


def test_nonzero_start_time():
    el, h, _ = W.plain_3body(6)
    s, tt, so, to = run_pair(el, h, 120.0, t0=7300.25)
    compare(s, tt, so, to, 120.0)


def test_second_call_continues_counts():
    """A second intr(s, tt) with the same TransitTiming appends transits (count in/out)."""
    el, h, _ = W.plain_3body(7)
    ic = nbg.ElementsIC(0.0, 3, el)
    s = nbg.State(ic)
    tt = nbg.TransitTiming(400.0, ic)
    intr = nbg.Integrator(nbg.ahl21, h, 0.0, 200.0)
    intr(s, tt)
    intr(s, tt)
    x, v, jinit = ic.init_nbody()
    so = O.OState(x, v, ic.m, jac_init=jinit)
    to = O.OTiming(3, tt.ntt, 0)
    O.integrate_transits(so, to, h, 200.0)
    O.integrate_transits(so, to, h, 200.0)
    compare(s, tt, so, to, 400.0)


def test_three_argument_call_with_dstate():
    """s, d = dState(ic); intr(s, tt, d; grad) (Transits.jl:140) gives the bits of intr(s, tt; grad)."""
    el, h, _ = W.plain_3body(8)
    ic = nbg.ElementsIC(0.0, 3, el)
    s1, d = nbg.dState(ic)
    s2 = nbg.State(ic)
    t1, t2 = nbg.TransitTiming(150.0, ic), nbg.TransitTiming(150.0, ic)
    intr = nbg.Integrator(nbg.ahl21, h, 0.0, 150.0)
    assert intr(s1, t1, d, grad=True) is None
    intr(s2, t2, grad=True)
    for k in ("x", "v", "jac_step", "dqdt", "t"):
        assert np.array_equal(getattr(s1, k), getattr(s2, k)), k
    for k in ("tt", "dtdq0", "dtdelements", "count"):
        assert np.array_equal(getattr(t1, k), getattr(t2, k)), k
    assert t1.count.sum() > 0


def test_ntt_overflow_counts_and_drops():
    """Transits beyond ntt are counted but not stored (timing.jl:18-19)."""
    el, h, tmax = W.plain_3body(8)
    ic = nbg.ElementsIC(0.0, 3, el)
    s = nbg.State(ic)
    tt = nbg.TransitTiming(60.0, ic)  # sized for 60 days, integrated for 200
    nbg.Integrator(nbg.ahl21, h, 0.0, 200.0)(s, tt)
    x, v, jinit = ic.init_nbody()
    so = O.OState(x, v, ic.m, jac_init=jinit)
    to = O.OTiming(3, tt.ntt, 0)
    O.integrate_transits(so, to, h, 200.0)
    assert int(to.count.max()) > tt.ntt
    compare(s, tt, so, to, 200.0)


@pytest.mark.parametrize("tmax", [0.5, 2.5, 100.0])
def test_massless_pair_reuses_previous_jacobian(tmax):
    """Two massless bodies: kepler_driftij_gamma! returns before refilling jac_ij (ahl21.jl:713)."""
    el, h, _ = W.plain_3body(9)
    el4 = np.zeros((4, 7))
    el4[:3] = el
    el4[3] = [1e-5, 35.0, 3.0, 0.01, 0.0, np.pi / 2, 0.0]
    masses = el4[:, 0].copy()
    masses[2] = masses[3] = 0.0  # test particles, set on the State after the initial conditions
    s, tt, so, to = run_pair(el4, h, tmax, masses=masses)
    assert np.all(np.isfinite(so.jac_step))
    compare(s, tt, so, to, tmax)


def _batch_inputs(specs):
    states, timings, hs, tms, grads = [], [], [], [], []
    for el, h, tmax, grad in specs:
        ic = nbg.ElementsIC(0.0, el.shape[0], el)
        states.append(nbg.State(ic))
        timings.append(nbg.TransitTiming(tmax, ic))
        hs.append(h)
        tms.append(tmax)
        grads.append(grad)
    return states, timings, hs, tms, grads


def test_alone_and_in_batch_are_identical():
    """Each system's result is bitwise the same alone and inside a mixed batch."""
    els, hs, tms = W.batch_uneven(24, seed=21, nmin=2, nmax=6)
    specs = [(el, h, min(tm, 60.0), bool(q % 3)) for q, (el, h, tm) in enumerate(zip(els, hs, tms))]
    states, timings, hs, tms, grads = _batch_inputs(specs)
    b = nbg.Batch([s.n for s in states], 0, hs, tms, [t.ntt for t in timings], grads)
    for q in range(len(states)):
        b.set_system(q, states[q], timings[q])
    b.run()
    for q in (0, 5, 11, 17, 23):
        s1, t1, _, _, g1 = _batch_inputs([specs[q]])
        b1 = nbg.Batch([s1[0].n], 0, hs[q], tms[q], [t1[0].ntt], grads[q])
        b1.set_system(0, s1[0], t1[0])
        b1.run()
        for k in ("x", "v", "tt", "count", "jac_step", "dtdq0", "dtdelements", "dqdt"):
            assert np.array_equal(b.view(k, q), b1.view(k, 0)), (q, k)


def test_async_batch_is_the_synchronous_call():
    """nbg_batch_create / submit / run / wait (Batch.start / wait) gives the synchronous call's bits; a wait with
    a zero limit either times out or returns the finished run."""
    els, hs, tms = W.batch_uneven(16, seed=41, nmin=2, nmax=7)
    specs = [(el, h, min(tm, 80.0), bool(q % 4)) for q, (el, h, tm) in enumerate(zip(els, hs, tms))]
    states, timings, hs, tms, grads = _batch_inputs(specs)
    bs, ba = [nbg.Batch([s.n for s in states], 0, hs, tms, [t.ntt for t in timings], grads) for _ in range(2)]
    for q in range(len(states)):
        bs.set_system(q, states[q], timings[q])
        ba.set_system(q, states[q], timings[q])
    bs.run()
    ba.start()
    try:
        ba.wait(timeout_ms=0)
        finished = True
    except nbg.NbgError as e:
        assert e.code == nbg._lib.NBG_ETIMEOUT
        finished = False
    if not finished:
        ba.wait()
    with pytest.raises(nbg.NbgError):
        ba.wait()  # nothing left to wait for
    for k in nbg.Batch.FIELDS:
        assert np.array_equal(bs.arrays[k], ba.arrays[k]), k
    assert np.array_equal(bs.status, ba.status)


def test_two_contexts_run_at_the_same_time():
    """Two contexts integrate the same batch at the same time from two library threads (asynchronous batches);
    each result is bitwise the batch run alone."""
    els, hs, tms = W.batch_uneven(12, seed=43, nmin=2, nmax=6)
    specs = [(el, h, min(tm, 60.0), True) for el, h, tm in zip(els, hs, tms)]
    states, timings, hs, tms, grads = _batch_inputs(specs)

    def make():
        b = nbg.Batch([s.n for s in states], 0, hs, tms, [t.ntt for t in timings], grads)
        for q in range(len(states)):
            b.set_system(q, states[q], timings[q])
        return b

    ref = make().run()
    c1, c2 = nbg.Context(0), nbg.Context(0)
    b1, b2 = make(), make()
    b1.start(c1)
    try:
        b2.start(c2)
    except nbg.NbgError:
        b1.wait()
        raise
    errs = []
    for b in (b1, b2):  # both runs end before either context is closed
        try:
            b.wait()
        except nbg.NbgError as e:
            errs.append(e)
    c1.close()
    c2.close()
    assert not errs, errs
    for k in nbg.Batch.FIELDS:
        assert np.array_equal(ref.arrays[k], b1.arrays[k]) and np.array_equal(ref.arrays[k], b2.arrays[k]), k


def test_batch_matches_oracle():
    els, hs, tms = W.batch_uneven(12, seed=31, nmin=2, nmax=9)
    specs = [(el, h, min(tm, 50.0), True) for el, h, tm in zip(els, hs, tms)]
    states, timings, hs, tms, grads = _batch_inputs(specs)
    gs = [s.copy() for s in states]
    status = nbg.integrate_transits_batch(gs, timings, hs, tms, True)
    # a transit Newton search that stops at ITMAX is allowed (the reference continues silently)
    assert np.all((status & ~np.uint32(nbg._lib.NBG_STATUS_NEWTON_ITMAX)) == 0)
    for q, (el, h, tmax, _) in enumerate(specs):
        x, v, jinit = states[q].x, states[q].v, states[q].jac_init
        so = O.OState(x, v, states[q].m, jac_init=jinit)
        to = O.OTiming(states[q].n, timings[q].ntt, 0)
        O.integrate_transits(so, to, h, tmax)
        compare(gs[q], timings[q], so, to, tmax)


@pytest.mark.parametrize("grad", [True, False])
def test_team_producer_is_bitwise_the_one_lane_producer(grad):
    """The team form of the orbit producer (level-parallel sweeps) and its wide
    form (two lanes per pair solve) against the one-lane form, all in
    multi-warp blocks holding their SM's shared memory too, for every body
    count: bitwise the same x, v, jac_step, transit times and derivatives."""
    specs = []
    for n in range(2, 11):
        els, hs, tms = W.batch_uneven(3, seed=40 + n, nmin=n, nmax=n)
        specs += [(el, h, 90 * h, grad) for el, h in zip(els, hs)]
    states, timings, hs, tms, grads = _batch_inputs(specs)
    out = []
    for mode, layout in ((0, (1, 0, 0)), (1, (1, 0, 0)), (0, (4, 200, 32)), (1, (4, 200, 32)), (1, (3, 0, 0)),
                         (2, (1, 0, 0)), (2, (4, 200, 32))):
        ctx = nbg.Context(0)
        ctx.set_orbit_team(mode)
        ctx.set_producer_layout(*layout)
        b = nbg.Batch([s.n for s in states], 0, hs, tms, [t.ntt for t in timings], grads)
        for q in range(len(states)):
            b.set_system(q, states[q], timings[q])
        b.run(ctx)
        out.append(b)
        ctx.close()
    assert sum(int(c) for c in out[0].arrays["count"]) > 0
    for b in out[1:]:
        for k in ("x", "v", "xerror", "verror", "tt", "count", "jac_step", "jac_error", "dtdq0", "dtdelements",
                  "dqdt"):
            assert np.array_equal(out[0].arrays[k], b.arrays[k]), k


@pytest.mark.parametrize("n", [3, 5, 8])
@pytest.mark.parametrize("grad", [True, False])
def test_plain_integration_to_time(n, grad):
    """intr(s, time) (Integrator.jl:159-197) with a fractional last step, forward and back."""
    els, hs, _ = W.batch_uneven(2, seed=60 + n, nmin=n, nmax=n)
    el, h = els[0], hs[0]
    for time in (37.3 * h + 0.123 * h, -21.6 * h):
        ic = nbg.ElementsIC(0.0, n, el)
        s = nbg.State(ic)
        so = O.OState(s.x.copy(order="F"), s.v.copy(order="F"), ic.m, jac_init=s.jac_init.copy(order="F"), t=0.0)
        nbg.Integrator(nbg.ahl21, h, 0.0, 100.0)(s, float(time), grad=grad)
        O.integrate_time(so, h, time, grad=grad)
        assert s.t[0] == so.t[0] == time
        P.check_state(s, so, check_jac=grad)


def test_plain_integration_steps_and_default():
    """intr(s, N) for N > 0 and N < 0 (Integrator.jl:210-233) and intr(s) (Integrator.jl:247)."""
    el, h, _ = W.plain_3body(2)
    ic = nbg.ElementsIC(0.0, 3, el)
    for N in (57, -33):
        s = nbg.State(ic)
        so = O.OState(s.x.copy(order="F"), s.v.copy(order="F"), ic.m, jac_init=s.jac_init.copy(order="F"), t=0.0)
        nbg.Integrator(nbg.ahl21, h, 0.0, 100.0)(s, N)
        O.integrate_nsteps(so, h, N)
        assert s.t[0] == so.t[0]
        P.check_state(s, so)
    # a negative Integrator step with N > 0 takes the same backward steps as N < 0, and both calls leave
    # intr.h positive (Integrator.jl:215-229)
    s3, s4 = nbg.State(ic), nbg.State(ic)
    i3, i4 = nbg.Integrator(nbg.ahl21, -h, 0.0, 100.0), nbg.Integrator(nbg.ahl21, h, 0.0, 100.0)
    i3(s3, 20)
    i4(s4, -20)
    assert i3.h == h and i4.h == h
    assert s3.t[0] < 0.0
    for k in ("x", "v", "jac_step", "dqdt", "t"):
        assert np.array_equal(getattr(s3, k), getattr(s4, k)), k
    s = nbg.State(ic)
    s2 = nbg.State(ic)
    intr = nbg.Integrator(nbg.ahl21, h, 0.0, 12.25)
    intr(s)
    intr(s2, 12.25)
    for k in ("x", "v", "jac_step", "dqdt", "t"):
        assert np.array_equal(getattr(s, k), getattr(s2, k)), k


def test_plain_integration_batch_is_bitwise_single():
    els, hs, tms = W.batch_uneven(10, seed=71, nmin=2, nmax=9)
    states = [nbg.State(nbg.ElementsIC(0.0, el.shape[0], el)) for el in els]
    times = [min(t, 41.7 * h) for t, h in zip(tms, hs)]
    singles = [st.copy() for st in states]
    for st, h, tm in zip(singles, hs, times):
        nbg.Integrator(nbg.ahl21, h, 0.0, 1.0)(st, float(tm))
    import ctypes
    b = nbg.Batch([st.n for st in states], 0, hs, times, 1, True)
    for q, st in enumerate(states):
        b.set_system(q, st)
    a = b.arrays
    p = nbg._lib.ptr
    nbg._lib.check(nbg._lib.load().nbg_batch_integrate(
        nbg.default_context().handle, b.nsys, b.descriptors(), p(a["t"]), p(a["x"]), p(a["v"]), p(a["m"]),
        p(a["xerror"]), p(a["verror"]), p(a["jac_step"]), p(a["jac_error"]), p(a["dqdt"]), p(a["pair"], nbg._lib._U8)))
    for q, st in enumerate(singles):
        for k in ("x", "v", "jac_step", "dqdt"):
            assert np.array_equal(b.view(k, q), np.asarray(getattr(st, k)).ravel(order="F")), (q, k)
        assert b.view("t", q)[0] == st.t[0] == times[q]


def _check_tbv(tp, to, tmax, grad, jac_init=None):
    """TransitParameters parity: each row of ttbv and of the derivatives with the tolerances of
    tests/parity.py (t: 1e-10 tmax absolute; v_sky, b_sky^2: 1e-10 relative to the row's scale)."""
    P.check_counts(tp.count, to.count)
    P.check_tt(tp.ttbv[0], to.ttbv[0], to.count, tmax)
    for r in (1, 2):
        for j, c in enumerate(to.count):
            k = min(int(c), tp.ntt)
            if k:
                ref = to.ttbv[r, j, :k]
                assert np.max(np.abs(tp.ttbv[r, j, :k] - ref)) <= 1e-10 * np.max(np.abs(ref)), (r, j)
    if grad:
        P.check_transit_derivs(tp.dtbvdq0[0], to.dtbvdq0[0], to.count, "dtbvdq0[0]")
        P.check_transit_derivs(tp.dtbvdelements[0], to.dtbvdelements[0], to.count, "dtbvdelements[0]",
                               to.dtbvdq0[0], jac_init)
        for r in (1, 2):
            P.check_rows_normwise(tp.dtbvdq0[r], to.dtbvdq0[r], to.count, "dtbvdq0[%d]" % r)
            P.check_rows_normwise(tp.dtbvdelements[r], to.dtbvdelements[r], to.count, "dtbvdelements[%d]" % r)


def _oracle_tbv(s, ic, n, ntt, h, tmax, grad):
    so = O.OState(s.x.copy(order="F"), s.v.copy(order="F"), ic.m, jac_init=s.jac_init.copy(order="F"), t=0.0)
    to = O.OParams(n, ntt, 0)
    O.integrate_transit_parameters(so, to, h, tmax, grad=grad)
    return so, to


@pytest.mark.parametrize("grad", [True, False])
@pytest.mark.parametrize("n", [3, 6])
def test_transit_parameters_match_oracle(n, grad):
    """intr(s, ttbv::TransitParameters; grad) (Transits.jl:68-110, timing.jl:82-98, :155-193)."""
    els, hs, _ = W.batch_uneven(2, seed=80 + n, nmin=n, nmax=n)
    el, h = els[1], hs[1]
    tmax = 300 * h
    ic = nbg.ElementsIC(0.0, n, el)
    s = nbg.State(ic)
    tp = nbg.TransitParameters(tmax, ic)
    so, to = _oracle_tbv(s, ic, n, tp.ntt, h, tmax, grad)
    nbg.Integrator(nbg.ahl21, h, 0.0, tmax)(s, tp, grad=grad)
    assert to.count.sum() >= 2
    _check_tbv(tp, to, tmax, grad, so.jac_init)
    # t rows equal the TransitTiming call's tt bitwise; with grad, row 1 is its dtdq0
    s2 = nbg.State(ic)
    tt = nbg.TransitTiming(tmax, ic)
    nbg.Integrator(nbg.ahl21, h, 0.0, tmax)(s2, tt, grad=grad)
    assert np.array_equal(tt.tt, tp.ttbv[0]) and np.array_equal(tt.count, tp.count)
    if grad:
        assert np.array_equal(tt.dtdq0, tp.dtbvdq0[0])


def test_transit_parameters_plain_3body_full_length():
    """The plain 3-body configuration, 2000 steps and about 150 transits.  Its orbits are exactly
    edge-on, so b_sky^2 and its derivatives are rounding noise (about 1e-18); the t and v_sky rows carry
    the check."""
    el, h, tmax = W.plain_3body(4)
    ic = nbg.ElementsIC(0.0, 3, el)
    s = nbg.State(ic)
    tp = nbg.TransitParameters(tmax, ic)
    so, to = _oracle_tbv(s, ic, 3, tp.ntt, h, tmax, True)
    nbg.Integrator(nbg.ahl21, h, 0.0, tmax)(s, tp, grad=True)
    assert to.count.sum() > 100
    P.check_counts(tp.count, to.count)
    P.check_tt(tp.ttbv[0], to.ttbv[0], to.count, tmax)
    P.check_transit_derivs(tp.dtbvdq0[0], to.dtbvdq0[0], to.count, "dtbvdq0[0]")
    P.check_rows_normwise(tp.dtbvdq0[1], to.dtbvdq0[1], to.count, "dtbvdq0[1]")
    assert np.max(np.abs(tp.ttbv[2])) < 1e-12 and np.max(np.abs(tp.dtbvdq0[2])) < 1e-12
    P.check_state(s, so)


@pytest.mark.parametrize("n", [3, 7])
def test_cartesian_output_trajectory(n):
    """intr(s, o::CartesianOutput) (Outputs.jl:26-49): the state saved at the start of every step
    against the oracle stepping one step at a time, and the final state bitwise that of intr(s, N)."""
    els, hs, _ = W.batch_uneven(2, seed=90 + n, nmin=n, nmax=n)
    el, h = els[0], hs[0]
    nstep = 150  # more than two chunks
    ic = nbg.ElementsIC(0.0, n, el)
    s = nbg.State(ic)
    s2 = s.copy()
    o = nbg.CartesianOutput(n, nstep)
    intr = nbg.Integrator(nbg.ahl21, h, 0.0, 1e4)
    intr(s, o)
    nbg.Integrator(nbg.ahl21, h, 0.0, 1e4)(s2, nstep)
    for k in ("x", "v", "jac_step", "dqdt"):
        assert np.array_equal(getattr(s, k), getattr(s2, k)), k
    assert s.t[0] == s2.t[0]
    so = O.OState(ic.init_nbody()[0], ic.init_nbody()[1], ic.m, jac_init=s.jac_init.copy(order="F"), t=0.0)
    for i in range(nstep):
        assert o.t[i] == (0.0 if i == 0 else 0.0 + h * i)
        for k in ("x", "v"):
            ref = getattr(so, k)
            assert np.max(np.abs(getattr(o, k)[i] - ref)) <= 1e-10 * np.max(np.abs(ref)), (i, k)
        colmax = np.max(np.abs(so.jac_step), axis=0, keepdims=True)
        assert np.all(np.abs(o.jac_step[i] - so.jac_step) <= 1e-9 * (np.abs(so.jac_step) + 1e-4 * colmax)), i
        O.integrate_nsteps(so, h, 1)


def test_autotuner_leaves_inputs_and_results_unchanged():
    """nbg_autotune_device times candidates on copies: the caller's device arrays are untouched, and the
    integration after tuning is bitwise the one with the default mapping."""
    import torch
    els, hs, tms = W.batch_uneven(40, seed=99, nmin=2, nmax=7)
    specs = [(el, h, min(tm, 90 * h), True) for el, h, tm in zip(els, hs, tms)]
    states, timings, hs, tms, grads = _batch_inputs(specs)

    def batch():
        b = nbg.Batch([s.n for s in states], 0, hs, tms, [t.ntt for t in timings], grads)
        for q in range(len(states)):
            b.set_system(q, states[q], timings[q])
        return b

    b0 = batch()
    b0.run()
    b = batch()
    dev = {k: torch.from_numpy(a.copy()).cuda() for k, a in b.arrays.items()}
    before = {k: t.clone() for k, t in dev.items()}
    ctx = nbg.Context(0)
    res = b.autotune_device(dev, ctx, trial_steps=40)
    assert len(res) >= 6 and all(r["ms"] > 0 for r in res)
    for k in dev:
        assert torch.equal(dev[k], before[k]), k
    b.run_device(dev, ctx)
    for k in ("x", "v", "tt", "count", "jac_step", "dtdq0", "dtdelements"):
        assert np.array_equal(dev[k].cpu().numpy(), b0.arrays[k]), k
    ctx.close()
