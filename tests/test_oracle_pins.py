"""Pins of the CPU oracle against the reference's own tests, restated.

NbodyGradient.jl's test suite stores no golden numbers: every check is a
comparison of analytic derivatives with two-sided finite differences run in
BigFloat, or a grad / no-grad identity.  These tests restate them against the
oracle, with __float128 (x86) / binary128 long double (Arm) standing in for
BigFloat.  The setups follow the reference test files cited per test; the
reference's test/elements.txt is read in place when it is present, and the
same checks run on seeded synthetic systems everywhere.
"""
import numpy as np
import pytest

import oracle_lib as O
import parity as P
from nbg import workloads as W

close = O.maxabs_close


def _tilt(x, v, third=False):
    """perturb! / tilt of the reference tests (test_integrator.jl:17-26)."""
    x, v = x.copy(order="F"), v.copy(order="F")
    x[1, 0] = 5e-1 * np.sqrt(x[0, 0] ** 2 + x[2, 0] ** 2)
    x[1, 1] = -5e-1 * np.sqrt(x[0, 1] ** 2 + x[2, 1] ** 2)
    v[1, 0] = 5e-1 * np.sqrt(v[0, 0] ** 2 + v[2, 0] ** 2)
    v[1, 1] = -5e-1 * np.sqrt(v[0, 1] ** 2 + v[2, 1] ** 2)
    if third:
        x[1, 2] = -5e-1 * np.sqrt(x[0, 1] ** 2 + x[2, 1] ** 2)
        v[1, 2] = -5e-1 * np.sqrt(v[0, 1] ** 2 + v[2, 1] ** 2)
    return x, v


def _kepler_pin(x, v, m, h, drift_first):
    s = O.OState(x, v, m)
    O.kepler_driftij(s, 0, 1, h, drift_first)
    xa, va = s.x.copy(), s.v.copy()
    s2 = O.OState(xa, va, m)
    jac, dq = O.kepler_driftij(s2, 0, 1, h, drift_first)
    jn, dqn = O.fd_kepler_driftij(xa, va, m, 0, 1, h, drift_first)
    assert close(jn, jac + np.eye(14))
    assert close(dq, dqn)


@pytest.mark.parametrize("drift_first", [True, False])
@pytest.mark.parametrize("hyperbolic", [False, True])
def test_kepler_driftij_reference_setup(ref_elements, drift_first, hyperbolic):
    """test/test_kepler_driftij_gamma.jl:4-282 (h = 0.25, masses x1e-3 for the hyperbolic case)."""
    x, v, _ = O.init_nbody(ref_elements[:3], 7257.93115525)
    x, v = _tilt(x, v)
    m = ref_elements[:3, 0].copy()
    if hyperbolic:
        m *= 1e-3
    _kepler_pin(x, v, m, 0.25, drift_first)


@pytest.mark.parametrize("drift_first", [True, False])
@pytest.mark.parametrize("seed", [0, 1])
def test_kepler_driftij_synthetic(drift_first, seed):
    el, h, _ = W.plain_3body(seed)
    x, v, _ = O.init_nbody(el, 0.0)
    x, v = _tilt(x, v)
    _kepler_pin(x, v, el[:, 0], 0.25, drift_first)


def _kick_setup(ref_elements):
    el = ref_elements[:3].copy()
    el[1, 0] = 1.0
    el[2, 0] = 1.0
    x, v, _ = O.init_nbody(el, 7257.93115525)
    x, v = _tilt(x, v)
    pair = np.ones((3, 3), dtype=np.uint8)
    pair[0, 1:] = 0
    pair[1:, 0] = 0
    return x, v, el[:, 0].copy(), pair


def test_kickfast_reference_setup(ref_elements):
    """test/test_kickfast.jl: planets kicked, star-planet pairs Keplerian; h = 0.05."""
    x, v, m, pair = _kick_setup(ref_elements)
    s = O.OState(x, v, m, pair=pair)
    jac, _ = O.kickfast(s, 0.05)
    jn = O.fd_map_jacobian(x, v, m, 1, 0.05, pair=pair)
    assert close(jn - np.eye(jn.shape[0]), jac)


@pytest.mark.parametrize("op,which", [(4, 1), (3, 2)])
def test_phi_correctors(ref_elements, op, which):
    """test/test_phic.jl (kick pairs) and test/test_phisalpha.jl (Kepler pairs, alpha = 2)."""
    if which == 1:
        x, v, m, pair = _kick_setup(ref_elements)
    else:
        x, v, _ = O.init_nbody(ref_elements[:3], 7257.93115525)
        x, v = _tilt(x, v)
        m, pair = ref_elements[:3, 0].copy(), np.zeros((3, 3), dtype=np.uint8)
    s = O.OState(x, v, m, pair=pair)
    jac, _ = O.phi(s, 0.05, 2.0, which)
    jn = O.fd_map_jacobian(x, v, m, op, 0.05, pair=pair)
    assert close(jn - np.eye(jn.shape[0]), jac)


def test_integrator_jacobian_and_dqdt(ref_elements):
    """test/test_integrator.jl:1-185: jac_step after 100 steps (h = 0.05), dqdt after one step,
    and bit-identical x, v between grad and no-grad over 2000 days."""
    e = ref_elements[:3].copy()
    e[1, 0] *= 100.0
    e[2, 0] *= 100.0
    e[:, -1] = 0.0
    t0 = 7257.93115525
    x, v, _ = O.init_nbody(e, t0)
    xp, vp = _tilt(x, v, third=True)
    m = e[:, 0]
    s = O.OState(xp, vp, m, t=t0)
    O.integrate_nsteps(s, 0.05, 100, grad=True)
    jn = O.fd_map_jacobian(xp, vp, m, 0, 0.05, nsteps=100)
    assert close(np.arcsinh(s.jac_step), np.arcsinh(jn))
    s1 = O.OState(x, v, m, t=t0)
    O.integrate_nsteps(s1, 0.05, 1, grad=True)
    assert close(s1.dqdt, O.fd_dqdt(x, v, m, 0.05))
    sg, sn = O.OState(x, v, m, t=t0), O.OState(x, v, m, t=t0)
    O.integrate_time(sg, 0.05, t0 + 2000.0, grad=True)
    O.integrate_time(sn, 0.05, t0 + 2000.0, grad=False)
    assert np.array_equal(sg.x, sn.x) and np.array_equal(sg.v, sn.v)


def test_integrator_jacobian_synthetic():
    el, h, _ = W.plain_3body(2)
    x, v, _ = O.init_nbody(el, 0.0)
    s = O.OState(x, v, el[:, 0])
    O.integrate_nsteps(s, h, 50, grad=True)
    jn = O.fd_map_jacobian(x, v, el[:, 0], 0, h, nsteps=50)
    assert close(np.arcsinh(s.jac_step), np.arcsinh(jn))


def _transit_setup(ref_elements):
    N = 3
    t0 = 7257.93115525 - 7300.0 - 0.5
    e = ref_elements[:N].copy()
    e[1:, 2] -= 7300.0
    e[:, -1] = 0.0
    e[1, 0] *= 10.0
    e[2, 0] *= 10.0
    return e, t0


def test_transit_timing_derivatives(ref_elements):
    """test/test_transit_timing.jl:1-89 for ti = 1 (h = 0.04, tmax = 10, dq0 = 1e-10)."""
    e, t0 = _transit_setup(ref_elements)
    N, h, tmax, ti = 3, 0.04, 10.0, 0
    x, v, jinit = O.init_nbody(e, t0)
    ntt = O.ntt_for(tmax, e[:, 1])
    s = O.OState(x, v, e[:, 0], jac_init=jinit, t=t0)
    tt = O.OTiming(N, ntt, ti)
    O.integrate_transits(s, tt, h, tmax, grad=True)
    num = O.fd_dtdelements(e, t0, h, tmax, ti, ntt, dq0=1e-10)
    mask = np.zeros(tt.dtdq0.shape, dtype=bool)
    for jq in range(N):
        for iq in range(7):
            for i in range(N):
                if i == ti:
                    continue
                for k in range(tt.count[i]):
                    if iq not in (4, 5) and not (jq == 0 and iq < 6) and not (jq == i and iq == 6):
                        mask[i, k, iq, jq] = True
    a, b = np.arcsinh(tt.dtdelements), np.arcsinh(num)
    assert close(a[mask], b[mask])
    assert close(a, b)


def test_transit_parameters_derivatives(ref_elements):
    """test/test_transit_parameters.jl: d(t, v_sky, b_sky^2)/d elements against quad
    differences (h = 0.04, tmax = 10, dq0 = 1e-10), masked and unmasked."""
    e, t0 = _transit_setup(ref_elements)
    N, h, tmax = 3, 0.04, 10.0
    x, v, jinit = O.init_nbody(e, t0)
    ntt = O.ntt_for(tmax, e[:, 1])
    s = O.OState(x, v, e[:, 0], jac_init=jinit, t=t0)
    tp = O.OParams(N, ntt)
    O.integrate_transit_parameters(s, tp, h, tmax, grad=True)
    assert tp.count[1:].sum() >= 2
    num = O.fd_dtbvdelements(e, t0, h, tmax, 0, ntt, dq0=1e-10)
    mask = np.zeros(tp.dtbvdq0.shape, dtype=bool)
    for jq in range(N):
        for iq in range(7):
            for i in range(1, N):
                for k in range(tp.count[i]):
                    if iq not in (4, 5) and not (jq == 0 and iq < 6) and not (jq == i and iq == 6):
                        mask[:, i, k, iq, jq] = True
    a, b = np.arcsinh(tp.dtbvdelements), np.arcsinh(num)
    assert close(a[mask], b[mask])
    assert close(a, b)


def test_transit_parameters_times_equal_transit_timing(ref_elements):
    """ttbv[1, :, :] of TransitParameters is TransitTiming's tt (same Newton search), with and without grad;
    v_sky and b_sky^2 are those of the converged state."""
    e, t0 = _transit_setup(ref_elements)
    x, v, jinit = O.init_nbody(e, t0)
    ntt = O.ntt_for(60.0, e[:, 1])
    for grad in (True, False):
        s1 = O.OState(x, v, e[:, 0], jac_init=jinit, t=t0)
        s2 = O.OState(x, v, e[:, 0], jac_init=jinit, t=t0)
        tt, tp = O.OTiming(3, ntt), O.OParams(3, ntt)
        O.integrate_transits(s1, tt, 0.04, 60.0, grad=grad)
        O.integrate_transit_parameters(s2, tp, 0.04, 60.0, grad=grad)
        assert np.array_equal(tt.tt, tp.ttbv[0]) and np.array_equal(tt.count, tp.count)
        if grad:
            assert np.array_equal(tt.dtdq0, tp.dtbvdq0[0])
        for i in range(1, 3):
            k = int(tp.count[i])
            assert np.all(tp.ttbv[1, i, :k] > 0) and np.all(tp.ttbv[2, i, :k] < 1.0)


def test_transit_parameters_double_against_quad():
    """The double-precision restatement of TransitParameters against the same code in quad precision
    (100 steps, a mildly inclined 3-body system): the derivative rows agree normwise to 1e-8 of each
    transit row (the rule the GPU parity tests apply to the v_sky and b_sky^2 rows)."""
    els, hs, _ = W.batch_uneven(2, seed=83, nmin=3, nmax=3)
    el, h = els[1], hs[1]
    tmax = 100 * h
    x, v, jinit = O.init_nbody(el, 0.0)
    ntt = O.ntt_for(tmax, el[:, 1])
    out = []
    for quad in (False, True):
        s = O.OState(x, v, el[:, 0], jac_init=jinit)
        tp = O.OParams(3, ntt)
        O.integrate_transit_parameters(s, tp, h, tmax, grad=True, quad=quad)
        out.append(tp)
    d, q = out
    assert np.array_equal(d.count, q.count) and d.count.sum() >= 1
    for r in range(3):
        P.check_rows_normwise(d.dtbvdq0[r], q.dtbvdq0[r], d.count, "dtbvdq0[%d]" % r)


def test_transit_times_grad_equals_nograd(ref_elements):
    """test/test_transit_timing.jl:92-97: tt bit-identical with and without gradients over 2000 d."""
    e, t0 = _transit_setup(ref_elements)
    x, v, jinit = O.init_nbody(e, t0)
    ntt = O.ntt_for(2000.0, e[:, 1])
    s1 = O.OState(x, v, e[:, 0], jac_init=jinit, t=t0)
    s2 = O.OState(x, v, e[:, 0], jac_init=jinit, t=t0)
    t1, t2 = O.OTiming(3, ntt), O.OTiming(3, ntt)
    O.integrate_transits(s1, t1, 0.04, 2000.0, grad=False)
    O.integrate_transits(s2, t2, 0.04, 2000.0, grad=True)
    assert np.array_equal(t1.tt, t2.tt) and np.array_equal(t1.count, t2.count)


def test_findtransit_recovers_epochs(ref_elements):
    """test/test_findtransit.jl: 7 bodies, h = 0.01, tmax = 10; first transit = input t0 to 1e-6."""
    n, t0 = 7, 7257.0
    x, v, jinit = O.init_nbody(ref_elements[:n], t0)
    s = O.OState(x, v, ref_elements[:n, 0], jac_init=jinit, t=t0)
    tt = O.OTiming(n, O.ntt_for(10.0, ref_elements[:n, 1]))
    O.integrate_transits(s, tt, 0.01, 10.0, grad=False)
    for i in range(1, n):
        assert abs((ref_elements[i, 2] - tt.tt[i, 0]) / ref_elements[i, 2]) < 1e-6


def test_transit_timing_derivatives_synthetic():
    el, h, _ = W.plain_3body(1)
    tmax = 45.0
    x, v, jinit = O.init_nbody(el, 0.0)
    ntt = O.ntt_for(tmax, el[:, 1])
    s = O.OState(x, v, el[:, 0], jac_init=jinit)
    tt = O.OTiming(3, ntt)
    O.integrate_transits(s, tt, h, tmax, grad=True)
    assert tt.count.sum() >= 3
    num = O.fd_dtdelements(el, 0.0, h, tmax, 0, ntt, dq0=1e-10)
    assert close(np.arcsinh(tt.dtdelements), np.arcsinh(num))


def test_kepler_init_jacobian():
    """test/test_kepler_init.jl: kepler_init's 7x7 Jacobian for ten random orbits (P = 1.5, t0 ~ U(0, P),
    e cos w and e sin w ~ N(0, 1) redrawn until e < 0.2, I and Omega ~ U(0, pi), mass 1, time 2.4) against
    two-sided quad differences (steps 1e-15, as the reference's BigFloat ones) and against the same formulae
    evaluated in quad; isapprox with maxabs norm at Julia's default rtol."""
    rng = np.random.default_rng(17)
    period, mass, time = 1.5, 1.0, 2.4
    for _ in range(10):
        el = np.ones(6)
        while el[2] ** 2 + el[3] ** 2 >= 0.2 ** 2:
            el = np.array([period, rng.uniform() * period, rng.standard_normal(), rng.standard_normal(),
                           rng.uniform() * np.pi, rng.uniform() * np.pi])
        _, _, jac = O.kepler_init(time, mass, el)
        _, _, jac_q = O.kepler_init(time, mass, el, quad=True)
        num = O.fd_kepler_init(time, mass, el, [1e-15] * 7)
        assert close(jac, num)
        assert close(jac, jac_q)


def test_init_nbody_jacobian(ref_elements):
    """test/test_init_nbody.jl: jac_init against two-sided differences (steps 1e-12 / 1e-10)."""
    t0 = 7257.93115525 - 7300.0
    e = ref_elements[:3].copy()
    e[:, 2] -= 7300.0
    _, _, jac = O.init_nbody(e, t0)
    dq = [1e-10, 1e-10, 1e-10, 1e-10, 1e-10, 1e-10, 1e-12]  # (P, t0, ecos, esin, I, Omega, m)
    num = O.fd_init_nbody(e, t0, dq, dq_star_mass=1e-15)
    assert close(jac, num)


def test_init_nbody_jacobian_synthetic():
    els, _, _ = W.batch_8body(1)
    _, _, jac = O.init_nbody(els[0], 0.0)
    num = O.fd_init_nbody(els[0], 0.0, [1e-10] * 6 + [1e-13], dq_star_mass=1e-15)
    assert close(jac, num)


def keplerian_element_rows(H):
    """The elements row each Keplerian (row i < N - 1 of H) takes in kepcalc (init_nbody.jl:60-95): i + 1,
    shifted by one row after next for a Keplerian that starts a new branch (its H row is zero on body 1)."""
    rows, b = [], 0
    for i in range(H.shape[0] - 1):
        if H[i, 0] == 0:
            b += 1
        rows.append(i + 1 + b)
        if b > 0:
            b -= 2
        elif b < 0:
            b = 0
    return rows


def test_init_nbody_jacobian_double_binary():
    """jac_init for the hierarchy [4, 2, 1] (two binaries orbiting each other; the inverse A-matrix and its mass
    derivatives are no longer those of nested Jacobi coordinates) against two-sided quad differences.
    jac_init's element columns are per Keplerian (block i + 1 for row i of H, init_nbody.jl:84-86), the
    Keplerians take elements rows 1, 3, 2 here (the outer orbit is row 2), and the mass columns are per body;
    the differences perturb element row r into block r, so the orbital blocks are compared through that map."""
    import nbg
    H = nbg.hierarchy([4, 2, 1])
    el = np.array([[1.0, 0, 0, 0, 0, 0, 0],                                  # body a
                   [0.8, 10.0, 2.0, 0.01, 0.02, np.pi / 2, 0.0],              # body b; orbit a-b
                   [0.5, 400.0, 100.0, 0.05, 0.03, np.pi / 2 + 0.02, 0.0],    # body c; orbit (ab)-(cd)
                   [0.3, 12.0, 5.0, -0.02, 0.01, np.pi / 2 - 0.01, 0.1]])     # body d; orbit c-d
    rows = keplerian_element_rows(H)
    assert rows == [1, 3, 2]
    _, _, jac = O.init_nbody(el, 0.0, H)
    num = O.fd_init_nbody(el, 0.0, [1e-10] * 6 + [1e-12], dq_star_mass=1e-15, H=H)
    mapped = num.copy()
    for i, r in enumerate(rows):
        mapped[:, 7 * (i + 1):7 * (i + 1) + 6] = num[:, 7 * r:7 * r + 6]
    assert close(jac, mapped)
    assert not close(jac, num)  # the row-by-row layout differs for this hierarchy


@pytest.mark.parametrize("kick", [False, True])
def test_skip_zero_products_is_bitwise_dense(kick):
    """The oracle's zero-skipping products (used by the long GPU parity runs) give bitwise the dense
    products' integration: state, Jacobian, transit times and their derivatives."""
    el, h, _ = W.plain_3body(3)
    if kick:
        el = np.vstack([el, [2e-5, 41.0, 7.0, 0.01, -0.02, np.pi / 2, 0.0]])
    n = el.shape[0]
    x, v, jinit = O.init_nbody(el, 0.0)
    pair = np.zeros((n, n), dtype=np.uint8)
    if kick:
        pair[0, 3] = pair[3, 0] = 1
    tmax = 60.0
    out = []
    for skip in (False, True):
        s = O.OState(x, v, el[:, 0], jac_init=jinit, pair=pair)
        t = O.OTiming(n, O.ntt_for(tmax, el[1:, 1]), 0)
        if skip:
            with O.skip_zero_products():
                O.integrate_transits(s, t, h, tmax)
        else:
            O.integrate_transits(s, t, h, tmax)
        out.append((s, t))
    (a, ta), (b, tb) = out
    assert int(ta.count.sum()) > 0
    for k in ("x", "v", "xerror", "verror", "jac_step", "jac_error", "dqdt"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    for k in ("tt", "dtdq0", "dtdelements", "count"):
        assert np.array_equal(getattr(ta, k), getattr(tb, k)), k
    assert O.lib().oracle_set_skip_zero_products(0) == 0  # the context manager restored the default
