"""Inputs the reference would carry silently into NaNs, on the GPU path.

The reference never checks its State during the integration: non-finite
values propagate (src/integrator/Integrator.jl:137-143 only prints whether
x, v and jac_step are finite).  The library raises NBG_STATUS_NONFINITE for
such a system in the batched calls' status words and NBG_ENONFINITE from the
single-system calls (a NonFiniteWarning in the Python mirror, whose outputs
are written as computed).  A bad system never disturbs the others of its
batch.  Eccentricities of 1 or more fail on the host as in the reference
(its sqrt of a negative number throws); on the device initial conditions
they give non-finite coordinates, which the integration flags.  A massless
planet is a test particle and integrates normally.
"""
import warnings

import numpy as np
import pytest

import nbg
import oracle_lib as O
import parity as P
from conftest import has_gpu
from nbg import workloads as W

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not has_gpu(), reason="needs a CUDA GPU")]

NONFINITE = nbg._lib.NBG_STATUS_NONFINITE


def _specs(seed, nsys=5):
    els, hs, tms = W.batch_uneven(nsys, seed=seed, nmin=3, nmax=5)
    out = []
    for el, h, tm in zip(els, hs, tms):
        ic = W.ic_of(el)
        tmax = min(tm, 40.0)
        out.append((nbg.State(ic), nbg.TransitTiming(tmax, ic), h, tmax))
    return out


def _batch(specs, grad=True):
    b = nbg.Batch([s.n for s, _, _, _ in specs], 0, [h for _, _, h, _ in specs], [t for _, _, _, t in specs],
                  [tt.ntt for _, tt, _, _ in specs], grad)
    for q, (s, tt, _, _) in enumerate(specs):
        b.set_system(q, s, tt)
    return b


@pytest.mark.parametrize("grad", [True, False])
def test_nan_position_is_flagged_and_isolated(grad):
    specs = _specs(71)
    clean = _batch(specs, grad).run()
    specs[2][0].x[0, 1] = np.nan
    b = _batch(specs, grad).run()
    assert b.status[2] & NONFINITE
    assert not np.all(np.isfinite(b.view("x", 2)))
    for q in (0, 1, 3, 4):
        assert (b.status[q] & NONFINITE) == 0
        for k in ("x", "v", "tt", "count", "jac_step", "dtdq0", "dtdelements"):
            assert np.array_equal(b.view(k, q), clean.view(k, q)), (q, k)


def test_single_call_warns_and_writes_the_values():
    s, tt, h, tmax = _specs(72, nsys=1)[0]
    s.v[1, 2] = np.inf
    with pytest.warns(nbg.NonFiniteWarning):
        nbg.Integrator(nbg.ahl21, h, 0.0, tmax)(s, tt, grad=True)
    assert not np.all(np.isfinite(s.x))
    assert s.t[0] == float(np.rint(tmax / h)) * h  # the call ran to its end and set s.t as the reference does
    s2, tt2, h2, tmax2 = _specs(72, nsys=1)[0]
    s2.x[0, 1] = np.nan
    with pytest.warns(nbg.NonFiniteWarning):
        nbg.Integrator(nbg.ahl21, h2, 0.0, tmax2)(s2, 10.0 * h2, grad=False)  # intr(s, time)


def test_finite_call_raises_no_warning():
    s, tt, h, tmax = _specs(73, nsys=1)[0]
    with warnings.catch_warnings():
        warnings.simplefilter("error", nbg.NonFiniteWarning)
        nbg.Integrator(nbg.ahl21, h, 0.0, tmax)(s, tt, grad=True)


def test_eccentricity_of_one_or_more():
    el, h, _ = W.plain_3body(5)
    el[2, 3] = 1.2  # e cos(omega) = 1.2: e > 1
    ic = nbg.ElementsIC(0.0, 3, el)
    with pytest.raises(ValueError):
        nbg.State(ic)  # host initial conditions: sqrt of a negative number, as the reference throws
    x, v, jinit = nbg.init_nbody_batch([ic])[0]  # device initial conditions: non-finite coordinates
    assert not np.all(np.isfinite(x))
    n = 3
    b = nbg.Batch([n], 0, h, 20.0, [nbg.TransitTiming(20.0, W.ic_of(W.plain_3body(5)[0])).ntt], True)
    b.view("x", 0)[:] = x.ravel(order="F")
    b.view("v", 0)[:] = v.ravel(order="F")
    b.view("m", 0)[:] = el[:, 0]
    b.view("jac_step", 0)[:] = np.eye(7 * n).ravel(order="F")
    b.view("jac_init", 0)[:] = np.nan_to_num(jinit).ravel(order="F")
    b.run()
    assert b.status[0] & NONFINITE


def test_massless_planet_is_a_test_particle():
    """m = 0 for the outer planet, set on the State after the initial conditions (in nested Jacobi
    elements a massless outermost body makes the coordinate transform 0/0, in the reference too)."""
    el, h, _ = W.plain_3body(6)
    tmax = 60.0
    ic = nbg.ElementsIC(0.0, 3, el)
    s = nbg.State(ic)
    s.m[2] = 0.0
    tt = nbg.TransitTiming(tmax, ic)
    x, v, jinit = s.x.copy(order="F"), s.v.copy(order="F"), s.jac_init.copy(order="F")
    with warnings.catch_warnings():
        warnings.simplefilter("error", nbg.NonFiniteWarning)
        nbg.Integrator(nbg.ahl21, h, 0.0, tmax)(s, tt, grad=True)
    so = O.OState(x, v, s.m, jac_init=jinit)
    to = O.OTiming(3, tt.ntt, 0)
    O.integrate_transits(so, to, h, tmax)
    assert to.count.sum() > 0 and np.all(np.isfinite(to.dtdq0))
    P.check_counts(tt.count, to.count)
    P.check_tt(tt.tt, to.tt, to.count, tmax)
    P.check_state(s, so)
    P.check_transit_derivs(tt.dtdq0, to.dtdq0, to.count)
