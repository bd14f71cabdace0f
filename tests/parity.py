"""Parity rules between the CUDA path and the CPU oracle.

Tolerances (FP64 throughout):
  tt            |gpu - ref| <= 1e-10 * |tmax|                    (absolute, days)
  dtdq0         per transit row (body j, transit c) with scale
                s = max_{k,p} |ref[j,c,k,p]|:
                |gpu - ref| <= 1e-8 * (|ref| + 1e-4 * s)
                i.e. 1e-8 relative, with an absolute floor of 1e-12 of the row
                scale for entries more than 4 decades below it
  dtdelements   = dtdq0 * jac_init, a sum of 7N products: its error bound is
                1e-8 * (|ref| + (|dtdq0| |jac_init|)[entry] + 1e-4 * s)
  x, v          |gpu - ref| <= 1e-10 * max|ref|  (per array)
  jac_step      |gpu - ref| <= 1e-9 * (|ref| + 1e-4 * max|ref column|)
  dqdt          |gpu - ref| <= 1e-9 * max|ref|
  count         identical
  TransitParameters (ttbv rows t, v_sky, b_sky^2):
  t row         as tt and dtdq0
  v_sky, b_sky^2  values |gpu - ref| <= 1e-10 * max|ref row|; derivatives
                normwise per transit row: max|gpu - ref| <= 1e-8 * max|ref|
                (the maxabs-norm isapprox of test/test_transit_parameters.jl,
                there over the whole array).  Entry-wise relative bounds do not
                hold for these rows: at mid-transit the sky separation is
                small, the b_sky^2 derivatives weigh position derivatives by
                it, and the double-precision reference itself is off from a
                quad-precision run by up to 1e-11 of the row scale there
The GPU and the oracle differ by rounding only (transcendental function
implementations, FMA use in the operator products, the factored pair update
and the adjoint form of the transit derivative); the tolerances bound how
far chaotic growth over the integration may carry those ulp differences.
"""
import numpy as np

TT_TOL = 1e-10
DT_RTOL = 1e-8
DT_FLOOR = 1e-4


def check_counts(gpu_count, ref_count):
    assert np.array_equal(np.asarray(gpu_count), np.asarray(ref_count)), (gpu_count, ref_count)


def check_tt(gpu_tt, ref_tt, count, tmax):
    ntt = gpu_tt.shape[1]
    err = 0.0
    for j, c in enumerate(count):
        k = min(int(c), ntt)
        if k:
            err = max(err, float(np.max(np.abs(gpu_tt[j, :k] - ref_tt[j, :k]))))
    assert err <= TT_TOL * abs(tmax), "tt differs by %g > %g" % (err, TT_TOL * abs(tmax))
    return err


def check_rows_normwise(gpu, ref, count, name, rtol=DT_RTOL):
    """gpu, ref: (n, ntt, 7, n); per transit row max|gpu - ref| <= rtol * max|ref|."""
    worst = 0.0
    for j, c in enumerate(count):
        for t in range(min(int(c), gpu.shape[1])):
            s = float(np.max(np.abs(ref[j, t])))
            e = float(np.max(np.abs(gpu[j, t] - ref[j, t])))
            if s == 0.0:
                assert e == 0.0, (name, j, t)
                continue
            worst = max(worst, e / (rtol * s))
            assert e <= rtol * s, "%s[%d,%d]: max error %.3g > %.3g x row max %.3g" % (name, j, t, e, rtol, s)
    return worst


def check_transit_derivs(gpu, ref, count, name="dtdq0", dtdq0=None, jac_init=None):
    """gpu, ref: (n, ntt, 7, n) arrays; rows beyond count are ignored.

    For dtdelements pass the reference dtdq0 and jac_init: the bound then
    includes the magnitude of the 7N products summed into each entry.
    """
    worst = 0.0
    ntt = gpu.shape[1]
    n = gpu.shape[0]
    for j, c in enumerate(count):
        for t in range(min(int(c), ntt)):
            r = ref[j, t]
            g = gpu[j, t]
            s = float(np.max(np.abs(r)))
            if s == 0.0:
                assert np.all(g == 0.0)
                continue
            mag = np.abs(r)
            if dtdq0 is not None:
                row = np.abs(dtdq0[j, t]).ravel(order="F")  # index q + 7 p
                mag = mag + (row @ np.abs(jac_init)).reshape((7, n), order="F")
            tol = DT_RTOL * (mag + DT_FLOOR * s)
            err = np.abs(g - r) / tol
            ratio = float(np.max(err))
            worst = max(worst, ratio)
            if ratio > 1.0:
                k, p = np.unravel_index(int(np.argmax(err)), err.shape)
                raise AssertionError("%s[%d,%d,%d,%d]: gpu %.17g ref %.17g, error %.3g x tolerance (row scale %.3g)"
                                     % (name, j, t, k, p, g[k, p], r[k, p], ratio, s))
    return worst


def check_state(gs, rs, x_rtol=1e-10, j_rtol=1e-9, check_jac=True):
    for k in ("x", "v"):
        g, r = getattr(gs, k), getattr(rs, k)
        err = float(np.max(np.abs(g - r)))
        assert err <= x_rtol * float(np.max(np.abs(r))), "%s differs by %g" % (k, err)
    if check_jac:
        g, r = gs.jac_step, rs.jac_step
        colmax = np.max(np.abs(r), axis=0, keepdims=True)
        tol = j_rtol * (np.abs(r) + 1e-4 * colmax)
        err = np.abs(g - r) / tol
        ratio = float(np.max(err))
        if ratio > 1.0:
            a, b = np.unravel_index(int(np.argmax(err)), err.shape)
            raise AssertionError("jac_step[%d,%d]: gpu %.17g ref %.17g, error %.3g x tolerance (column max %.3g)"
                                 % (a, b, g[a, b], r[a, b], ratio, colmax[0, b]))
        dq = float(np.max(np.abs(gs.dqdt - rs.dqdt)))
        assert dq <= j_rtol * max(1e-300, float(np.max(np.abs(rs.dqdt)))), "dqdt differs by %g" % dq
