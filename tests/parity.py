"""Parity rules between the CUDA path and the CPU oracle.

Tolerances (FP64 throughout):
  tt            |gpu - ref| <= 1e-10 * |tmax|                    (absolute, days)
  dtdq0,        per transit row (body j, transit c) with scale
  dtdelements   s = max_{k,p} |ref[j,c,k,p]|:
                |gpu - ref| <= 1e-8 * (|ref| + 1e-4 * s)
                i.e. 1e-8 relative, with an absolute floor of 1e-12 of the row
                scale for entries more than 4 decades below it
  x, v          |gpu - ref| <= 1e-10 * max|ref|  (per array)
  jac_step      |gpu - ref| <= 1e-9 * (|ref| + 1e-6 * max|ref column|)
  dqdt          |gpu - ref| <= 1e-9 * max|ref|
  count         identical
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


def check_transit_derivs(gpu, ref, count, name="dtdq0"):
    """gpu, ref: (n, ntt, 7, n) arrays; rows beyond count are ignored."""
    worst = 0.0
    ntt = gpu.shape[1]
    for j, c in enumerate(count):
        for t in range(min(int(c), ntt)):
            r = ref[j, t]
            g = gpu[j, t]
            s = float(np.max(np.abs(r)))
            if s == 0.0:
                assert np.all(g == 0.0)
                continue
            tol = DT_RTOL * (np.abs(r) + DT_FLOOR * s)
            ratio = float(np.max(np.abs(g - r) / tol))
            worst = max(worst, ratio)
            assert ratio <= 1.0, "%s[%d,%d]: error %.3g x tolerance" % (name, j, t, ratio)
    return worst


def check_state(gs, rs, x_rtol=1e-10, j_rtol=1e-9, check_jac=True):
    for k in ("x", "v"):
        g, r = getattr(gs, k), getattr(rs, k)
        err = float(np.max(np.abs(g - r)))
        assert err <= x_rtol * float(np.max(np.abs(r))), "%s differs by %g" % (k, err)
    if check_jac:
        g, r = gs.jac_step, rs.jac_step
        colmax = np.max(np.abs(r), axis=0, keepdims=True)
        tol = j_rtol * (np.abs(r) + 1e-6 * colmax)
        ratio = float(np.max(np.abs(g - r) / tol))
        assert ratio <= 1.0, "jac_step error %.3g x tolerance" % ratio
        dq = float(np.max(np.abs(gs.dqdt - rs.dqdt)))
        assert dq <= j_rtol * max(1e-300, float(np.max(np.abs(rs.dqdt)))), "dqdt differs by %g" % dq
