"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

Test infrastructure: only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg use this module.  Array conventions are the reference's Julia
column-major layouts (numpy arrays in Fortran order); body indices are
0-based.
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB_PATH = os.path.join(ORACLE_DIR, "_build", "liboracle.so")

_lib = None

_D = ctypes.POINTER(ctypes.c_double)
_U8 = ctypes.POINTER(ctypes.c_uint8)
_I64 = ctypes.POINTER(ctypes.c_int64)


def build():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
    return _lib


def _p(a, ctype=_D):
    if a is None:
        return ctypes.cast(None, ctype)
    assert a.flags["F_CONTIGUOUS"] or a.ndim <= 1, "arrays must be column-major"
    return a.ctypes.data_as(ctype)


def f64(a):
    return np.asfortranarray(np.array(a, dtype=np.float64))


def init_nbody(elements, t0, H=None):
    """ElementsIC(t0, H, elements) -> init_nbody: returns x (3,n), v (3,n), jac_init (7n,7n)."""
    el = f64(elements)
    n = el.shape[0]
    x = np.zeros((3, n), order="F")
    v = np.zeros((3, n), order="F")
    jac = np.zeros((7 * n, 7 * n), order="F")
    Hm = None if H is None else f64(H)
    rc = lib().oracle_init_nbody(n, ctypes.c_double(t0), _p(el), _p(Hm), _p(x), _p(v), _p(jac))
    assert rc == 0
    return x, v, jac


class OState:
    """Mirror of the reference State fields the oracle reads and writes."""

    def __init__(self, x, v, m, jac_init=None, t=0.0, pair=None):
        self.x = f64(x)
        self.v = f64(v)
        self.m = f64(m)
        n = self.x.shape[1]
        self.n = n
        M = 7 * n
        self.xerror = np.zeros((3, n), order="F")
        self.verror = np.zeros((3, n), order="F")
        self.jac_step = np.asfortranarray(np.eye(M))
        self.jac_error = np.zeros((M, M), order="F")
        self.dqdt = np.zeros(M)
        self.jac_init = f64(jac_init) if jac_init is not None else np.asfortranarray(np.eye(M))
        self.pair = np.asfortranarray(np.zeros((n, n), dtype=np.uint8) if pair is None else np.array(pair, dtype=np.uint8))
        self.t = np.array([t], dtype=np.float64)

    def copy(self):
        o = OState.__new__(OState)
        for k, val in self.__dict__.items():
            o.__dict__[k] = val.copy() if isinstance(val, np.ndarray) else val
        return o


def ntt_for(tmax, periods):
    """TransitTiming's ntt (Transits.jl:44-45)."""
    periods = np.asarray(periods, dtype=np.float64)
    with np.errstate(divide="ignore"):
        q = tmax / periods
    ok = np.isfinite(q)
    return int(np.max(np.ceil(np.abs(q[ok])).astype(np.int64) + 3))


class OTiming:
    def __init__(self, n, ntt, ti=0):
        self.n, self.ntt, self.ti = n, ntt, ti
        self.tt = np.zeros((n, ntt), order="F")
        self.dtdq0 = np.zeros((n, ntt, 7, n), order="F")
        self.dtdelements = np.zeros((n, ntt, 7, n), order="F")
        self.count = np.zeros(n, dtype=np.int64)


class skip_zero_products:
    """Context manager: the oracle's dense products skip exact-zero operator
    entries inside the block (bitwise the same results for finite inputs,
    several times faster for N >= 8; the CPU baseline never sets it)."""

    def __enter__(self):
        self._prev = lib().oracle_set_skip_zero_products(1)
        return self

    def __exit__(self, *exc):
        lib().oracle_set_skip_zero_products(self._prev)
        return False


def integrate_transits(s, tt, h, tmax, grad=True):
    rc = lib().oracle_integrate_transits(
        s.n, tt.ti, ctypes.c_double(h), ctypes.c_double(tmax), int(grad), _p(s.t), _p(s.x), _p(s.v), _p(s.m),
        _p(s.xerror), _p(s.verror), _p(s.jac_step), _p(s.jac_error), _p(s.dqdt), _p(s.pair, _U8), _p(s.jac_init),
        tt.ntt, _p(tt.tt), _p(tt.dtdq0), _p(tt.dtdelements), _p(tt.count, _I64))
    assert rc == 0


class OParams:
    """TransitParameters (Transits.jl:68-110): ttbv 3 x n x ntt (t, v_sky, b_sky^2), dtbvdq0 and
    dtbvdelements 3 x n x ntt x 7 x n."""

    def __init__(self, n, ntt, ti=0):
        self.n, self.ntt, self.ti = n, ntt, ti
        self.ttbv = np.zeros((3, n, ntt), order="F")
        self.dtbvdq0 = np.zeros((3, n, ntt, 7, n), order="F")
        self.dtbvdelements = np.zeros((3, n, ntt, 7, n), order="F")
        self.count = np.zeros(n, dtype=np.int64)


def integrate_transit_parameters(s, tp, h, tmax, grad=True, quad=False):
    """quad=True runs the same restatement in quad precision (outputs rounded to double)."""
    fn = lib().oracle_integrate_transit_parameters_quad if quad else lib().oracle_integrate_transit_parameters
    rc = fn(
        s.n, tp.ti, ctypes.c_double(h), ctypes.c_double(tmax), int(grad), _p(s.t), _p(s.x), _p(s.v), _p(s.m),
        _p(s.xerror), _p(s.verror), _p(s.jac_step), _p(s.jac_error), _p(s.dqdt), _p(s.pair, _U8), _p(s.jac_init),
        tp.ntt, _p(tp.ttbv), _p(tp.dtbvdq0), _p(tp.dtbvdelements), _p(tp.count, _I64))
    assert rc == 0


def integrate_time(s, h, time, grad=True):
    rc = lib().oracle_integrate_time(
        s.n, ctypes.c_double(h), ctypes.c_double(time), int(grad), _p(s.t), _p(s.x), _p(s.v), _p(s.m),
        _p(s.xerror), _p(s.verror), _p(s.jac_step), _p(s.jac_error), _p(s.dqdt), _p(s.pair, _U8))
    assert rc == 0


def integrate_nsteps(s, h, nsteps, grad=True):
    rc = lib().oracle_integrate_nsteps(
        s.n, ctypes.c_double(h), ctypes.c_int64(nsteps), int(grad), _p(s.t), _p(s.x), _p(s.v), _p(s.m),
        _p(s.xerror), _p(s.verror), _p(s.jac_step), _p(s.jac_error), _p(s.dqdt), _p(s.pair, _U8))
    assert rc == 0


def ahl21_step(s, h, grad=True):
    rc = lib().oracle_ahl21_step(s.n, ctypes.c_double(h), int(grad), _p(s.x), _p(s.v), _p(s.m), _p(s.xerror),
                                 _p(s.verror), _p(s.jac_step), _p(s.jac_error), _p(s.dqdt), _p(s.pair, _U8))
    assert rc == 0


def kepler_driftij(s, i, j, h, drift_first):
    jac = np.zeros((14, 14), order="F")
    dq = np.zeros(14)
    rc = lib().oracle_kepler_driftij(s.n, i, j, ctypes.c_double(h), int(drift_first), _p(s.x), _p(s.v), _p(s.m),
                                     _p(s.xerror), _p(s.verror), _p(jac), _p(dq))
    assert rc == 0
    return jac, dq


def kickfast(s, h):
    M = 7 * s.n
    jac = np.zeros((M, M), order="F")
    dq = np.zeros(M)
    rc = lib().oracle_kickfast(s.n, ctypes.c_double(h), _p(s.x), _p(s.v), _p(s.m), _p(s.xerror), _p(s.verror),
                               _p(s.pair, _U8), _p(jac), _p(dq))
    assert rc == 0
    return jac, dq


def phi(s, h, alpha=2.0, which=0):
    M = 7 * s.n
    jac = np.zeros((M, M), order="F")
    dq = np.zeros(M)
    rc = lib().oracle_phi(s.n, ctypes.c_double(h), ctypes.c_double(alpha), which, _p(s.x), _p(s.v), _p(s.m),
                          _p(s.xerror), _p(s.verror), _p(s.pair, _U8), _p(jac), _p(dq))
    assert rc == 0
    return jac, dq


# ----------------------------------------------------------- quad-precision pins
def fd_kepler_driftij(x, v, m, i, j, h, drift_first, dlnq=1e-15):
    x, v, m = f64(x), f64(v), f64(m)
    jac = np.zeros((14, 14), order="F")
    dq = np.zeros(14)
    lib().oracle_fd_kepler_driftij(x.shape[1], i, j, ctypes.c_double(h), int(drift_first), _p(x), _p(v), _p(m),
                                   ctypes.c_double(dlnq), _p(jac), _p(dq))
    return jac, dq


def fd_map_jacobian(x, v, m, op, h, nsteps=1, pair=None, dlnq=1e-15, nthreads=8):
    x, v, m = f64(x), f64(v), f64(m)
    n = x.shape[1]
    pr = None if pair is None else np.asfortranarray(np.array(pair, dtype=np.uint8))
    jac = np.zeros((7 * n, 7 * n), order="F")
    lib().oracle_fd_map_jacobian(n, op, ctypes.c_double(h), ctypes.c_int64(nsteps), _p(x), _p(v), _p(m),
                                 _p(pr, _U8), ctypes.c_double(dlnq), nthreads, _p(jac))
    return jac


def fd_dqdt(x, v, m, h, pair=None, dlnq=1e-15):
    x, v, m = f64(x), f64(v), f64(m)
    n = x.shape[1]
    pr = None if pair is None else np.asfortranarray(np.array(pair, dtype=np.uint8))
    out = np.zeros(7 * n)
    lib().oracle_fd_dqdt(n, ctypes.c_double(h), _p(x), _p(v), _p(m), _p(pr, _U8), ctypes.c_double(dlnq), _p(out))
    return out


def fd_dtdelements(elements, t0, h, tmax, ti, ntt, dq0=1e-10, H=None, nthreads=8):
    el = f64(elements)
    n = el.shape[0]
    out = np.zeros((n, ntt, 7, n), order="F")
    Hm = None if H is None else f64(H)
    lib().oracle_fd_dtdelements(n, ctypes.c_double(t0), _p(el), _p(Hm), ctypes.c_double(h), ctypes.c_double(tmax),
                                ti, ntt, ctypes.c_double(dq0), nthreads, _p(out))
    return out


def fd_dtbvdelements(elements, t0, h, tmax, ti, ntt, dq0=1e-10, H=None, nthreads=8):
    el = f64(elements)
    n = el.shape[0]
    out = np.zeros((3, n, ntt, 7, n), order="F")
    Hm = None if H is None else f64(H)
    lib().oracle_fd_dtbvdelements(n, ctypes.c_double(t0), _p(el), _p(Hm), ctypes.c_double(h),
                                  ctypes.c_double(tmax), ti, ntt, ctypes.c_double(dq0), nthreads, _p(out))
    return out


def order_run_quad(x, v, m, h, nsteps, pair=None, kick_den=6.0, alpha=2.0):
    """nsteps of the no-gradient ahl21!(s, h) in quad precision.  Returns (x, v, max relative energy error):
    x and v as (hi, lo) double pairs of the quad result."""
    x, v, m = f64(x), f64(v), f64(m)
    n = x.shape[1]
    xh, xl, vh, vl = (np.zeros((3, n), order="F") for _ in range(4))
    de = ctypes.c_double()
    pr = None if pair is None else np.asfortranarray(np.array(pair, dtype=np.uint8))
    rc = lib().oracle_order_run_quad(n, ctypes.c_double(h), ctypes.c_int64(nsteps), _p(x), _p(v), _p(m),
                                     _p(pr, _U8), ctypes.c_double(kick_den), ctypes.c_double(alpha), _p(xh),
                                     _p(xl), _p(vh), _p(vl), ctypes.byref(de))
    assert rc == 0
    return (xh, xl), (vh, vl), de.value


def kepler_init(time, mass, el6, quad=False):
    """kepler_init with its 7x7 Jacobian: returns x (3), v (3), jac (7, 7)."""
    e = f64(el6)
    x, v, jac = np.zeros(3), np.zeros(3), np.zeros((7, 7), order="F")
    lib().oracle_kepler_init(ctypes.c_double(time), ctypes.c_double(mass), _p(e), int(quad), _p(x), _p(v), _p(jac))
    return x, v, jac


def fd_kepler_init(time, mass, el6, dq):
    jac = np.zeros((7, 7), order="F")
    lib().oracle_fd_kepler_init(ctypes.c_double(time), ctypes.c_double(mass), _p(f64(el6)), _p(f64(dq)), _p(jac))
    return jac


def fd_init_nbody(elements, t0, dq, dq_star_mass=1e-15, H=None):
    el = f64(elements)
    n = el.shape[0]
    out = np.zeros((7 * n, 7 * n), order="F")
    Hm = None if H is None else f64(H)
    dqa = f64(dq)
    lib().oracle_fd_init_nbody(n, ctypes.c_double(t0), _p(el), _p(Hm), _p(dqa), ctypes.c_double(dq_star_mass),
                               _p(out))
    return out


def maxabs_close(a, b, rtol=np.sqrt(np.finfo(float).eps)):
    """isapprox(a, b; norm=maxabs) with Julia's default rtol = sqrt(eps)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b))) <= rtol * max(float(np.max(np.abs(a))), float(np.max(np.abs(b))))
