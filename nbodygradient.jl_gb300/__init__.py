"""nbodygradient.jl_gb300 -- GB300 (sm_103a) implementation of NbodyGradient.jl's
AHL21 integration with forward Jacobian propagation and transit timing.

The Python API mirrors the reference's Julia API for this path so that the
same call sequence works (names, argument meaning and error behaviour):

    ic  = ElementsIC(t0, H, elements)          # src/ics/InitialConditions.jl:142
    s   = State(ic)                            # src/integrator/Integrator.jl:82
    tt  = TransitTiming(tmax, ic)              # src/transits/Transits.jl:42
    intr = Integrator(ahl21, h, t0, tmax)      # src/integrator/Integrator.jl:17
    intr(s, tt, grad=True)                     # src/transits/Transits.jl:173

fills tt.tt, tt.dtdq0, tt.dtdelements and advances s, computed by libnbg_cuda
(CUDA, FP64) through its C ABI (include/nbg.h).  Body indices in this Python
mirror are 1-based where the Julia API is (TransitTiming's ti), 0-based in
the arrays.  There is no CPU fallback: without the CUDA library or a GPU the
calls raise NbgError.
"""
import math
import os

import numpy as np

# Each group of a batch runs on three CUDA streams of its own: ask the driver
# for 32 hardware work queues (the default 8 makes groups' streams share
# queues and serialise) before the process creates its CUDA context.  The
# library does the same when it is loaded; a caller's own setting is kept.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from . import _lib, build, workloads
from ._lib import Context, NbgError, NonFiniteWarning, SystemDesc, default_context, device_info
from .ics import CartesianIC, Elements, ElementsIC, hierarchy, hierarchy_nested, init_nbody, kepler_init

__all__ = ["Elements", "ElementsIC", "CartesianIC", "State", "TransitTiming", "TransitParameters", "CartesianOutput",
           "Integrator",
           "ahl21", "set_state", "initialize", "dState", "Derivatives",
           "Context", "NbgError", "NonFiniteWarning", "default_context", "device_info", "integrate_transits_batch", "Batch", "Server",
           "init_nbody_batch", "hierarchy",
           "hierarchy_nested", "init_nbody", "kepler_init"]


def ahl21(*args, **kwargs):
    """Scheme marker for Integrator(ahl21, ...); the step itself runs on the GPU."""
    raise TypeError("ahl21 is the integration scheme passed to Integrator; call the Integrator instead")


class State:
    """Current state of a system (src/integrator/Integrator.jl:49-103)."""

    def __init__(self, ic):
        x, v, jac_init = ic.init_nbody()
        n = ic.nbody
        M = 7 * n
        self.n = n
        self.x = np.asfortranarray(x, dtype=np.float64)
        self.v = np.asfortranarray(v, dtype=np.float64)
        self.t = np.array([ic.t0], dtype=np.float64)
        self.m = np.array(ic.m, dtype=np.float64)
        self.jac_step = np.asfortranarray(np.eye(M))
        self.dqdt = np.zeros(M)
        self.jac_init = np.asfortranarray(jac_init, dtype=np.float64)
        self.pair = np.asfortranarray(np.zeros((n, n), dtype=np.uint8))
        self.xerror = np.zeros((3, n), order="F")
        self.verror = np.zeros((3, n), order="F")
        self.dqdt_error = np.zeros(M)
        self.jac_error = np.zeros((M, M), order="F")

    def copy(self):
        o = State.__new__(State)
        for k, val in self.__dict__.items():
            o.__dict__[k] = val.copy(order="K") if isinstance(val, np.ndarray) else val
        return o

    def isfinite(self):
        return bool(np.all(np.isfinite(self.x)) and np.all(np.isfinite(self.v)) and np.all(np.isfinite(self.jac_step)))


class Derivatives:
    """The reference's preallocated step scratch (src/PreAllocArrays.jl:65-113), as taken by the three-argument
    intr(s, tt, d; grad) (Transits.jl:140).  The GPU path keeps its scratch on the device, so this holds the
    body count only.  Derivatives(n) or, as in Julia, Derivatives(T, n)."""

    def __init__(self, *args):
        if len(args) not in (1, 2):
            raise TypeError("Derivatives(n) or Derivatives(T, n)")
        self.n = int(args[-1])


def dState(ic):
    """State(ic) and a Derivatives for it (src/integrator/Integrator.jl:106-110)."""
    return State(ic), Derivatives(ic.nbody)


def initialize(s, ic):
    """initialize! (src/integrator/Integrator.jl:112-121): x, v and jac_init from ic, zero Kahan errors; the
    other State fields are kept."""
    x, v, jac_init = ic.init_nbody()
    s.x[...] = x
    s.v[...] = v
    s.jac_init[...] = jac_init
    s.xerror[...] = 0.0
    s.verror[...] = 0.0


def set_state(s_old, s_new):
    """set_state! (src/integrator/Integrator.jl:123-134)."""
    for k in ("t", "x", "v", "jac_step", "xerror", "verror", "jac_error", "dqdt", "dqdt_error"):
        getattr(s_old, k)[...] = getattr(s_new, k)


def _ntt(tmax, periods):
    periods = np.asarray(periods, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        q = tmax / periods
    ok = np.isfinite(q)
    return int(np.max(np.ceil(np.abs(q[ok])).astype(np.int64) + 3))


class TransitTiming:
    """Transit times and derivatives (src/transits/Transits.jl:14-56).  ti is 1-based.

    ntt defaults to the reference's max_i ceil(|tmax / P_i|) + 3; a larger
    value may be given so that a batch of systems shares one output shape.
    """

    def __init__(self, tmax, ic, ti=1, ntt=None):
        n = ic.nbody
        if not (1 <= ti <= n):
            raise ValueError("ti must be in 1..%d" % n)
        ntt_ref = _ntt(tmax, ic.elements[:, 1])
        if ntt is not None and ntt < ntt_ref:
            raise ValueError("ntt = %d is below the reference's %d" % (ntt, ntt_ref))
        ntt = ntt_ref if ntt is None else int(ntt)
        self.n, self.ntt, self.ti = n, ntt, ti
        self.tt = np.zeros((n, ntt), order="F")
        self.dtdq0 = np.zeros((n, ntt, 7, n), order="F")
        self.dtdelements = np.zeros((n, ntt, 7, n), order="F")
        self.count = np.zeros(n, dtype=np.int64)
        self.occs = [i for i in range(1, n + 1) if i != ti]

    def zero_out(self):
        for a in (self.tt, self.dtdq0, self.dtdelements):
            a[...] = 0.0
        self.count[...] = 0


class TransitParameters:
    """Transit times, sky velocities, impact parameters and derivatives
    (src/transits/Transits.jl:68-110).  ttbv[0] = t, ttbv[1] = v_sky,
    ttbv[2] = b_sky^2 (row index first, as the reference's 3 x n x ntt)."""

    def __init__(self, tmax, ic, ti=1, ntt=None):
        n = ic.nbody
        if not (1 <= ti <= n):
            raise ValueError("ti must be in 1..%d" % n)
        ntt_ref = _ntt(tmax, ic.elements[:, 1])
        if ntt is not None and ntt < ntt_ref:
            raise ValueError("ntt = %d is below the reference's %d" % (ntt, ntt_ref))
        ntt = ntt_ref if ntt is None else int(ntt)
        self.n, self.ntt, self.ti = n, ntt, ti
        self.ttbv = np.zeros((3, n, ntt), order="F")
        self.dtbvdq0 = np.zeros((3, n, ntt, 7, n), order="F")
        self.dtbvdelements = np.zeros((3, n, ntt, 7, n), order="F")
        self.count = np.zeros(n, dtype=np.int64)
        self.occs = [i for i in range(1, n + 1) if i != ti]

    def zero_out(self):
        for a in (self.ttbv, self.dtbvdq0, self.dtbvdelements):
            a[...] = 0.0
        self.count[...] = 0


class CartesianOutput:
    """Positions, velocities and Jacobian at every step (src/outputs/Outputs.jl:7-20).

    After intr(s, o): o.t[i], o.x[i] (3 x N), o.v[i] and, with jac=True,
    o.jac_step[i] (7N x 7N) hold the state at the start of step i + 1, as the
    reference's o.states[i + 1].  The reference's JLD2 file output stays with
    the caller (o.filename is kept for it)."""

    def __init__(self, nbody, nstep, filename="data.jld2", file=False, jac=True):
        self.nbody, self.nstep, self.filename, self.file = int(nbody), int(nstep), filename, file
        n, M = self.nbody, 7 * self.nbody
        self.t = np.zeros(self.nstep)
        self.x = np.zeros((self.nstep, 3, n))
        self.v = np.zeros((self.nstep, 3, n))
        self.jac_step = np.zeros((self.nstep, M, M)) if jac else None

    @property
    def states(self):
        """One lightweight record per saved step with t, x, v (and jac_step)."""
        out = []
        for i in range(self.nstep):
            r = type("SavedState", (), {})()
            r.t = np.array([self.t[i]])
            r.x = np.asfortranarray(self.x[i])
            r.v = np.asfortranarray(self.v[i])
            if self.jac_step is not None:
                r.jac_step = self.jac_step[i]
            out.append(r)
        return out


class Integrator:
    """Integrator(scheme, h, t0, tmax) (src/integrator/Integrator.jl:17-31).

    Accepted forms, as in the reference: Integrator(ahl21, h, t0, tmax),
    Integrator(ahl21, h, tmax), Integrator(h, tmax).
    """

    def __init__(self, *args):
        if args and callable(args[0]):
            scheme, rest = args[0], args[1:]
        else:
            scheme, rest = ahl21, args
        if scheme is not ahl21:
            raise NbgError(_lib.NBG_EUNSUPPORTED, "only the ahl21 scheme is implemented on the GPU")
        if len(rest) == 3:
            h, t0, tmax = rest
        elif len(rest) == 2:
            h, tmax = rest
            t0 = 0.0
        else:
            raise TypeError("Integrator(scheme, h, t0, tmax) or Integrator(scheme, h, tmax)")
        self.scheme = scheme
        self.h, self.t0, self.tmax = float(h), float(t0), float(tmax)

    def __call__(self, s, tt=None, d=None, *, grad=True, return_arrays=False, ctx=None):
        """intr(s, tt::TransitTiming; grad)   Transits.jl:173  (transit times; also TransitParameters)
        intr(s, tt, d::Derivatives; grad)   Transits.jl:140  (the same with preallocated scratch, e.g. dState)
        intr(s, time::float; grad)          Integrator.jl:159 (integrate to time)
        intr(s, N::int; grad)               Integrator.jl:210 (N steps)
        intr(s; grad)                       Integrator.jl:247 (to s.t + tmax)
        intr(s, o::CartesianOutput)         Outputs.jl:26

        grad is keyword-only, as in the reference.  return_arrays=True returns a Derivatives for the
        three-argument form, as the reference does (a fresh one: the step scratch itself lives on the device).
        A State that ends non-finite raises NonFiniteWarning (the reference propagates the values silently);
        the outputs are written as computed."""
        if d is not None:
            if not isinstance(d, Derivatives):
                raise TypeError("the third argument of intr(s, tt, d) is a Derivatives (dState(ic) makes one)")
            if not isinstance(tt, (TransitTiming, TransitParameters)):
                raise TypeError("intr(s, tt, d) takes a TransitTiming or TransitParameters")
            if d.n != s.n:
                raise ValueError("Derivatives for %d bodies, State for %d" % (d.n, s.n))
        ctx = ctx or default_context()
        L = _lib.load()
        p = _lib.ptr
        if tt is None or isinstance(tt, (float, np.floating, int, np.integer)):
            args = (p(s.t), p(s.x), p(s.v), p(s.m), p(s.xerror), p(s.verror), p(s.jac_step), p(s.jac_error),
                    p(s.dqdt), p(s.pair, _lib._U8))
            if tt is None:
                tt = float(s.t[0] + self.tmax)
            if isinstance(tt, (int, np.integer)) and not isinstance(tt, bool):
                _lib.check_values(L.nbg_integrate_steps(ctx.handle, s.n, self.h, int(tt), int(bool(grad)), *args))
                if self.h < 0:  # intr(s, N) leaves intr.h positive (Integrator.jl:228-229)
                    self.h = -self.h
            else:
                _lib.check_values(L.nbg_integrate(ctx.handle, s.n, self.h, float(tt), int(bool(grad)), *args))
            return None
        if isinstance(tt, CartesianOutput):
            if tt.nbody != s.n:
                raise ValueError("CartesianOutput has %d bodies, the State %d" % (tt.nbody, s.n))
            # C-order per-step blocks: step i's x is the column-major 3 x N block x_raw[i]
            xr = np.zeros((tt.nstep, 3 * s.n))
            vr = np.zeros((tt.nstep, 3 * s.n))
            jr = None if tt.jac_step is None else np.zeros((tt.nstep, 49 * s.n * s.n))
            _lib.check_values(L.nbg_integrate_cartesian(
                ctx.handle, s.n, self.h, self.tmax, tt.nstep, p(s.t), p(s.x), p(s.v), p(s.m), p(s.xerror),
                p(s.verror), p(s.jac_step), p(s.jac_error), p(s.dqdt), p(s.pair, _lib._U8), p(tt.t), p(xr), p(vr),
                p(jr)))
            for i in range(tt.nstep):
                tt.x[i] = xr[i].reshape((3, s.n), order="F")
                tt.v[i] = vr[i].reshape((3, s.n), order="F")
                if jr is not None:
                    tt.jac_step[i] = jr[i].reshape((7 * s.n, 7 * s.n), order="F")
            return None
        if isinstance(tt, TransitParameters):
            _lib.check_values(L.nbg_integrate_transit_parameters(
                ctx.handle, s.n, tt.ti - 1, self.h, self.tmax, int(bool(grad)), p(s.t), p(s.x), p(s.v), p(s.m),
                p(s.xerror), p(s.verror), p(s.jac_step), p(s.jac_error), p(s.dqdt), p(s.pair, _lib._U8),
                p(s.jac_init), tt.ntt, p(tt.ttbv), p(tt.dtbvdq0), p(tt.dtbvdelements), p(tt.count, _lib._I64)))
            return Derivatives(s.n) if return_arrays and d is None else None
        if not isinstance(tt, TransitTiming):
            raise NbgError(_lib.NBG_EUNSUPPORTED,
                           "intr(s, tt) takes a TransitTiming, a TransitParameters, a time or a step count")
        _lib.check_values(L.nbg_integrate_transits(
            ctx.handle, s.n, tt.ti - 1, self.h, self.tmax, int(bool(grad)), p(s.t), p(s.x), p(s.v), p(s.m),
            p(s.xerror), p(s.verror), p(s.jac_step), p(s.jac_error), p(s.dqdt), p(s.pair, _lib._U8), p(s.jac_init),
            tt.ntt, p(tt.tt), p(tt.dtdq0), p(tt.dtdelements), p(tt.count, _lib._I64)))
        # intr(s, tt; return_arrays=true) hands back the step scratch for later three-argument calls
        # (Transits.jl:173-180); the scratch of this path lives on the device, so a fresh Derivatives is
        # returned (usable the same way; its contents are not the last step's scratch)
        return Derivatives(s.n) if return_arrays and d is None else None


class Batch:
    """Packed arrays of many systems in the C ABI's batched layout.

    Every field is one flat float64 (int64 / uint8) array holding the
    systems' Julia column-major arrays back to back.  Built from State /
    TransitTiming pairs or directly from packed arrays; run() integrates all
    systems in one GPU plan.
    """

    FIELDS = ("t", "x", "v", "m", "xerror", "verror", "jac_step", "jac_error", "dqdt", "pair", "jac_init", "tt",
              "dtdq0", "dtdelements", "count")

    def __init__(self, n, ti, h, tmax, ntt, grad=True):
        n = np.atleast_1d(np.asarray(n, dtype=np.int32))
        nsys = len(n)

        def bc(a, dt):
            a = np.asarray(a, dtype=dt)
            return np.broadcast_to(a, (nsys,)).copy() if a.ndim == 0 else a.astype(dt)

        self.nsys = nsys
        self.n = n
        self.ti = bc(ti, np.int32)
        self.h = bc(h, np.float64)
        self.tmax = bc(tmax, np.float64)
        self.ntt = bc(ntt, np.int32)
        self.grad = bc(int(grad) if np.ndim(grad) == 0 else grad, np.int32)
        M = 7 * n.astype(np.int64)
        self.sizes = {
            "t": np.ones(nsys, np.int64), "x": 3 * n.astype(np.int64), "v": 3 * n.astype(np.int64),
            "m": n.astype(np.int64), "xerror": 3 * n.astype(np.int64), "verror": 3 * n.astype(np.int64),
            "jac_step": M * M, "jac_error": M * M, "dqdt": M, "pair": n.astype(np.int64) ** 2, "jac_init": M * M,
            "tt": n.astype(np.int64) * self.ntt, "dtdq0": n.astype(np.int64) * self.ntt * 7 * n,
            "dtdelements": n.astype(np.int64) * self.ntt * 7 * n, "count": n.astype(np.int64),
        }
        self.offsets = {k: np.concatenate([[0], np.cumsum(v)]) for k, v in self.sizes.items()}
        dt = {"pair": np.uint8, "count": np.int64}
        self.arrays = {k: np.zeros(int(self.offsets[k][-1]), dtype=dt.get(k, np.float64)) for k in self.FIELDS}
        self.status = np.zeros(nsys, dtype=np.uint32)

    def view(self, field, s):
        a, b = self.offsets[field][s], self.offsets[field][s + 1]
        return self.arrays[field][a:b]

    def set_system(self, s, state, timing=None):
        n = int(self.n[s])
        if state.n != n:
            raise ValueError("system %d: n mismatch" % s)
        self.view("t", s)[:] = state.t
        for k in ("x", "v", "xerror", "verror", "jac_step", "jac_error", "jac_init", "pair"):
            self.view(k, s)[:] = np.asarray(getattr(state, k)).ravel(order="F")
        self.view("m", s)[:] = state.m
        self.view("dqdt", s)[:] = state.dqdt
        if timing is not None:
            self.view("tt", s)[:] = timing.tt.ravel(order="F")
            self.view("dtdq0", s)[:] = timing.dtdq0.ravel(order="F")
            self.view("dtdelements", s)[:] = timing.dtdelements.ravel(order="F")
            self.view("count", s)[:] = timing.count

    def get_system(self, s, state, timing=None):
        n = int(self.n[s])
        M = 7 * n
        state.t[:] = self.view("t", s)
        state.x[...] = self.view("x", s).reshape((3, n), order="F")
        state.v[...] = self.view("v", s).reshape((3, n), order="F")
        state.xerror[...] = self.view("xerror", s).reshape((3, n), order="F")
        state.verror[...] = self.view("verror", s).reshape((3, n), order="F")
        state.jac_step[...] = self.view("jac_step", s).reshape((M, M), order="F")
        state.jac_error[...] = self.view("jac_error", s).reshape((M, M), order="F")
        state.dqdt[...] = self.view("dqdt", s)
        if timing is not None:
            ntt = timing.ntt
            timing.tt[...] = self.view("tt", s).reshape((n, ntt), order="F")
            timing.dtdq0[...] = self.view("dtdq0", s).reshape((n, ntt, 7, n), order="F")
            timing.dtdelements[...] = self.view("dtdelements", s).reshape((n, ntt, 7, n), order="F")
            timing.count[...] = self.view("count", s)

    def descriptors(self):
        d = (SystemDesc * self.nsys)()
        for s in range(self.nsys):
            d[s].n, d[s].ti, d[s].grad, d[s].ntt = int(self.n[s]), int(self.ti[s]), int(self.grad[s]), int(self.ntt[s])
            d[s].h, d[s].tmax = float(self.h[s]), float(self.tmax[s])
        return d

    def run(self, ctx=None):
        """nbg_batch_integrate_transits on the packed host arrays (in place)."""
        ctx = ctx or default_context()
        L = _lib.load()
        p = _lib.ptr
        a = self.arrays
        _lib.check(L.nbg_batch_integrate_transits(
            ctx.handle, self.nsys, self.descriptors(), p(a["t"]), p(a["x"]), p(a["v"]), p(a["m"]), p(a["xerror"]),
            p(a["verror"]), p(a["jac_step"]), p(a["jac_error"]), p(a["dqdt"]), p(a["pair"], _lib._U8),
            p(a["jac_init"]), p(a["tt"]), p(a["dtdq0"]), p(a["dtdelements"]), p(a["count"], _lib._I64),
            p(self.status, _lib._U32)))
        return self

    def start(self, ctx=None, device=0):
        """nbg_batch_create / submit / run: the same integration as run(), on a library thread; returns at once.
        The packed arrays belong to the run until wait() has returned.  Without ctx the run gets a context of
        its own on `device` (closed by wait()), so calls on the default context may go on meanwhile; a context
        passed in takes no other call until wait() has returned."""
        import ctypes
        if getattr(self, "_async", None) is not None:
            raise NbgError(_lib.NBG_EINVAL, "this batch is already running (wait() first)")
        own = ctx is None
        ctx = Context(device) if own else ctx
        L = _lib.load()
        p = _lib.ptr
        a = self.arrays
        h = ctypes.c_void_p()
        _lib.check(L.nbg_batch_create(ctx.handle, self.nsys, self.descriptors(), ctypes.byref(h)))
        rc = L.nbg_batch_submit(
            h, p(a["t"]), p(a["x"]), p(a["v"]), p(a["m"]), p(a["xerror"]), p(a["verror"]), p(a["jac_step"]),
            p(a["jac_error"]), p(a["dqdt"]), p(a["pair"], _lib._U8), p(a["jac_init"]), p(a["tt"]), p(a["dtdq0"]),
            p(a["dtdelements"]), p(a["count"], _lib._I64), p(self.status, _lib._U32))
        if rc == _lib.NBG_OK:
            rc = L.nbg_batch_run(h)
        if rc != _lib.NBG_OK:
            err = NbgError(rc, _lib.last_error())
            L.nbg_batch_destroy(h)
            if own:
                ctx.close()
            raise err
        self._async = (h, ctx, own)
        return self

    def wait(self, timeout_ms=-1):
        """nbg_batch_wait for a run started by start(); raises NbgError (code NBG_ETIMEOUT) while it continues.
        Once the run has ended, its batch handle is destroyed and its error, if any, raised."""
        if getattr(self, "_async", None) is None:
            raise NbgError(_lib.NBG_EINVAL, "no run in progress (start() first)")
        L = _lib.load()
        h, ctx, own = self._async
        rc = L.nbg_batch_wait(h, int(timeout_ms))
        if rc == _lib.NBG_ETIMEOUT:
            _lib.check(rc)
        err = NbgError(rc, _lib.last_error()) if rc != _lib.NBG_OK else None
        L.nbg_batch_destroy(h)
        self._async = None
        if own:
            ctx.close()
        if err is not None:
            raise err
        return self

    def __del__(self):
        # a run in progress writes into this batch's arrays: it ends before they are released
        if getattr(self, "_async", None) is not None:
            try:
                self.wait()
            except Exception:
                pass

    def run_device(self, dev_arrays, ctx=None):
        """nbg_batch_integrate_transits_device on device buffers (a dict of torch CUDA tensors)."""
        ctx = ctx or default_context()
        L = _lib.load()
        d = dev_arrays
        vp = lambda k: __import__("ctypes").c_void_p(d[k].data_ptr())
        _lib.check(L.nbg_batch_integrate_transits_device(
            ctx.handle, self.nsys, self.descriptors(), vp("t"), vp("x"), vp("v"), vp("m"), vp("xerror"),
            vp("verror"), vp("jac_step"), vp("jac_error"), vp("dqdt"), vp("pair"), vp("jac_init"), vp("tt"),
            vp("dtdq0"), vp("dtdelements"), vp("count"), __import__("ctypes").c_void_p(self.status.ctypes.data)))
        return self

    def autotune_device(self, dev_arrays, ctx=None, trial_steps=256):
        """nbg_autotune_device on device buffers: picks the fastest mapping for this batch on ctx and
        returns the candidates' predicted times (a list of dicts, the chosen one first)."""
        import ctypes
        ctx = ctx or default_context()
        L = _lib.load()
        d = dev_arrays
        vp = lambda k: ctypes.c_void_p(d[k].data_ptr())
        rep = (_lib.TuningResult * 32)()
        nrep = ctypes.c_int(0)
        _lib.check(L.nbg_autotune_device(
            ctx.handle, self.nsys, self.descriptors(), vp("t"), vp("x"), vp("v"), vp("m"), vp("xerror"),
            vp("verror"), vp("jac_step"), vp("jac_error"), vp("dqdt"), vp("pair"), vp("jac_init"), int(trial_steps),
            rep, 32, ctypes.byref(nrep)))
        out = [{k: (list(getattr(rep[q], k)) if k == "trial_ms" else getattr(rep[q], k))
                for k, _ in _lib.TuningResult._fields_ if k != "pad"} for q in range(nrep.value)]
        return out[:1] + sorted(out[1:], key=lambda r: r["ms"])

    def run_device_noalloc(self, dev_arrays, ctx=None):
        """nbg_batch_integrate_transits_noalloc on device buffers: the same call
        with every working buffer taken from the library's fixed scratch array
        (at most NBG_NOALLOC_MAX_SYSTEMS systems); the library allocates no
        device memory."""
        import ctypes
        ctx = ctx or default_context()
        L = _lib.load()
        d = dev_arrays
        vp = lambda k: ctypes.c_void_p(d[k].data_ptr())
        _lib.check(L.nbg_batch_integrate_transits_noalloc(
            ctx.handle, self.nsys, self.descriptors(), vp("t"), vp("x"), vp("v"), vp("m"), vp("xerror"),
            vp("verror"), vp("jac_step"), vp("jac_error"), vp("dqdt"), vp("pair"), vp("jac_init"), vp("tt"),
            vp("dtdq0"), vp("dtdelements"), vp("count"), ctypes.c_void_p(self.status.ctypes.data)))
        return self


class Server:
    """Continuous-batching request server (nbg_server_* in include/nbg.h).

    submit(s, tt, intr, grad) queues intr(s, tt; grad) for a State and a
    fresh TransitTiming and returns a request id; result(id, s, tt) waits for
    it, fills s and tt in place exactly as intr(s, tt; grad) would, and returns
    the request's latency record.  Requests from any thread; requests that
    arrive while others run join them on the GPU at the next chunk boundary.
    """

    def __init__(self, device=0, slots_per_group=0, chunk_steps=0, max_inflight=0, orbit_lanes=0,
                 hbm_budget_bytes=0, orbit_team=0):
        import ctypes
        L = _lib.load()
        cfg = _lib.ServerConfig(int(slots_per_group), int(chunk_steps), int(max_inflight), int(orbit_lanes),
                                int(hbm_budget_bytes), int(orbit_team), 0)
        h = ctypes.c_void_p()
        _lib.check(L.nbg_server_start(int(device), ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h

    def submit(self, s, tt, intr, grad=True):
        import ctypes
        if tt.count.any():
            raise ValueError("the server takes a fresh TransitTiming (count == 0)")
        L = _lib.load()
        p = _lib.ptr
        d = SystemDesc(s.n, tt.ti - 1, int(bool(grad)), tt.ntt, float(intr.h), float(intr.tmax))
        rid = ctypes.c_int64()
        _lib.check(L.nbg_server_enqueue(self._h, ctypes.byref(d), float(s.t[0]), p(s.x), p(s.v), p(s.m),
                                        p(s.xerror), p(s.verror), p(s.jac_step), p(s.jac_error), p(s.dqdt),
                                        p(s.pair, _lib._U8), p(s.jac_init), ctypes.byref(rid)))
        return rid.value

    def wait_any(self, timeout_ms=-1):
        import ctypes
        rid = ctypes.c_int64()
        _lib.check(_lib.load().nbg_server_wait_any(self._h, int(timeout_ms), ctypes.byref(rid)))
        return rid.value

    def result(self, rid, s, tt, timeout_ms=-1):
        """Collect request rid into (s, tt); returns its info as a dict."""
        import ctypes
        info = _lib.RequestInfo()
        p = _lib.ptr
        _lib.check(_lib.load().nbg_server_poll(
            self._h, int(rid), int(timeout_ms), p(s.t), p(s.x), p(s.v), p(s.xerror), p(s.verror), p(s.jac_step),
            p(s.jac_error), p(s.dqdt), p(tt.tt), p(tt.dtdq0), p(tt.dtdelements), p(tt.count, _lib._I64),
            ctypes.byref(info)))
        return {k: getattr(info, k) for k, _ in _lib.RequestInfo._fields_}

    def cancel(self, rid):
        """Withdraw request rid (nbg_server_cancel): result(rid, ...) then raises NbgError with
        NBG_ECANCELLED.  Raises NbgError (NBG_EINVAL) when the request has already finished."""
        _lib.check(_lib.load().nbg_server_cancel(self._h, int(rid)))

    def stats(self):
        import ctypes
        st = _lib.ServerStats()
        _lib.check(_lib.load().nbg_server_stats(self._h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in _lib.ServerStats._fields_}

    def stop(self):
        if self._h is not None and self._h.value:
            h, self._h = self._h, None
            _lib.check(_lib.load().nbg_server_stop(h))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.stop()

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass


def init_nbody_batch(ics, ctx=None):
    """init_nbody for many ElementsIC on the GPU (nbg_batch_init_nbody): returns a list of
    (x, v, jac_init) tuples, as ic.init_nbody() returns them on the host."""
    ctx = ctx or default_context()
    n = np.array([ic.nbody for ic in ics], dtype=np.int32)
    t0 = np.array([ic.t0 for ic in ics], dtype=np.float64)
    el = np.concatenate([np.asfortranarray(ic.elements, dtype=np.float64).ravel(order="F") for ic in ics])
    nested = all(np.array_equal(ic.H, hierarchy_nested(ic.nbody)) for ic in ics)
    H = None if nested else np.concatenate(
        [np.asfortranarray(ic.H, dtype=np.float64).ravel(order="F") for ic in ics])
    x = np.zeros(int(3 * n.sum()))
    v = np.zeros(int(3 * n.sum()))
    J = np.zeros(int((49 * n.astype(np.int64) ** 2).sum()))
    p = _lib.ptr
    _lib.check(_lib.load().nbg_batch_init_nbody(ctx.handle, len(ics), p(n, __import__("ctypes").POINTER(
        __import__("ctypes").c_int32)), p(t0), p(el), p(H), p(x), p(v), p(J)))
    out, ax, aJ = [], 0, 0
    for k in n:
        k = int(k)
        out.append((x[ax:ax + 3 * k].reshape((3, k), order="F"), v[ax:ax + 3 * k].reshape((3, k), order="F"),
                    J[aJ:aJ + 49 * k * k].reshape((7 * k, 7 * k), order="F")))
        ax += 3 * k
        aJ += 49 * k * k
    return out


def integrate_transits_batch(states, timings, h, tmax, grad=True, ctx=None):
    """Integrate many (State, TransitTiming) pairs in one GPU plan; updates them in place."""
    nsys = len(states)
    b = Batch([s.n for s in states], [t.ti - 1 for t in timings], h, tmax, [t.ntt for t in timings], grad)
    for q in range(nsys):
        b.set_system(q, states[q], timings[q])
    b.run(ctx)
    for q in range(nsys):
        b.get_system(q, states[q], timings[q])
    return b.status.copy()
