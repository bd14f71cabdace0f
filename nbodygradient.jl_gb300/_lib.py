"""ctypes binding of libnbg_cuda (include/nbg.h).

The library is built in-tree by build.py.  Loading fails loudly when it is
missing or cannot be loaded: there is no CPU fallback for any entry point.
"""
import ctypes
import os

import numpy as np

from . import build as _build

NBG_OK = 0
NBG_EINVAL = -1
NBG_ECUDA = -2
NBG_ENOMEM = -3
NBG_EUNSUPPORTED = -4
NBG_ENONFINITE = -5
NBG_ETIMEOUT = -6
NBG_ECANCELLED = -7

NBG_STATUS_NONFINITE = 1
NBG_STATUS_NTT_OVERFLOW = 2
NBG_STATUS_NEWTON_ITMAX = 4

MIN_BODIES = 2
MAX_BODIES = 10

# Every entry point include/nbg.h declares.
EXPORTS = (
    "nbg_create", "nbg_destroy", "nbg_last_error", "nbg_version", "nbg_device_info",
    "nbg_integrate_transits", "nbg_batch_integrate_transits", "nbg_batch_integrate_transits_device",
    "nbg_set_tuning", "nbg_last_timing", "nbg_last_launch_count", "nbg_fp64_peak", "nbg_fp64_mma_peak", "nbg_fp64_warp_issue",
    "nbg_set_profiling", "nbg_last_kernel_stats", "nbg_set_orbit_lanes", "nbg_set_orbit_team",
    "nbg_set_producer_layout", "nbg_last_host_time",
    "nbg_batch_integrate_transits_noalloc",
    "nbg_integrate", "nbg_integrate_steps", "nbg_batch_integrate",
    "nbg_integrate_transit_parameters", "nbg_batch_integrate_transit_parameters",
    "nbg_batch_init_nbody", "nbg_batch_init_nbody_device", "nbg_integrate_cartesian", "nbg_autotune_device",
    "nbg_server_start", "nbg_server_enqueue", "nbg_server_wait_any", "nbg_server_poll", "nbg_server_stats",
    "nbg_server_cancel", "nbg_server_stop", "nbg_batch_create", "nbg_batch_submit", "nbg_batch_run", "nbg_batch_wait",
    "nbg_batch_destroy",
)


class NbgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("libnbg_cuda error %d: %s" % (code, msg))
        self.code = code


class SystemDesc(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("ti", ctypes.c_int32), ("grad", ctypes.c_int32), ("ntt", ctypes.c_int32),
                ("h", ctypes.c_double), ("tmax", ctypes.c_double)]


class DeviceInfo(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 128), ("sm_count", ctypes.c_int), ("cc_major", ctypes.c_int),
                ("cc_minor", ctypes.c_int), ("total_mem", ctypes.c_size_t), ("min_bodies", ctypes.c_int),
                ("max_bodies", ctypes.c_int)]


class TuningResult(ctypes.Structure):
    _fields_ = [("chunk_steps", ctypes.c_int32), ("orbit_team", ctypes.c_int32), ("orbit_lanes", ctypes.c_int32),
                ("producer_warps", ctypes.c_int32), ("producer_smem_kb", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("ms", ctypes.c_double), ("system_steps_per_s", ctypes.c_double),
                ("trial_ms", ctypes.c_double * 4)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("slots_per_group", ctypes.c_int32), ("chunk_steps", ctypes.c_int32),
                ("max_inflight", ctypes.c_int32), ("orbit_lanes", ctypes.c_int32),
                ("hbm_budget_bytes", ctypes.c_uint64), ("orbit_team", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class RequestInfo(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int64), ("n", ctypes.c_int32), ("grad", ctypes.c_int32), ("nsteps", ctypes.c_int64),
                ("queue_ms", ctypes.c_double), ("run_ms", ctypes.c_double), ("latency_ms", ctypes.c_double),
                ("status", ctypes.c_uint32), ("rc", ctypes.c_int32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("admitted", ctypes.c_int64), ("completed", ctypes.c_int64),
                ("failed", ctypes.c_int64), ("running", ctypes.c_int64), ("pending", ctypes.c_int64),
                ("chunks", ctypes.c_int64), ("kernels", ctypes.c_int64), ("hbm_groups", ctypes.c_uint64),
                ("hbm_outputs_in_use", ctypes.c_uint64), ("hbm_budget", ctypes.c_uint64),
                ("groups", ctypes.c_int32), ("pad", ctypes.c_int32)]


_D = ctypes.POINTER(ctypes.c_double)
_U8 = ctypes.POINTER(ctypes.c_uint8)
_I64 = ctypes.POINTER(ctypes.c_int64)
_U32 = ctypes.POINTER(ctypes.c_uint32)
_VP = ctypes.c_void_p

_lib = None


def lib_path():
    return _build.LIB_PATH


def load(build_if_missing=True):
    """Load libnbg_cuda.so (building it first if needed) and declare prototypes."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise NbgError(NBG_EUNSUPPORTED, "libnbg_cuda.so not built (run nbodygradient.jl_gb300/build.py)")
    L = ctypes.CDLL(path)
    L.nbg_create.argtypes = [ctypes.c_int, ctypes.POINTER(_VP)]
    L.nbg_destroy.argtypes = [_VP]
    L.nbg_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.nbg_version.argtypes = []
    L.nbg_device_info.argtypes = [ctypes.c_int, ctypes.POINTER(DeviceInfo)]
    L.nbg_integrate_transits.argtypes = [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_int, _D, _D, _D, _D, _D, _D, _D, _D, _D, _U8, _D, ctypes.c_int64,
                                         _D, _D, _D, _I64]
    plain = [_D, _D, _D, _D, _D, _D, _D, _D, _D, _U8]
    L.nbg_integrate.argtypes = [_VP, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int] + plain
    L.nbg_integrate_steps.argtypes = [_VP, ctypes.c_int, ctypes.c_double, ctypes.c_int64, ctypes.c_int] + plain
    L.nbg_batch_integrate.argtypes = [_VP, ctypes.c_int, ctypes.POINTER(SystemDesc)] + plain
    L.nbg_integrate_cartesian.argtypes = [_VP, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int64] + \
        plain + [_D, _D, _D, _D]
    batch_args = [_VP, ctypes.c_int, ctypes.POINTER(SystemDesc), _D, _D, _D, _D, _D, _D, _D, _D, _D, _U8, _D, _D, _D,
                  _D, _I64, _U32]
    L.nbg_batch_integrate_transits.argtypes = batch_args
    _I32 = ctypes.POINTER(ctypes.c_int32)
    L.nbg_batch_init_nbody.argtypes = [_VP, ctypes.c_int, _I32, _D, _D, _D, _D, _D, _D]
    L.nbg_batch_init_nbody_device.argtypes = [_VP, ctypes.c_int, _I32, _D] + [_VP] * 5
    L.nbg_batch_integrate_transit_parameters.argtypes = batch_args
    L.nbg_integrate_transit_parameters.argtypes = L.nbg_integrate_transits.argtypes
    L.nbg_batch_integrate_transits_device.argtypes = [_VP, ctypes.c_int, ctypes.POINTER(SystemDesc)] + [_VP] * 16
    L.nbg_batch_integrate_transits_noalloc.argtypes = [_VP, ctypes.c_int, ctypes.POINTER(SystemDesc)] + [_VP] * 16
    L.nbg_autotune_device.argtypes = [_VP, ctypes.c_int, ctypes.POINTER(SystemDesc)] + [_VP] * 11 + \
        [ctypes.c_int, ctypes.POINTER(TuningResult), ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.nbg_set_tuning.argtypes = [_VP, ctypes.c_int, ctypes.c_int]
    L.nbg_last_timing.argtypes = [_VP, _D, _D, _D, _D]
    L.nbg_last_launch_count.argtypes = [_VP]
    L.nbg_last_launch_count.restype = ctypes.c_int64
    L.nbg_fp64_peak.argtypes = [_VP, _D]
    L.nbg_fp64_mma_peak.argtypes = [_VP, ctypes.c_int, _D, _D]
    L.nbg_fp64_warp_issue.argtypes = [_VP, ctypes.c_int, ctypes.c_int, _D]
    L.nbg_set_profiling.argtypes = [_VP, ctypes.c_int]
    L.nbg_set_orbit_lanes.argtypes = [_VP, ctypes.c_int]
    L.nbg_set_orbit_team.argtypes = [_VP, ctypes.c_int]
    L.nbg_set_producer_layout.argtypes = [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.nbg_last_host_time.argtypes = [_VP, _D]
    L.nbg_last_kernel_stats.argtypes = [_VP, _I64, _I64]
    L.nbg_server_start.argtypes = [ctypes.c_int, ctypes.POINTER(ServerConfig), ctypes.POINTER(_VP)]
    L.nbg_server_enqueue.argtypes = [_VP, ctypes.POINTER(SystemDesc), ctypes.c_double, _D, _D, _D, _D, _D, _D, _D,
                                     _D, _U8, _D, _I64]
    L.nbg_server_wait_any.argtypes = [_VP, ctypes.c_int32, _I64]
    L.nbg_server_poll.argtypes = [_VP, ctypes.c_int64, ctypes.c_int32, _D, _D, _D, _D, _D, _D, _D, _D, _D, _D, _D,
                                  _I64, ctypes.POINTER(RequestInfo)]
    L.nbg_server_stats.argtypes = [_VP, ctypes.POINTER(ServerStats)]
    L.nbg_server_stop.argtypes = [_VP]
    L.nbg_server_cancel.argtypes = [_VP, ctypes.c_int64]
    L.nbg_batch_create.argtypes = [_VP, ctypes.c_int, ctypes.POINTER(SystemDesc), ctypes.POINTER(_VP)]
    L.nbg_batch_submit.argtypes = [_VP, _D, _D, _D, _D, _D, _D, _D, _D, _D, _U8, _D, _D, _D, _D, _I64, _U32]
    L.nbg_batch_run.argtypes = [_VP]
    L.nbg_batch_wait.argtypes = [_VP, ctypes.c_int32]
    L.nbg_batch_destroy.argtypes = [_VP]
    _lib = L
    return L


def last_error():
    buf = ctypes.create_string_buffer(512)
    load().nbg_last_error(buf, 512)
    return buf.value.decode(errors="replace")


def check(rc):
    if rc != NBG_OK:
        raise NbgError(rc, last_error())
    return rc


class NonFiniteWarning(RuntimeWarning):
    """A system's x, v or jac_step ended non-finite (NBG_ENONFINITE)."""


def check_values(rc):
    """check() for the reference-facing calls: NBG_ENONFINITE becomes a warning, because the reference
    lets non-finite values propagate into the State without raising (the outputs are written as computed)."""
    if rc == NBG_ENONFINITE:
        import warnings
        warnings.warn(last_error(), NonFiniteWarning, stacklevel=3)
        return rc
    return check(rc)


def ptr(a, ctype=_D):
    if a is None:
        return ctypes.cast(None, ctype)
    if not (a.flags["F_CONTIGUOUS"] or a.flags["C_CONTIGUOUS"]):
        raise ValueError("array must be contiguous")
    return a.ctypes.data_as(ctype)


class Context:
    """One libnbg_cuda context (a CUDA stream plus cached device buffers)."""

    def __init__(self, device=0):
        L = load()
        h = _VP()
        check(L.nbg_create(device, ctypes.byref(h)))
        self._h = h
        self.device = device

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h is not None and self._h.value:
            load().nbg_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tuning(self, chunk_steps=0, overlap=-1):
        check(load().nbg_set_tuning(self._h, int(chunk_steps), int(overlap)))

    def last_timing(self):
        """(total, orbit, transit, jacobian) device ms of the last call."""
        a, b, c, d = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(load().nbg_last_timing(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(d)))
        return a.value, b.value, c.value, d.value

    def last_host_ms(self):
        """Host time (ms) the last batched call spent enqueueing its chunk loop."""
        v = ctypes.c_double()
        check(load().nbg_last_host_time(self._h, ctypes.byref(v)))
        return v.value

    def last_launch_count(self):
        return int(load().nbg_last_launch_count(self._h))

    def set_orbit_lanes(self, systems_per_warp=0):
        check(load().nbg_set_orbit_lanes(self._h, int(systems_per_warp)))

    def set_orbit_team(self, mode=-1):
        """-1 automatic, 0 one lane per system, 1 a team of lanes per system."""
        check(load().nbg_set_orbit_team(self._h, int(mode)))

    def set_producer_layout(self, warps_per_block=1, smem_kb=0, guard_kb=0):
        check(load().nbg_set_producer_layout(self._h, int(warps_per_block), int(smem_kb), int(guard_kb)))

    def set_profiling(self, on=True):
        """0 / False: off; 1 / True: every kernel kind; 2: the Jacobian consumer; 3: one sampled consumer launch."""
        check(load().nbg_set_profiling(self._h, int(on)))

    def last_kernel_stats(self):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        check(load().nbg_last_kernel_stats(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def fp64_peak_tflops(self):
        v = ctypes.c_double()
        check(load().nbg_fp64_peak(self._h, ctypes.byref(v)))
        return v.value

    def fp64_warp_issue_cycles(self, warps, chains):
        """SM cycles per warp-DFMA of the slowest of `warps` warps of one block running `chains` chains."""
        v = ctypes.c_double()
        check(load().nbg_fp64_warp_issue(self._h, int(warps), int(chains), ctypes.byref(v)))
        return v.value

    def fp64_mma_peak_tflops(self, with_dfma=False):
        """(TFLOP/s, DFMA share of those flops) of the FP64 tensor-core probe."""
        v, sh = ctypes.c_double(), ctypes.c_double()
        check(load().nbg_fp64_mma_peak(self._h, int(with_dfma), ctypes.byref(v), ctypes.byref(sh)))
        return v.value, sh.value


_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def device_info(device=0):
    d = DeviceInfo()
    check(load().nbg_device_info(device, ctypes.byref(d)))
    return {"name": d.name.decode(), "sm_count": d.sm_count, "cc": (d.cc_major, d.cc_minor),
            "total_mem": d.total_mem, "min_bodies": d.min_bodies, "max_bodies": d.max_bodies}


def as_f64(a, shape=None):
    a = np.asfortranarray(a, dtype=np.float64)
    if shape is not None and a.shape != shape:
        raise ValueError("expected shape %s, got %s" % (shape, a.shape))
    return a
