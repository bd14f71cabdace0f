"""The C ABI library: it builds, loads, exports every symbol include/nbg.h
declares, and reports errors cleanly (these checks need no GPU)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import nbg
from conftest import ROOT, has_gpu

HEADER = os.path.join(ROOT, "include", "nbg.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nbg_[a-z0-9_]+)\s*\(", src)))


def test_header_declarations_match_binding():
    decl = declared_functions()
    assert decl, "no declarations found"
    assert sorted(nbg._lib.EXPORTS) == decl


def test_library_exports_every_declared_symbol():
    path = nbg.build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (nbg_[a-z0-9_]+)$", out, flags=re.M))
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing
    L = nbg._lib.load()
    for f in declared_functions():
        assert hasattr(L, f)


def test_built_for_sm_103a_only():
    """Every unit compiles for exactly one target, sm_103a (no PTX for other architectures, no JIT), with
    separately rounded products (--fmad=false) and no host FP contraction."""
    flags = nbg.build.NVCC_FLAGS
    gencodes = [flags[i + 1] for i, f in enumerate(flags) if f == "-gencode"]
    assert gencodes == ["arch=compute_103a,code=sm_103a"]
    assert not any(f.startswith(("-arch", "--gpu-architecture", "-code")) for f in flags)
    assert "--fmad=false" in flags and "-ffp-contract=off" in flags


def test_version_and_error_buffer():
    L = nbg._lib.load()
    assert L.nbg_version() >= 100
    buf = ctypes.create_string_buffer(64)
    assert L.nbg_last_error(buf, 64) == 0
    assert L.nbg_last_error(None, 0) == nbg._lib.NBG_EINVAL


def test_null_arguments_are_rejected_without_a_gpu():
    L = nbg._lib.load()
    assert L.nbg_set_tuning(None, 16, 0) == nbg._lib.NBG_EINVAL
    assert L.nbg_last_timing(None, None, None, None, None) == nbg._lib.NBG_EINVAL
    assert L.nbg_integrate_transits(None, 3, 0, 0.5, 10.0, 1, *([None] * 11), 10, None, None, None, None) \
        == nbg._lib.NBG_EINVAL
    assert "NULL" in nbg._lib.last_error()


@pytest.mark.skipif(has_gpu(), reason="checks the no-GPU error path")
def test_context_creation_fails_loudly_without_gpu():
    with pytest.raises(nbg.NbgError):
        nbg.Context(0)


def test_new_entry_points_reject_null_arguments_without_a_gpu():
    L = nbg._lib.load()
    E = nbg._lib.NBG_EINVAL
    assert L.nbg_set_producer_layout(None, 4, 200, 32) == E
    assert L.nbg_set_orbit_team(None, 1) == E
    assert L.nbg_last_host_time(None, None) == E
    assert L.nbg_integrate(None, 3, 0.5, 10.0, 1, *([None] * 10)) == E
    assert L.nbg_integrate_steps(None, 3, 0.5, 10, 1, *([None] * 10)) == E
    assert L.nbg_integrate_cartesian(None, 3, 0.5, 10.0, 5, *([None] * 14)) == E
    assert L.nbg_batch_init_nbody(None, 1, None, None, None, None, None, None, None) == E
    assert L.nbg_autotune_device(None, 1, None, *([None] * 11), 64, None, 0, None) == E
    assert L.nbg_integrate_transit_parameters(None, 3, 0, 0.5, 10.0, 1, *([None] * 11), 10, None, None, None,
                                              None) == E
    assert L.nbg_server_enqueue(None, None, 0.0, *([None] * 10), None) == E
    assert L.nbg_server_stats(None, None) == E
    assert L.nbg_server_stop(None) == nbg._lib.NBG_OK
    assert L.nbg_server_cancel(None, 1) == E


def test_transit_parameters_and_cartesian_output_shapes():
    from nbg import workloads as W
    el, _, _ = W.plain_3body(0)
    ic = W.ic_of(el)
    tp = nbg.TransitParameters(1000.0, ic)
    assert tp.ntt == 103 and tp.ttbv.shape == (3, 3, 103) and tp.dtbvdq0.shape == (3, 3, 103, 7, 3)
    assert tp.occs == [2, 3]
    with pytest.raises(ValueError):
        nbg.TransitParameters(1000.0, ic, ntt=5)
    o = nbg.CartesianOutput(3, 7)
    assert o.x.shape == (7, 3, 3) and o.jac_step.shape == (7, 21, 21) and len(o.states) == 7
    assert nbg.CartesianOutput(3, 7, jac=False).jac_step is None


@pytest.mark.skipif(has_gpu(), reason="checks the no-GPU error path")
def test_server_start_fails_loudly_without_gpu():
    with pytest.raises(nbg.NbgError):
        nbg.Server()


def test_async_batch_argument_and_order_checks_without_a_gpu():
    """nbg_batch_*: NULL arguments, descriptor checks at create, and call-order errors (no run is started)."""
    import ctypes
    L = nbg._lib.load()
    E, U, OK = nbg._lib.NBG_EINVAL, nbg._lib.NBG_EUNSUPPORTED, nbg._lib.NBG_OK
    d = (nbg.SystemDesc * 2)()
    for q in range(2):
        d[q].n, d[q].ti, d[q].grad, d[q].ntt, d[q].h, d[q].tmax = 3, 0, 1, 10, 0.5, 10.0
    h = ctypes.c_void_p()
    assert L.nbg_batch_create(None, 2, d, ctypes.byref(h)) == E
    assert L.nbg_batch_submit(None, *([None] * 16)) == E
    assert L.nbg_batch_run(None) == E and L.nbg_batch_wait(None, 0) == E
    assert L.nbg_batch_destroy(None) == OK
    # create() stores the context pointer without using it, so its checks run without a GPU context
    fake_ctx = ctypes.c_void_p(1)
    assert L.nbg_batch_create(fake_ctx, 0, d, ctypes.byref(h)) == E
    assert L.nbg_batch_create(fake_ctx, 2, d, None) == E
    d[1].n = 11
    assert L.nbg_batch_create(fake_ctx, 2, d, ctypes.byref(h)) == U
    d[1].n, d[1].ti = 3, 3
    assert L.nbg_batch_create(fake_ctx, 2, d, ctypes.byref(h)) == E
    d[1].ti, d[1].h = 0, 0.0
    assert L.nbg_batch_create(fake_ctx, 2, d, ctypes.byref(h)) == E
    d[1].h = 0.5
    assert L.nbg_batch_create(fake_ctx, 2, d, ctypes.byref(h)) == OK and h.value
    assert L.nbg_batch_run(h) == E and "submitted" in nbg._lib.last_error()
    assert L.nbg_batch_wait(h, 0) == E and "not running" in nbg._lib.last_error()
    assert L.nbg_batch_submit(h, *([None] * 16)) == E
    assert L.nbg_batch_destroy(h) == OK


def test_derivatives_dstate_and_initialize_without_a_gpu():
    """dState / Derivatives / initialize (Integrator.jl:106-121) and the argument checks of intr(s, tt, d)."""
    from nbg import workloads as W
    el, h, _ = W.plain_3body(0)
    ic = W.ic_of(el)
    s, d = nbg.dState(ic)
    assert isinstance(d, nbg.Derivatives) and d.n == 3 and nbg.Derivatives(np.float64, 3).n == 3
    x0 = s.x.copy()
    s.x[...] += 1.0
    s.xerror[...] = 1e-20
    s.jac_init[...] = 0.0
    nbg.initialize(s, ic)
    assert np.array_equal(s.x, x0) and not s.xerror.any() and np.array_equal(s.jac_init, nbg.State(ic).jac_init)
    intr = nbg.Integrator(nbg.ahl21, h, 0.0, 10.0)
    tt = nbg.TransitTiming(10.0, ic)
    with pytest.raises(TypeError):
        intr(s, tt, object())
    with pytest.raises(TypeError):
        intr(s, 5.0, d)
    with pytest.raises(ValueError):
        intr(s, tt, nbg.Derivatives(4))
    with pytest.raises(TypeError):
        intr(s, tt, d, True)  # grad is keyword-only


def test_binding_argument_counts_match_the_header():
    """Every ctypes binding declares as many arguments as the header's prototype, with a compatible kind
    (integer, floating point or pointer) at each position."""
    import test_julia_shim as S
    protos = S.header_prototypes()
    L = nbg._lib.load()
    ints = {ctypes.c_int, ctypes.c_int32, ctypes.c_int64, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_uint64}
    for name in nbg._lib.EXPORTS:
        fn = getattr(L, name)
        if fn.argtypes is None:
            assert protos[name][1] == [], name  # nbg_version(void)
            continue
        ctypes_ = protos[name][1]
        assert len(fn.argtypes) == len(ctypes_), (name, len(fn.argtypes), len(ctypes_))
        for pos, (py, c) in enumerate(zip(fn.argtypes, ctypes_)):
            if c.endswith("*"):
                assert py is ctypes.c_void_p or py is ctypes.c_char_p or issubclass(py, ctypes._Pointer), (name, pos)
            elif c == "double":
                assert py is ctypes.c_double, (name, pos)
            else:
                assert py in ints, (name, pos, c)
