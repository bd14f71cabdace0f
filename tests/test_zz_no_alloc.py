"""nbg_batch_integrate_transits_noalloc: the allocation-free entry point.

It runs the same kernels as nbg_batch_integrate_transits_device with every
working buffer taken from the library's fixed scratch array.  Its results
must match the pooled entry point's within the parity tolerances, on two
calls in a row (the second call finds the first call's contents in the
shared scratch), for a mixed batch of body counts, gradient flags and
transit-timing lengths.  Named to run after every other test file, and
self-contained so that it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import nbg
import parity as P
from conftest import has_gpu

W = nbg.workloads

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not has_gpu(), reason="needs a CUDA GPU")]


def _batch():
    els, hs, tms = W.batch_uneven(20, seed=47, nmin=2, nmax=8)
    states, timings, grads = [], [], []
    for q, (el, tm) in enumerate(zip(els, tms)):
        ic = nbg.ElementsIC(0.0, el.shape[0], el)
        states.append(nbg.State(ic))
        timings.append(nbg.TransitTiming(min(tm, 60.0), ic))
        grads.append(q % 4 != 3)
    tms = [min(tm, 60.0) for tm in tms]
    b = nbg.Batch([s.n for s in states], 0, hs, tms, [t.ntt for t in timings], grads)
    for q in range(len(states)):
        b.set_system(q, states[q], timings[q])
    return b, tms


def _run(b, fn):
    import torch
    dev = {k: torch.from_numpy(a.copy()).cuda() for k, a in b.arrays.items()}
    fn(dev)
    torch.cuda.synchronize()
    return {k: t.cpu().numpy() for k, t in dev.items()}, b.status.copy()


class _S:
    pass


def _system(b, out, q):
    n = b.n[q]
    M = 7 * n
    ntt = int(b.ntt[q])
    v = lambda k: out[k][b.offsets[k][q]:b.offsets[k][q + 1]]
    s = _S()
    s.x = v("x").reshape((3, n), order="F")
    s.v = v("v").reshape((3, n), order="F")
    s.jac_step = v("jac_step").reshape((M, M), order="F")
    s.dqdt = v("dqdt")
    s.tt = v("tt").reshape((n, ntt), order="F")
    s.dtdq0 = v("dtdq0").reshape((n, ntt, 7, n), order="F")
    s.dtdelements = v("dtdelements").reshape((n, ntt, 7, n), order="F")
    s.count = v("count")
    s.t = v("t")
    s.jac_init = v("jac_init").reshape((M, M), order="F")
    return s


def _compare(b, tms, got, ref):
    for q in range(b.nsys):
        g, r = _system(b, got, q), _system(b, ref, q)
        P.check_counts(g.count, r.count)
        assert g.t[0] == r.t[0]
        P.check_tt(g.tt, r.tt, r.count, tms[q])
        P.check_state(g, r, check_jac=bool(b.grad[q]))
        if b.grad[q]:
            P.check_transit_derivs(g.dtdq0, r.dtdq0, r.count)
            P.check_transit_derivs(g.dtdelements, r.dtdelements, r.count, "dtdelements", r.dtdq0, r.jac_init)


def test_noalloc_matches_pooled_entry_point_twice():
    ctx = nbg.Context(0)
    b, tms = _batch()
    ref, ref_status = _run(b, lambda dev: b.run_device(dev, ctx))
    assert ref["count"].sum() > 0
    for _ in range(2):
        got, status = _run(b, lambda dev: b.run_device_noalloc(dev, ctx))
        assert np.array_equal(status, ref_status)
        _compare(b, tms, got, ref)


def test_noalloc_repeat_call_leaves_device_memory_unchanged():
    """After the first call on the device (which, under lazy module loading, reserves the fixed
    scratch array), a call changes the device's free memory by not one byte."""
    import torch
    ctx = nbg.Context(0)
    b, _ = _batch()
    dev = {k: torch.from_numpy(a.copy()).cuda() for k, a in b.arrays.items()}
    b.run_device_noalloc(dev, ctx)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    b.run_device_noalloc(dev, ctx)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_shrinks_its_chunk_to_fit():
    """With the context's chunk set to 4096 steps the working set cannot fit the 64 MiB scratch
    (the operator records of one 2-body gradient group alone take 4096 x 172 x 32 doubles =
    180 MB), so the call shortens its chunk; results still match the pooled entry point."""
    ctx = nbg.Context(0)
    ctx.set_tuning(chunk_steps=4096)
    ref_ctx = nbg.Context(0)
    b, tms = _batch()
    ref, ref_status = _run(b, lambda dev: b.run_device(dev, ref_ctx))
    got, status = _run(b, lambda dev: b.run_device_noalloc(dev, ctx))
    assert np.array_equal(status, ref_status)
    _compare(b, tms, got, ref)


def test_noalloc_rejects_too_many_systems():
    ctx = nbg.Context(0)
    L = nbg._lib.load()
    nsys = 129  # one more than NBG_NOALLOC_MAX_SYSTEMS
    desc = (nbg._lib.SystemDesc * nsys)()
    rc = L.nbg_batch_integrate_transits_noalloc(ctx.handle, nsys, desc, *([None] * 16))
    assert rc == nbg._lib.NBG_EINVAL
    buf = ctypes.create_string_buffer(512)
    L.nbg_last_error(buf, 512)
    assert b"NBG_NOALLOC_MAX_SYSTEMS" in buf.value
