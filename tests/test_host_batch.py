"""The Python Batch's packed layout (host logic only, no GPU): systems of mixed
body counts back to back in the C ABI's batched layout (include/nbg.h)."""
import numpy as np
import pytest

import nbg
from nbg import workloads as W


def _filled_inputs(els, tms, seed=0):
    """States and TransitTimings with every field set to distinct values."""
    rng = np.random.default_rng(seed)
    states, timings = [], []
    for el, tm in zip(els, tms):
        ic = W.ic_of(el)
        s, t = nbg.State(ic), nbg.TransitTiming(tm, ic)
        for k in ("x", "v", "xerror", "verror", "jac_step", "jac_error", "jac_init", "dqdt"):
            getattr(s, k)[...] = rng.standard_normal(getattr(s, k).shape)
        s.pair[...] = rng.integers(0, 2, s.pair.shape)
        s.t[0] = rng.standard_normal()
        for k in ("tt", "dtdq0", "dtdelements"):
            getattr(t, k)[...] = rng.standard_normal(getattr(t, k).shape)
        t.count[...] = rng.integers(0, 5, t.count.shape)
        states.append(s)
        timings.append(t)
    return states, timings


def test_batch_packing_round_trip():
    """Offsets are the documented running sums, descriptors carry each system's settings, and set_system /
    get_system round-trip every field bitwise."""
    els, hs, tms = W.batch_uneven(5, seed=3, nmin=2, nmax=6)
    states, timings = _filled_inputs(els, tms)
    ti, grad = [0, 1, 0, 1, 0], [True, False, True, True, False]
    b = nbg.Batch([s.n for s in states], ti, hs, tms, [t.ntt for t in timings], grad)
    for q in range(5):
        b.set_system(q, states[q], timings[q])
    n = np.array([s.n for s in states], dtype=np.int64)
    ntt = np.array([t.ntt for t in timings], dtype=np.int64)
    assert b.offsets["x"][3] == 3 * n[:3].sum()
    assert b.offsets["dtdq0"][4] == (7 * n[:4] ** 2 * ntt[:4]).sum()
    assert b.offsets["jac_step"][-1] == (49 * n ** 2).sum() and b.offsets["tt"][-1] == (n * ntt).sum()
    d = b.descriptors()
    assert [d[q].n for q in range(5)] == list(n) and [d[q].ti for q in range(5)] == ti
    assert [d[q].grad for q in range(5)] == [int(g) for g in grad]
    assert [d[q].h for q in range(5)] == list(hs) and [d[q].tmax for q in range(5)] == list(tms)
    assert [d[q].ntt for q in range(5)] == list(ntt)
    for q in range(5):
        ic = W.ic_of(els[q])
        s2, t2 = nbg.State(ic), nbg.TransitTiming(tms[q], ic)
        b.get_system(q, s2, t2)
        for k in ("t", "x", "v", "xerror", "verror", "jac_step", "jac_error", "dqdt"):
            assert np.array_equal(getattr(s2, k), getattr(states[q], k)), (q, k)
        for k in ("tt", "dtdq0", "dtdelements", "count"):
            assert np.array_equal(getattr(t2, k), getattr(timings[q], k)), (q, k)
        # inputs only: packed as the State holds them
        assert np.array_equal(b.view("pair", q), states[q].pair.ravel(order="F"))
        assert np.array_equal(b.view("jac_init", q), states[q].jac_init.ravel(order="F"))


def test_batch_rejects_a_mismatched_state():
    els, hs, tms = W.batch_uneven(2, seed=5, nmin=3, nmax=3)
    b = nbg.Batch([3, 3], 0, hs, tms, 200)
    el4, _, _ = W.batch_uneven(1, seed=6, nmin=4, nmax=4)
    s4 = nbg.State(W.ic_of(el4[0]))
    with pytest.raises(ValueError):
        b.set_system(0, s4)
