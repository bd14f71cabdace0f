"""Parity at the benchmark configurations' full integration spans.

Each test integrates a whole benchmark batch on the GPU, over every system's
own full span, and compares a sample of its systems with the oracle run over
the same span on host threads (concurrently with the GPU run):

  * batch_3body  (4096 x 3 bodies, h = 0.5 d, 1000 d): 32 systems;
  * batch_8body  (1024 x 8 bodies, h = 0.06 d, 1600 d = 26 667 steps):
    8 systems, the first and the last among them;
  * batch_uneven (2048 systems, N = 2..10, up to 77 k steps): the longest
    system of each body count from 8 to 10 and of the 9- and 10-body systems
    over 3000 d, and the shortest system of every body count.

Gates.  batch_3body uses the tolerances of tests/parity.py: tt within 1e-10
of the span, dtdq0 and dtdelements within 1e-8 relative entry by entry (with
the floor of 1e-4 of the transit row's scale).

The two long spans (batch_8body over 26 667 steps, batch_uneven up to 77 k)
are chaotic enough that FP64 does not reproduce them to those tolerances:
the oracle built on x86-64 and on AArch64 (same source, different libm)
disagrees with itself as much as the GPU disagrees with it.  They keep the
tt gate (1e-10 of the span) and identical counts, and measure everything
else against the reference's own reproducibility, which the test measures:
each sampled system is also run through the oracle with one initial
coordinate moved by one ulp.  A transit row (body j, transit c) of dtdq0 or
dtdelements passes when its largest deviation from the oracle, relative to
the row's largest entry (the maxabs norm of the reference's own test,
test/test_transit_timing.jl:87-88, applied per row), is within 1e-8, or
within 10 times the relative deviation that the one-ulp change causes in the
oracle's own rows up to that time.  x, v and each jac_step column follow the
same rule (1e-10 for x and v, 1e-8 per column).  The entrywise figures are
measured and reported.

Each test writes its worst ratios (error / tolerance, 1.0 = at the bound) to
the JSON-lines file named by NBG_PARITY_REPORT when that variable is set.

The oracle multiplies its operators with the exact-zero entries skipped:
bitwise the same results as its dense products (tests/test_oracle_pins.py),
several times faster at 8-10 bodies.
"""
import json
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import nbg
import oracle_lib as O
import parity as P
from conftest import has_gpu
from nbg import workloads as W

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not has_gpu(), reason="needs a CUDA GPU")]


def _report(name, **vals):
    path = os.environ.get("NBG_PARITY_REPORT")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps(dict(test=name, **vals)) + "\n")


ULP_FACTOR = 10.0


def _oracle_runs(jobs):
    """Runs (state, h, tmax, ntt, perturbed) jobs through the oracle on host threads; returns a future
    of [(OState, OTiming)].  A perturbed job moves the first planet's x coordinate up by one ulp.
    ctypes releases the GIL, so the GPU run proceeds meanwhile."""
    threads = max(1, (os.cpu_count() or 2) - 2)

    def one(job):
        s, h, tmax, ntt, pert = job
        x = s.x.copy(order="F")
        if pert:
            x[0, 1] = np.nextafter(x[0, 1], np.inf)
        so = O.OState(x, s.v, s.m, jac_init=s.jac_init)
        to = O.OTiming(s.n, ntt, 0)
        O.integrate_transits(so, to, h, tmax)
        return so, to

    ex = ThreadPoolExecutor(max_workers=min(threads, len(jobs)))
    cm = O.skip_zero_products()
    cm.__enter__()
    futs = [ex.submit(one, j) for j in jobs]

    class Runs:
        def result(self):
            try:
                return [f.result() for f in futs]
            finally:
                ex.shutdown()
                cm.__exit__(None, None, None)

    return Runs()


def _gpu_batch(states, hs, tms, ntts):
    b = nbg.Batch([s.n for s in states], 0, hs, tms, ntts, True)
    for q, s in enumerate(states):
        b.set_system(q, s)
    return b


def _rows_within_reproducibility(gpu, ref, alt, tt, count, name):
    """Per transit row: the relative deviation e of gpu from ref and the one-ulp oracle's relative
    deviation d from ref, rows in time order; a row passes when e <= max(1e-8, ULP_FACTOR * (largest d
    so far)).  Returns (worst e / 1e-8, rows passing only through the reproducibility bound)."""
    rows = []
    for j, c in enumerate(count):
        for t in range(min(int(c), gpu.shape[1])):
            s = float(np.max(np.abs(ref[j, t])))
            if s == 0.0:
                assert np.all(gpu[j, t] == 0.0), (name, j, t)
                continue
            rows.append((float(tt[j, t]), j, t, float(np.max(np.abs(gpu[j, t] - ref[j, t]))) / s,
                         float(np.max(np.abs(alt[j, t] - ref[j, t]))) / s))
    rows.sort()
    env, worst, by_env = 0.0, 0.0, 0
    for time, j, t, e, d in rows:
        env = max(env, d)
        worst = max(worst, e / P.DT_RTOL)
        if e > P.DT_RTOL:
            by_env += 1
            assert e <= ULP_FACTOR * env, ("%s[%d,%d] at t = %.3f: deviation %.3g of the row scale, beyond 1e-8 and "
                                           "beyond %g x the one-ulp spread so far (%.3g)" % (name, j, t, time, e,
                                                                                             ULP_FACTOR, env))
    return worst, by_env


def _compare_system(b, q, so, to, tmax, normwise, alt=None):
    """Worst tolerance ratios of system q of the GPU batch against the oracle run (normwise: the
    transit derivatives per transit row, with alt = the one-ulp oracle run; else entry by entry)."""
    n = int(b.n[q])
    ntt = int(b.ntt[q])
    M = 7 * n
    P.check_counts(b.view("count", q), to.count)
    err_tt = P.check_tt(b.view("tt", q).reshape((n, ntt), order="F"), to.tt, to.count, tmax)
    g_dq = b.view("dtdq0", q).reshape((n, ntt, 7, n), order="F")
    g_de = b.view("dtdelements", q).reshape((n, ntt, 7, n), order="F")
    out = {"n": n, "transits": int(to.count.sum()), "tt": err_tt / (P.TT_TOL * abs(tmax))}
    if normwise:
        so_a, to_a = alt
        out["dtdq0"], out["dtdq0_rows_by_ulp_bound"] = _rows_within_reproducibility(
            g_dq, to.dtdq0, to_a.dtdq0, to.tt, to.count, "dtdq0")
        out["dtdelements"], out["dtdelements_rows_by_ulp_bound"] = _rows_within_reproducibility(
            g_de, to.dtdelements, to_a.dtdelements, to.tt, to.count, "dtdelements")
        a = _excess(g_dq, to.dtdq0, to.count)
        e = _excess(g_de, to.dtdelements, to.count, to.dtdq0, so.jac_init)
        out["entrywise"] = {"dtdq0_beyond": a[1], "dtdq0_checked": a[0], "dtdq0_worst": a[2],
                            "dtdelements_beyond": e[1], "dtdelements_worst": e[2]}
    else:
        out["dtdq0"] = P.check_transit_derivs(g_dq, to.dtdq0, to.count)
        out["dtdelements"] = P.check_transit_derivs(g_de, to.dtdelements, to.count, "dtdelements", to.dtdq0,
                                                    so.jac_init)
    gs = type("S", (), {})()
    gs.x = b.view("x", q).reshape((3, n), order="F")
    gs.v = b.view("v", q).reshape((3, n), order="F")
    gs.jac_step = b.view("jac_step", q).reshape((M, M), order="F")
    gs.dqdt = b.view("dqdt", q)
    if not normwise:
        P.check_state(gs, so)
    else:
        st = _state_ratios(gs, so)
        sp = _state_ratios(so_a, so)
        out["state"] = st
        out["state_one_ulp"] = sp
        assert st["x"] <= max(1e-10, ULP_FACTOR * sp["x"]), (st, sp)
        assert st["v"] <= max(1e-10, ULP_FACTOR * sp["v"]), (st, sp)
        assert st["jac_step_columns"] <= max(1e-8, ULP_FACTOR * sp["jac_step_columns"]), (st, sp)
    return out


def _state_ratios(gs, rs):
    """Final-state deviations relative to each array's scale (x, v) and to each jac_step column's."""
    r = {}
    for k in ("x", "v"):
        g, f = getattr(gs, k), getattr(rs, k)
        r[k] = float(np.max(np.abs(g - f)) / np.max(np.abs(f)))
    colmax = np.max(np.abs(rs.jac_step), axis=0)
    r["jac_step_columns"] = float(np.max(np.max(np.abs(gs.jac_step - rs.jac_step), axis=0) / colmax))
    return r


def _excess(gpu, ref, count, dtdq0=None, jac_init=None):
    """Entries of a transit-derivative array beyond the tests/parity.py tolerance: (entries checked,
    entries beyond, worst ratio, largest |entry| / row scale among those beyond)."""
    n, ntt = gpu.shape[0], gpu.shape[1]
    checked = beyond = 0
    worst = big = 0.0
    for j, c in enumerate(count):
        for t in range(min(int(c), ntt)):
            r, g = ref[j, t], gpu[j, t]
            s = float(np.max(np.abs(r)))
            if s == 0.0:
                continue
            mag = np.abs(r)
            if dtdq0 is not None:
                mag = mag + (np.abs(dtdq0[j, t]).ravel(order="F") @ np.abs(jac_init)).reshape((7, n), order="F")
            ratio = np.abs(g - r) / (P.DT_RTOL * (mag + P.DT_FLOOR * s))
            checked += ratio.size
            over = ratio > 1.0
            beyond += int(np.count_nonzero(over))
            worst = max(worst, float(np.max(ratio)))
            if over.any():
                big = max(big, float(np.max(np.abs(r[over]))) / s)
    return checked, beyond, worst, big


def _failure_stats(b, q, so, to):
    n, ntt = int(b.n[q]), int(b.ntt[q])
    g_dq = b.view("dtdq0", q).reshape((n, ntt, 7, n), order="F")
    g_de = b.view("dtdelements", q).reshape((n, ntt, 7, n), order="F")
    a = _excess(g_dq, to.dtdq0, to.count)
    e = _excess(g_de, to.dtdelements, to.count, to.dtdq0, so.jac_init)
    return ("dtdq0: %d of %d entries beyond, worst %.3g x, largest such entry %.2g of its row scale; "
            "dtdelements: %d of %d beyond, worst %.3g x, largest %.2g of its row scale" % (a[1], a[0], a[2], a[3],
                                                                                         e[1], e[0], e[2], e[3]))


def _dump(name, q, b, so, to):
    """Both sides of a failing system, for offline study (NBG_PARITY_DUMP: a directory)."""
    d = os.environ.get("NBG_PARITY_DUMP")
    if not d:
        return
    os.makedirs(d, exist_ok=True)
    arr = {"gpu_" + k: b.view(k, q) for k in ("x", "v", "tt", "dtdq0", "dtdelements", "count", "jac_step")}
    arr.update(ref_x=so.x, ref_v=so.v, ref_tt=to.tt, ref_dtdq0=to.dtdq0, ref_dtdelements=to.dtdelements,
               ref_count=to.count, ref_jac_step=so.jac_step, jac_init=so.jac_init)
    np.savez_compressed(os.path.join(d, "%s_system%d.npz" % (name, q)), **arr)


def _run_and_compare(name, states, hs, tms, ntts, sample, normwise=False):
    jobs = [(states[q], hs[q], tms[q], ntts[q], False) for q in sample]
    if normwise:
        jobs += [(states[q], hs[q], tms[q], ntts[q], True) for q in sample]
    runs = _oracle_runs(jobs)
    b = _gpu_batch(states, hs, tms, ntts)
    b.run()
    # NTT_OVERFLOW is the reference's own behaviour (transits beyond ntt counted and dropped, the counts
    # are compared below); a non-finite system is a failure
    nonfinite = np.nonzero(b.status & nbg._lib.NBG_STATUS_NONFINITE)[0]
    assert len(nonfinite) == 0, "non-finite systems: %s" % nonfinite.tolist()
    overflow = np.nonzero(b.status & nbg._lib.NBG_STATUS_NTT_OVERFLOW)[0].tolist()
    results = runs.result()
    alts = results[len(sample):] if normwise else [None] * len(sample)
    rows, failures = [], []
    for q, (so, to), alt in zip(sample, results[:len(sample)], alts):
        try:
            r = _compare_system(b, q, so, to, tms[q], normwise, alt)
        except AssertionError as e:
            failures.append("system %d (n = %d, %d steps): %s [%s]" % (q, int(b.n[q]), abs(round(tms[q] / hs[q])), e,
                                                                        _failure_stats(b, q, so, to)))
            _dump(name, q, b, so, to)
            continue
        r.update(system=int(q), steps=int(abs(round(tms[q] / hs[q]))))
        rows.append(r)
    worst = {k: max([r[k] for r in rows] or [0.0]) for k in ("tt", "dtdq0", "dtdelements")}
    _report(name, systems=len(states), sample=len(sample), worst=worst, rows=rows, failures=failures,
            ntt_overflow_systems=overflow)
    assert not failures, "\n".join(failures)
    return worst


def test_c1_full_batch_sample_of_32():
    """batch_3body: 4096 systems x 2000 steps; 32 systems spread over the batch against the oracle."""
    els, h, tmax = W.batch_3body(4096, seed=0)
    states = [nbg.State(W.ic_of(el)) for el in els]
    ntt = nbg.TransitTiming(tmax, W.ic_of(els[0])).ntt
    sample = sorted(set(np.linspace(0, len(els) - 1, 32).astype(int).tolist()))
    worst = _run_and_compare("batch_3body", states, [h] * len(els), [tmax] * len(els), [ntt] * len(els), sample)
    assert max(worst.values()) <= 1.0


def test_c2_full_span():
    """batch_8body: 1024 systems x 26 667 steps (1600 d); 8 systems, q = 0 and 1023 among them."""
    els, h, tmax = W.batch_8body(1024, seed=0)
    states = [nbg.State(W.ic_of(el)) for el in els]
    # every system's periods are within a few 1e-3 of each other: one transit array shape, with margin
    ntt = max(nbg.TransitTiming(tmax, W.ic_of(el)).ntt for el in els) + 2
    sample = [0, 1, 146, 292, 511, 731, 877, 1023]
    worst = _run_and_compare("batch_8body", states, [h] * len(els), [tmax] * len(els), [ntt] * len(els), sample,
                             normwise=True)
    assert worst["tt"] <= 1.0  # the derivative rows are gated inside, against 1e-8 or the one-ulp spread


def test_c3_full_span_longest_and_shortest():
    """batch_uneven: 2048 systems, N = 2..10, every system over its own span (up to 77 k steps): the
    longest system of N = 8, 9 and 10, the longest 9- and 10-body systems beyond 3000 d, and the
    shortest system of every body count against the oracle."""
    els, hs, tms = W.batch_uneven(2048, seed=0)
    ics = [W.ic_of(el) for el in els]
    states = [nbg.State(ic) for ic in ics]
    ntts = [nbg.TransitTiming(tm, ic).ntt for tm, ic in zip(tms, ics)]
    ns = np.array([s.n for s in states])
    steps = np.array([abs(round(t / h)) for t, h in zip(tms, hs)])
    sample = set()
    for n in (8, 9, 10):
        idx = np.where(ns == n)[0]
        sample.add(int(idx[np.argmax(steps[idx])]))
    for n in (9, 10):
        idx = np.where((ns == n) & (np.array(tms) > 3000.0))[0]
        sample.add(int(idx[np.argmax(steps[idx])]))
    for n in range(2, 11):
        idx = np.where(ns == n)[0]
        sample.add(int(idx[np.argmin(steps[idx])]))
    sample = sorted(sample, key=lambda q: -steps[q])  # longest oracle runs first
    worst = _run_and_compare("batch_uneven", states, hs, tms, ntts, sample, normwise=True)
    assert worst["tt"] <= 1.0  # the derivative rows are gated inside, against 1e-8 or the one-ulp spread
