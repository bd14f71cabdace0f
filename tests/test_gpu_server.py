"""The request server (nbg_server_* through its C ABI) on the GPU.

Requests of mixed body count, grad flag, pair pattern and length arrive
while others run; each result must be bitwise the same as the same request
served alone, bitwise the same as the batched entry point's, and within the
parity tolerances of the oracle.
"""
import threading
import time

import numpy as np
import pytest

import nbg
import oracle_lib as O
import parity as P
from conftest import has_gpu
from nbg import workloads as W

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not has_gpu(), reason="needs a CUDA GPU")]

FIELDS_S = ("t", "x", "v", "xerror", "verror", "jac_step", "jac_error", "dqdt")
FIELDS_T = ("tt", "dtdq0", "dtdelements", "count")


def make_requests(nreq=24, seed=11):
    """(State, TransitTiming, Integrator, grad) tuples: N in 2..6, 20..160 steps."""
    rng = np.random.default_rng(seed)
    els, hs, _ = W.batch_uneven(nreq, seed=seed, nmin=2, nmax=6)
    reqs = []
    for q, (el, h) in enumerate(zip(els, hs)):
        tmax = float(h * rng.integers(20, 161))
        ic = W.ic_of(el)
        s = nbg.State(ic)
        if q % 7 == 3 and s.n >= 3:
            s.pair[0, 1] = s.pair[1, 0] = 1  # a kick pair: its own group
        tt = nbg.TransitTiming(tmax, ic)
        reqs.append((s, tt, nbg.Integrator(nbg.ahl21, h, 0.0, tmax), bool(q % 2 == 0)))
    return reqs


def fresh(req):
    """A copy of the request's State and a zeroed TransitTiming of the same shape."""
    s, tt, intr, grad = req
    t2 = nbg.TransitTiming.__new__(nbg.TransitTiming)
    t2.__dict__.update(n=tt.n, ntt=tt.ntt, ti=tt.ti, occs=list(tt.occs))
    for k in ("tt", "dtdq0", "dtdelements", "count"):
        setattr(t2, k, np.zeros_like(getattr(tt, k), order="F"))
    return s.copy(), t2, intr, grad


def assert_same(a, b):
    (sa, ta), (sb, tb) = a, b
    for k in FIELDS_S:
        assert np.array_equal(getattr(sa, k), getattr(sb, k)), k
    for k in FIELDS_T:
        assert np.array_equal(getattr(ta, k), getattr(tb, k)), k


def serve_mix(srv, reqs, jitter_ms=3.0, seed=0):
    """Submit every request from a client thread at random intervals; collect all."""
    rng = np.random.default_rng(seed)
    outs = [fresh(r) for r in reqs]
    ids = [None] * len(reqs)

    def client():
        for q, (s, tt, intr, grad) in enumerate(outs):
            ids[q] = srv.submit(s, tt, intr, grad)
            time.sleep(rng.uniform(0, jitter_ms) * 1e-3)

    th = threading.Thread(target=client)
    th.start()
    th.join()
    infos = []
    for q, (s, tt, intr, grad) in enumerate(outs):
        infos.append(srv.result(ids[q], s, tt, timeout_ms=120000))
    return [(s, tt) for s, tt, _, _ in outs], infos


def test_mix_is_bitwise_alone_and_batched():
    reqs = make_requests()
    with nbg.Server(slots_per_group=32, chunk_steps=16) as srv:
        mix, infos = serve_mix(srv, reqs)
        assert all(i["rc"] == 0 for i in infos)
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["running"] == 0 and st["pending"] == 0
        assert st["groups"] >= 4
        # each request alone on the same server
        for q, r in enumerate(reqs):
            s, tt, intr, grad = fresh(r)
            srv.result(srv.submit(s, tt, intr, grad), s, tt, timeout_ms=120000)
            assert_same(mix[q], (s, tt))
    # the batched entry point gives the same bits
    for q, r in enumerate(reqs):
        s, tt, intr, grad = fresh(r)
        b = nbg.Batch([s.n], [tt.ti - 1], intr.h, intr.tmax, [tt.ntt], grad)
        b.set_system(0, s, tt)
        b.run()
        b.get_system(0, s, tt)
        assert_same(mix[q], (s, tt))


def test_refilled_slots_are_bitwise_alone():
    """96 short 3-body gradient requests in one group of 32 slots: slots retire and are refilled two chunks later
    while the previous chunk's operator and Jacobian kernels still run on the group's other streams; every result
    is bitwise the one of the same request alone (nbg_integrate_transits)."""
    rng = np.random.default_rng(23)
    els, hs, _ = W.batch_uneven(96, seed=23, nmin=3, nmax=3)
    reqs = []
    for el, h in zip(els, hs):
        tmax = float(h * rng.integers(20, 81))
        ic = W.ic_of(el)
        reqs.append((nbg.State(ic), nbg.TransitTiming(tmax, ic), nbg.Integrator(nbg.ahl21, h, 0.0, tmax), True))
    with nbg.Server(slots_per_group=32, chunk_steps=8, max_inflight=3) as srv:
        mix, infos = serve_mix(srv, reqs, jitter_ms=0.2, seed=4)
        st = srv.stats()
    assert all(i["rc"] == 0 for i in infos)
    assert st["groups"] == 1 and st["admitted"] == len(reqs)  # 96 requests through 32 slots: slots were reused
    assert max(i["queue_ms"] for i in infos) > 0.0
    for q, r in enumerate(reqs):
        s1, tt1, intr, _ = fresh(r)
        intr(s1, tt1, grad=True)
        assert_same(mix[q], (s1, tt1))


def test_served_results_match_oracle():
    reqs = make_requests(8, seed=5)
    with nbg.Server(slots_per_group=32, chunk_steps=8) as srv:
        mix, _ = serve_mix(srv, reqs, seed=1)
    for (s, tt), (s0, tt0, intr, grad) in zip(mix, reqs):
        so = O.OState(s0.x, s0.v, s0.m, jac_init=s0.jac_init, t=0.0, pair=s0.pair)
        to = O.OTiming(s0.n, tt0.ntt, 0)
        O.integrate_transits(so, to, intr.h, intr.tmax, grad=grad)
        P.check_counts(tt.count, to.count)
        P.check_tt(tt.tt, to.tt, to.count, intr.tmax)
        assert s.t[0] == so.t[0]
        P.check_state(s, so, check_jac=grad)
        if grad:
            P.check_transit_derivs(tt.dtdq0, to.dtdq0, to.count, "dtdq0")
            P.check_transit_derivs(tt.dtdelements, to.dtdelements, to.count, "dtdelements", to.dtdq0, so.jac_init)


def test_full_length_requests_and_latency_record():
    """Two full plain_3body requests (2000 steps) in the mix with short ones; latency fields are consistent."""
    el, h, tmax = W.plain_3body(0)
    longs = []
    for _ in range(2):
        ic = W.ic_of(el)
        longs.append((nbg.State(ic), nbg.TransitTiming(tmax, ic), nbg.Integrator(nbg.ahl21, h, 0.0, tmax), True))
    reqs = longs + make_requests(6, seed=3)
    with nbg.Server(slots_per_group=64) as srv:
        mix, infos = serve_mix(srv, reqs, seed=2)
    for inf in infos:
        assert inf["latency_ms"] >= inf["run_ms"] >= 0.0 and inf["queue_ms"] >= 0.0
        assert abs(inf["latency_ms"] - inf["queue_ms"] - inf["run_ms"]) < 1e-6 * max(1.0, inf["latency_ms"]) + 1e-3
    assert infos[0]["nsteps"] == 2000
    s, tt = mix[0]
    assert tt.count.sum() > 100
    # the same request through nbg_integrate_transits
    s1, tt1, intr, _ = fresh(reqs[0])
    intr(s1, tt1, grad=True)
    assert_same((s, tt), (s1, tt1))


def test_request_argument_errors():
    """Malformed requests are rejected at enqueue; unknown ids and empty waits report their own codes."""
    with nbg.Server(slots_per_group=32) as srv:
        el, h, tmax = W.plain_3body(1)
        ic = W.ic_of(el)
        s = nbg.State(ic)
        tt = nbg.TransitTiming(tmax, ic)
        tt.count[0] = 1
        with pytest.raises(ValueError):
            srv.submit(s, tt, nbg.Integrator(nbg.ahl21, h, 0.0, tmax))
        with pytest.raises(nbg.NbgError) as ei:
            srv.result(123456, s, tt, timeout_ms=0)
        assert ei.value.code == nbg._lib.NBG_EINVAL
        with pytest.raises(nbg.NbgError) as ei:
            srv.wait_any(timeout_ms=10)
        assert ei.value.code == nbg._lib.NBG_ETIMEOUT
        with pytest.raises(nbg.NbgError) as ei:
            srv.cancel(123456)
        assert ei.value.code == nbg._lib.NBG_EINVAL


def _long_3body(nreq, seed, steps=2000):
    """nreq 3-body gradient requests of `steps` steps (one group)."""
    els, hs, _ = W.batch_uneven(nreq, seed=seed, nmin=3, nmax=3)
    out = []
    for el, h in zip(els, hs):
        ic = W.ic_of(el)
        tmax = float(h * steps)
        out.append((nbg.State(ic), nbg.TransitTiming(tmax, ic), nbg.Integrator(nbg.ahl21, h, 0.0, tmax), True))
    return out


def _wait_admitted(srv, n, timeout_s=60.0):
    t0 = time.time()
    while srv.stats()["admitted"] < n:
        assert time.time() - t0 < timeout_s, srv.stats()
        time.sleep(0.002)


def _alone(req):
    s, tt, intr, grad = fresh(req)
    intr(s, tt, grad=grad)
    return s, tt


def test_cancel_waiting_and_running_requests():
    """32 slots hold 32 long requests; of 4 more that wait for a slot one is cancelled while waiting, and
    one of the running requests is cancelled mid-integration.  Both report NBG_ECANCELLED; every other
    request completes bitwise as alone, including the one admitted into the cancelled request's slot;
    cancelling a request that has finished is refused and leaves its result intact."""
    reqs = _long_3body(36, seed=51)
    with nbg.Server(slots_per_group=32, chunk_steps=8) as srv:
        outs = [fresh(r) for r in reqs]
        ids = [srv.submit(s, tt, intr, grad) for s, tt, intr, grad in outs]
        _wait_admitted(srv, 32)
        assert srv.stats()["pending"] == 4
        srv.cancel(ids[33])  # waiting for a slot
        srv.cancel(ids[5])   # running
        for q in (5, 33):
            s, tt, _, _ = outs[q]
            with pytest.raises(nbg.NbgError) as ei:
                srv.result(ids[q], s, tt, timeout_ms=120000)
            assert ei.value.code == nbg._lib.NBG_ECANCELLED
        infos = {}
        for q in range(36):
            if q in (5, 33):
                continue
            s, tt, _, _ = outs[q]
            infos[q] = srv.result(ids[q], s, tt, timeout_ms=120000)
        st = srv.stats()
        assert st["completed"] == 34 and st["failed"] == 2 and st["running"] == 0 and st["pending"] == 0
        # a finished request cannot be cancelled: the refusal leaves it collectable
        s, tt, intr, grad = fresh(reqs[0])
        rid = srv.submit(s, tt, intr, grad)
        srv.result(rid, s, tt, timeout_ms=120000)
        with pytest.raises(nbg.NbgError) as ei:
            srv.cancel(rid)
        assert ei.value.code == nbg._lib.NBG_EINVAL
    for q in (0, 6, 31, 32, 34, 35):
        assert_same((outs[q][0], outs[q][1]), _alone(reqs[q]))


def test_stop_cancels_requests_not_yet_admitted():
    """nbg_server_stop with requests still waiting for a slot: threads collecting them get
    NBG_ECANCELLED, the running requests run to completion, and stop returns cleanly."""
    reqs = _long_3body(35, seed=52)
    srv = nbg.Server(slots_per_group=32, chunk_steps=8)
    outs = [fresh(r) for r in reqs]
    ids = [srv.submit(s, tt, intr, grad) for s, tt, intr, grad in outs]
    _wait_admitted(srv, 32)
    codes = {}

    def collect(q):
        s, tt, _, _ = outs[q]
        try:
            srv.result(ids[q], s, tt, timeout_ms=120000)
            codes[q] = 0
        except nbg.NbgError as e:
            codes[q] = e.code

    threads = [threading.Thread(target=collect, args=(q,)) for q in (32, 33, 34)]
    for t in threads:
        t.start()
    time.sleep(0.05)
    srv.stop()
    for t in threads:
        t.join(timeout=60)
    assert codes == {32: nbg._lib.NBG_ECANCELLED, 33: nbg._lib.NBG_ECANCELLED, 34: nbg._lib.NBG_ECANCELLED}


def test_output_arena_too_small_requests_wait_then_complete():
    """An HBM budget whose output half holds one request's outputs at a time (transit arrays of
    ntt = 20000): four requests are admitted one after another, each waiting for the previous one's
    outputs to be released, and all complete bitwise as alone."""
    els, hs, _ = W.batch_uneven(4, seed=53, nmin=3, nmax=3)
    big = []
    for el, h in zip(els, hs):
        ic = W.ic_of(el)
        tmax = float(h * 400)
        big.append((nbg.State(ic), nbg.TransitTiming(tmax, ic, ntt=20000), nbg.Integrator(nbg.ahl21, h, 0.0, tmax),
                    True))
    # the group's slot buffers, measured on a server with room to spare
    with nbg.Server(slots_per_group=32, chunk_steps=8) as probe:
        s, tt, intr, grad = fresh(big[0])
        probe.result(probe.submit(s, tt, intr, grad), s, tt, timeout_ms=120000)
        group_bytes = probe.stats()["hbm_groups"]
    out_bytes = 8 * (3 * 20000 + 2 * 7 * 9 * 20000)  # tt, dtdq0, dtdelements of one request
    half = max(group_bytes, int(1.5 * out_bytes))
    with nbg.Server(slots_per_group=32, chunk_steps=8, hbm_budget_bytes=2 * half) as srv:
        outs = [fresh(r) for r in big]
        ids = [srv.submit(s, tt, intr, grad) for s, tt, intr, grad in outs]
        infos = [srv.result(i, o[0], o[1], timeout_ms=120000) for i, o in zip(ids, outs)]
    assert all(i["rc"] == 0 for i in infos)
    runs = sorted(infos, key=lambda i: i["queue_ms"])
    # one at a time: each later request waited at least most of an earlier one's run
    for k in range(1, 4):
        assert runs[k]["queue_ms"] >= 0.5 * runs[k - 1]["run_ms"], [(i["queue_ms"], i["run_ms"]) for i in runs]
    for q in range(4):
        assert_same((outs[q][0], outs[q][1]), _alone(big[q]))


def test_group_larger_than_budget_fails_with_enomem():
    """A 2 MB budget: a 3-body gradient group's slot buffers (its two halves of operator records alone
    take 2 MB) do not fit the 1 MB group half, so the request fails NBG_ENOMEM; a gradient-free group
    fits, but a request whose outputs (ntt = 60000: 1.4 MB) exceed the 1 MB output arena fails the same
    way; the server keeps serving and counts both failures."""
    with nbg.Server(slots_per_group=32, chunk_steps=8, hbm_budget_bytes=2 * 1024 * 1024) as srv:
        s, tt, intr, grad = fresh(_long_3body(1, seed=54, steps=100)[0])
        with pytest.raises(nbg.NbgError) as ei:
            srv.result(srv.submit(s, tt, intr, grad), s, tt, timeout_ms=120000)
        assert ei.value.code == nbg._lib.NBG_ENOMEM
        el, h, _ = W.plain_3body(2)
        ic = W.ic_of(el)
        s2, tt2 = nbg.State(ic), nbg.TransitTiming(10 * h, ic, ntt=60000)
        with pytest.raises(nbg.NbgError) as ei:
            srv.result(srv.submit(s2, tt2, nbg.Integrator(nbg.ahl21, h, 0.0, 10 * h), False), s2, tt2,
                       timeout_ms=120000)
        assert ei.value.code == nbg._lib.NBG_ENOMEM
        assert srv.stats()["failed"] == 2
