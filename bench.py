#!/usr/bin/env python3
"""Benchmark: batched AHL21 integration with Jacobian and transit timing (grad=true).

Metric: system-steps/s, the number of AHL21 steps of all systems
(sum over systems of round(tmax/h); transit-Newton sub-steps are not counted)
divided by the time of one pass over the workload.  One bench "step" is one
full integration of the whole synthetic batch: intr(s, tt; grad=true) for
every system.

Default workload (the configuration the metric is quoted on): batch_3body,
4096 3-body systems, h = 0.5 d, tmax = 1000 d (2000 steps each).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Arms:
  gb300      libnbg_cuda through its C ABI.  `value`: inputs already resident
             in HBM (nbg_batch_integrate_transits_device); `e2e`: the host API
             (nbg_batch_integrate_transits) on pinned host buffers with the
             host<->device copies inside the timed region.
  reference  the CPU restatement of the reference (oracle/, built from C++,
             Julia is not available) on all host cores, on a bounded sample of
             the same workload.

Under torchrun each rank integrates its own replica of the workload on its
own GPU (weak scaling, no collective on the data path); value is the sum of
all ranks' system-steps over the maximum rank time.
"""
import argparse
import ctypes
import importlib.util
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

# 32 hardware work queues for the library's per-group streams, set before
# torch creates the CUDA context (the library and package set the same default)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(ROOT, "nbodygradient.jl_gb300")


def load_package():
    if "nbg" in sys.modules:
        return sys.modules["nbg"]
    spec = importlib.util.spec_from_file_location("nbg", os.path.join(PKG_DIR, "__init__.py"),
                                                  submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["nbg"] = mod
    spec.loader.exec_module(mod)
    return mod


def flops_per_system_step(n):
    """Algorithmic FP64 flops of the Jacobian consumer per system-step (FMA = 2).

    Per column of jac_step and step: 2P pair updates of 132 flops (6 differences,
    a 6x6 product u = K D (66), the two mass-ratio scalings (12) and the Kahan
    sums of 12 rows (48)); the phi block 3N x 3N (18 N^2) with its Kahan sums
    (12 N); two drifts (30 N).  The zero-addend folds of 6N, 3N and 6N rows
    count one add per row (15 N): the warp tests s + e and runs the fold's
    other two adds only when one would change a row, which after a
    compensated add it almost never does.  7N columns.
    """
    P = n * (n - 1) // 2
    per_col = 2 * P * 132 + 18 * n * n + 57 * n
    return per_col * 7 * n


def build_workload(nbg, name, nsys=None, seed=0, tmax_override=0.0, bodies=0):
    W = nbg.workloads
    if name == "batch_3body":
        els, h, tmax = W.batch_3body(nsys or 4096, seed)
        hs, tms = [h] * len(els), [tmax] * len(els)
    elif name == "batch_8body":
        els, h, tmax = W.batch_8body(nsys or 1024, seed)
        hs, tms = [h] * len(els), [tmax] * len(els)
    elif name == "batch_uneven":
        els, hs, tms = W.batch_uneven(nsys or 2048, seed, nmin=bodies or 2, nmax=bodies or 10)
    elif name == "plain_3body":
        el, h, tmax = W.plain_3body(seed)
        els, hs, tms = [el], [h], [tmax]
    else:
        raise SystemExit("unknown workload %s" % name)
    if tmax_override > 0:  # a shorter integration of the same systems (profiling captures)
        tms = [tmax_override] * len(els)
    states, ics = [], []
    for el in els:
        ic = W.ic_of(el)
        ics.append(ic)
        states.append(nbg.State(ic))
    # one transit-array shape per body count (the CPU baseline packs equal shapes)
    ntt_n = {}
    for ic, tmax in zip(ics, tms):
        ntt_n[ic.nbody] = max(ntt_n.get(ic.nbody, 0), nbg.TransitTiming(tmax, ic).ntt)
    timings = [nbg.TransitTiming(tmax, ic, ntt=ntt_n[ic.nbody]) for ic, tmax in zip(ics, tms)]
    nsteps = [abs(int(np.rint(t / h))) for t, h in zip(tms, hs)]
    return states, timings, hs, tms, nsteps


def make_batch(nbg, states, timings, hs, tms, pinned=False):
    b = nbg.Batch([s.n for s in states], [t.ti - 1 for t in timings], hs, tms, [t.ntt for t in timings], True)
    if pinned:
        import torch
        for k, a in list(b.arrays.items()):
            t = torch.empty(a.shape, dtype=getattr(torch, str(a.dtype)), pin_memory=True)
            b.arrays[k] = t.numpy()
            b.arrays[k][...] = 0
            b.__dict__.setdefault("_pinned", []).append(t)
    for q in range(len(states)):
        b.set_system(q, states[q], timings[q])
    return b


class ClockSampler:
    """nvidia-smi SM clock / throttle-reason sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) >= 9:
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(nbg, states, timings, hs, tms, nsteps, target_s=12.0, nthreads=None):
    """The oracle (CPU restatement of the reference), batched over host threads, on a sample."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O
    O.build()
    L = O.lib()
    nthreads = nthreads or os.cpu_count() or 1
    # calibrate on one system, then size the sample to ~target_s of wall time
    total_ss, total_t, used = 0, 0.0, 0
    sample = max(1, nthreads)
    q = 0
    while total_t < target_s and q < len(states):
        idx = [(q + r) % len(states) for r in range(sample)]
        q += sample
        b = make_batch(nbg, [states[i] for i in idx], [timings[i] for i in idx], [hs[i] for i in idx],
                       [tms[i] for i in idx])
        a = b.arrays
        p = O._p
        n = int(b.n[0])
        assert np.all(b.n == n) and np.all(b.ntt == b.ntt[0]), "the batched oracle needs equal shapes"
        t0 = time.perf_counter()
        rc = L.oracle_integrate_transits_batch(
            len(idx), nthreads, n, int(b.ti[0]), p(b.h), p(b.tmax), 1, p(a["t"]), p(a["x"]), p(a["v"]), p(a["m"]),
            p(a["xerror"]), p(a["verror"]), p(a["jac_step"]), p(a["jac_error"]), p(a["dqdt"]), p(a["pair"], O._U8),
            p(a["jac_init"]), int(b.ntt[0]), p(a["tt"]), p(a["dtdq0"]), p(a["dtdelements"]), p(a["count"], O._I64))
        dt = time.perf_counter() - t0
        assert rc == 0
        total_ss += sum(nsteps[i] for i in idx)
        total_t += dt
        used += len(idx)
        if total_t < 1.0:
            sample *= 4
    return total_ss / total_t, nthreads, used, total_t


def cpu_rate_by_n(nbg, workload, seed, target_s=6.0, cap_steps=1500, nthreads=None):
    """The oracle's system-steps/s on a workload of mixed body counts: per body count, a sample of its
    systems integrated for their first min(nsteps, cap_steps) steps, one system per host thread, for about
    target_s of wall time; the rates are combined as the time the whole workload would take at them."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O
    from concurrent.futures import ThreadPoolExecutor
    O.build()
    nthreads = nthreads or os.cpu_count() or 1
    states, timings, hs, tms, nsteps = build_workload(nbg, workload, None, seed)
    by_n = {}
    for q, st in enumerate(states):
        by_n.setdefault(st.n, []).append(q)
    rates, total_t = {}, 0.0

    def one(q):
        s = states[q]
        so = O.OState(s.x, s.v, s.m, jac_init=s.jac_init)
        k = min(nsteps[q], cap_steps)
        tm = k * hs[q]
        to = O.OTiming(s.n, timings[q].ntt, 0)
        O.integrate_transits(so, to, hs[q], tm)
        return k

    for n, qs in sorted(by_n.items()):
        done, t_used, used = 0, 0.0, 0
        batch = nthreads
        while t_used < target_s / len(by_n) and used < len(qs):
            pick = [qs[(used + r) % len(qs)] for r in range(batch)]
            used += batch
            t0 = time.perf_counter()
            with ThreadPoolExecutor(max_workers=nthreads) as ex:
                done += sum(ex.map(one, pick))
            t_used += time.perf_counter() - t0
        rates[n] = done / t_used
        total_t += t_used
    steps_n = {n: sum(nsteps[q] for q in qs) for n, qs in by_n.items()}
    value = sum(steps_n.values()) / sum(steps_n[n] / rates[n] for n in steps_n)
    return value, {str(n): r for n, r in rates.items()}, nthreads, total_t


def replica_seed(seed, rank):
    """Each rank integrates its own draw of the workload (replicas, weak scaling)."""
    return seed + 1000 * rank


def reduce_max_ms(ms, dist):
    """Maximum of the per-rank step times (the job is as slow as its slowest rank)."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0])


def aggregate_value(system_steps_per_rank, world, ms):
    """Whole-job system-steps/s: all ranks' work over the slowest rank's time."""
    return system_steps_per_rank * world / (ms * 1e-3)


def _same_n(states):
    return len({s.n for s in states}) == 1


def run_reference(args, nbg, rank):
    """--impl reference: the oracle on the host cores, K timed bounded samples."""
    if rank != 0:
        return
    states, timings, hs, tms, nsteps = build_workload(nbg, args.workload, args.nsys, args.seed, args.tmax)
    if not _same_n(states):
        states_i = [i for i, s in enumerate(states) if s.n == states[0].n]
        states = [states[i] for i in states_i]
        timings = [timings[i] for i in states_i]
        hs = [hs[i] for i in states_i]
        tms = [tms[i] for i in states_i]
        nsteps = [nsteps[i] for i in states_i]
    vals = []
    for it in range(args.warmup + args.steps):
        v, cores, used, t = cpu_baseline(nbg, states, timings, hs, tms, nsteps, target_s=args.ref_seconds)
        if it >= args.warmup:
            vals.append((v, used, t))
    value = float(np.mean([v for v, _, _ in vals]))
    used = vals[-1][1]
    # the same restatement on one host thread, on a smaller sample
    v1, _, used1, t1 = cpu_baseline(nbg, states, timings, hs, tms, nsteps, target_s=min(4.0, args.ref_seconds),
                                    nthreads=1)
    line = {
        "impl": "reference", "metric": "system_steps_per_s", "value": value, "unit": "system-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": float(np.mean([t for _, _, t in vals])) * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "nsys": len(states), "grad": True},
        "cpu_baseline": {"value": value, "unit": "system-steps/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": "%d systems of %s per step (C++ restatement of the reference, "
                                   "Julia unavailable)" % (used, args.workload)},
        "e2e": {"value": value, "unit": "system-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "cpu_1core": {"value": v1, "unit": "system-steps/s", "cores": 1,
                      "sample": "%d systems of %s, %.1f s on one host thread" % (used1, args.workload, t1)},
    }
    if args.secondary != "none":
        sec = {}
        for name in [w for w in args.secondary.split(",") if w and w != "serve"]:
            v2, per_n, cores2, t2 = cpu_rate_by_n(nbg, name, args.seed)
            sec[name] = {"value": v2, "unit": "system-steps/s", "cores": cores2, "kind": "port",
                         "per_body_count": per_n,
                         "sample": "per body count, systems of %s integrated for their first 1500 steps, one per "
                                   "host thread, %.1f s in all; combined as the time of the whole workload" %
                                   (name, t2)}
        line["secondary"] = sec
    print(json.dumps(line), flush=True)


def serve_stream(nbg, srv, pool, rate, nreq, seed, timeout_s, fixed_tail=0):
    """Poisson arrivals (rate requests/s) of nreq requests drawn from pool;
    returns (infos, wall seconds from first arrival to last completion).
    The last fixed_tail entries of pool are sent once each, at random places
    in the stream (their infos carry probe = True); the rest are drawn."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, nreq) if rate > 0 else np.zeros(nreq)
    nbase = len(pool) - fixed_tail
    picks = np.concatenate([rng.integers(0, nbase, nreq - fixed_tail), np.arange(nbase, len(pool))])
    rng.shuffle(picks)
    ids, infos, lock = {}, [], threading.Lock()
    done = threading.Event()
    t_start = time.perf_counter()

    def client():
        t = t_start
        for q in range(nreq):
            t += gaps[q]
            d = t - time.perf_counter()
            if d > 0:
                time.sleep(d)
            s0, ic, h, tmax, grad = pool[picks[q]]
            s = s0.copy()
            tt = nbg.TransitTiming(tmax, ic)
            rid = srv.submit(s, tt, nbg.Integrator(nbg.ahl21, h, 0.0, tmax), grad)
            with lock:
                ids[rid] = (s, tt, picks[q] >= nbase)

    def collector():
        got = 0
        while got < nreq:
            try:
                rid = srv.wait_any(timeout_ms=int(timeout_s * 1000))
            except nbg.NbgError:
                break
            while True:
                with lock:
                    st = ids.pop(rid, None)
                if st is not None:
                    break
                time.sleep(1e-4)  # the client has not recorded this id yet
            infos.append(dict(srv.result(rid, st[0], st[1]), probe=bool(st[2])))
            got += 1
        done.set()

    tc, tr = threading.Thread(target=client), threading.Thread(target=collector)
    tc.start()
    tr.start()
    tc.join()
    tr.join()
    return infos, time.perf_counter() - t_start


def run_serve(args, nbg):
    """Serving: Poisson streams of single systems drawn as batch_uneven,
    50 % grad=true; system-steps/s and p50/p99 latency per body count."""
    W = nbg.workloads
    els, hs, tms = W.batch_uneven(args.serve_pool, args.seed + 11)
    rng = np.random.default_rng(args.seed + 12)
    pool = []
    for el, h, tmax in zip(els, hs, tms):
        ic = W.ic_of(el)
        tmax = min(tmax, args.serve_tmax_max) if args.serve_tmax_max > 0 else tmax
        pool.append((nbg.State(ic), ic, h, tmax, bool(rng.integers(0, 2))))
    rates = [float(r) for r in args.serve_rates.split(",")]
    out = []
    for k, rate in enumerate(rates):
        with nbg.Server(slots_per_group=args.serve_slots, chunk_steps=args.serve_chunk) as srv:
            infos, wall = serve_stream(nbg, srv, pool, rate, args.serve_requests, args.seed + 100 + k,
                                       args.serve_timeout)
            st = srv.stats()
        ok = [i for i in infos if i["rc"] == 0]
        steps = sum(i["nsteps"] for i in ok)
        per_n = {}
        for nb in sorted({i["n"] for i in ok}):
            lat = np.array([i["latency_ms"] for i in ok if i["n"] == nb])
            per_n[str(nb)] = {"requests": int(len(lat)), "p50_ms": float(np.percentile(lat, 50)),
                              "p99_ms": float(np.percentile(lat, 99))}
        lat = np.array([i["latency_ms"] for i in ok]) if ok else np.zeros(1)
        out.append({"rate_per_s": rate, "requests": args.serve_requests, "completed": len(ok),
                    "system_steps_per_s": steps / wall, "wall_s": wall,
                    "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                    "queue_p99_ms": float(np.percentile([i["queue_ms"] for i in ok], 99)) if ok else None,
                    "per_n": per_n, "chunks": st["chunks"], "kernels": st["kernels"], "groups": st["groups"]})
        print(json.dumps({"serve": out[-1]}), flush=True)
    return out


def measure_secondary(nbg, workload, device, seed, tune_steps):
    """One timed pass of a batch workload after the autotuner's trial runs (which warm its kernels
    up): system-steps/s, the consumer's roofline and the clocks of the pass."""
    import torch
    ctx = nbg.Context(device)
    states, timings, hs, tms, nsteps = build_workload(nbg, workload, None, seed)
    b = make_batch(nbg, states, timings, hs, tms)
    dev0 = {k: torch.from_numpy(a.copy()).cuda() for k, a in b.arrays.items()}
    dev = {k: torch.empty_like(t) for k, t in dev0.items()}

    def reset():
        for k in dev:
            dev[k].copy_(dev0[k])

    reset()
    t_tune = time.perf_counter()
    tuning = b.autotune_device(dev, ctx, trial_steps=tune_steps)
    t_tune = time.perf_counter() - t_tune
    reset()
    torch.cuda.synchronize()
    clk = ClockSampler(device)
    clk.start()
    ctx.set_profiling(3)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    b.run_device(dev, ctx)
    e1.record()
    torch.cuda.synchronize()
    ctx.set_profiling(0)
    clocks = clk.stop()
    ms = e0.elapsed_time(e1)
    _, _, _, jac_ms = ctx.last_timing()
    flops = sum(flops_per_system_step(s.n) * ns for s, ns in zip(states, nsteps))
    peak = ctx.fp64_peak_tflops()
    achieved = flops / (jac_ms * 1e-3) / 1e12 if jac_ms > 0 else None
    total = int(sum(nsteps))
    out = {"workload": workload, "nsys": len(states), "system_steps_per_pass": total,
           "body_counts": sorted({int(s.n) for s in states}), "longest_system_steps": int(max(nsteps)),
           "value": total / (ms * 1e-3), "unit": "system-steps/s", "ms_per_pass": ms, "timed_passes": 1,
           "warmup": "the autotuner's trial runs (%.1f s)" % t_tune,
           "launches": int(ctx.last_launch_count()),
           "autotuner": dict({k: tuning[0][k] for k in ("chunk_steps", "orbit_team", "producer_warps",
                                                          "producer_smem_kb")},
                             predicted_ms=tuning[0]["ms"], predicted_over_measured=tuning[0]["ms"] / ms,
                             trial_ms=tuning[0]["trial_ms"], trial_steps=tune_steps),
           "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                        "frac": (achieved / peak) if achieved else None, "kernel": "jacobian_chunk_kernel",
                        "kernel_ms": jac_ms, "peak_source": "measured live (nbg_fp64_peak, DFMA)"},
           "clocks": clocks}
    ctx.close()
    del dev, dev0
    torch.cuda.empty_cache()
    return out


def latency_table(nbg, device, steps=(256, 768)):
    """Single-system step latency: one batch_uneven system of each body count integrated with gradient and
    transit timing, one system per call, for two step counts; the difference of the two call times (best of 3
    after a warm-up call) over the difference of the step counts removes the call's fixed cost."""
    import torch
    W = nbg.workloads
    out = {}
    for n in range(2, 11):
        els, hs, _ = W.batch_uneven(1, seed=500 + n, nmin=n, nmax=n)
        ic = W.ic_of(els[0])
        h = hs[0]
        row = {}
        for team in ((0, 1, 2) if n >= 4 else (0, 2)):
            ctx = nbg.Context(device)
            ctx.set_orbit_team(team)
            best = {}
            for k in steps:
                tmax = k * h
                for rep in range(4):
                    s = nbg.State(ic)
                    tt = nbg.TransitTiming(tmax, ic)
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    nbg.Integrator(nbg.ahl21, h, 0.0, tmax)(s, tt, grad=True, ctx=ctx)
                    torch.cuda.synchronize()
                    dt = time.perf_counter() - t0
                    if rep > 0:
                        best[k] = min(best.get(k, dt), dt)
            name = {0: "one_lane", 1: "team", 2: "wide"}[team]
            row[name] = (best[steps[1]] - best[steps[0]]) * 1e3 / (steps[1] - steps[0])
            row["call_fixed_ms_" + name] = best[steps[0]] * 1e3 - row[name] * steps[0]
            # the kernels' summed device time per step in one more (longer) call, timed per launch
            ctx.set_profiling(1)
            s = nbg.State(ic)
            tt = nbg.TransitTiming(steps[1] * h, ic)
            nbg.Integrator(nbg.ahl21, h, 0.0, steps[1] * h)(s, tt, grad=True, ctx=ctx)
            ctx.set_profiling(0)
            tot, orb, tra, jac = ctx.last_timing()
            row["kernels_ms_per_step_" + name] = {"orbit": orb / steps[1], "transit": tra / steps[1],
                                                 "jacobian": jac / steps[1], "loop": tot / steps[1]}
            ctx.close()
        out[str(n)] = row
    return {"unit": "ms per grad step, one system per call (difference of two call lengths)", "steps": list(steps),
            "by_body_count": out}


def measure_serving(nbg, args, capacity):
    """The request server on config-4 draws (batch_uneven systems, tmax log-uniform 100..4000 d, half with
    gradient) arriving as a Poisson stream at 80 % of the GPU's capacity on this mix -- the batched
    throughput `capacity` (system-steps/s) of batch_uneven, converted to requests/s by the pool's mean
    request length -- with 8-body 1600-day gradient requests mixed in; p50 / p99 latency overall, per body
    count and for the 8-body 1600-day class."""
    W = nbg.workloads
    els, hs, tms = W.batch_uneven(args.serve_pool, args.seed + 11)
    rng = np.random.default_rng(args.seed + 12)
    pool = []
    for el, h, tmax in zip(els, hs, tms):
        ic = W.ic_of(el)
        pool.append((nbg.State(ic), ic, h, tmax, bool(rng.integers(0, 2))))
    mean_steps = float(np.mean([abs(round(t / h)) for _, _, h, t, _ in pool]))
    # the latency class of the target: 8-body systems drawn as batch_uneven, 1600 days, with gradient
    e8, h8, _ = W.batch_uneven(args.serve_probe, args.seed + 13, nmin=8, nmax=8)
    probes = [(nbg.State(W.ic_of(el)), W.ic_of(el), h, 1600.0, True) for el, h in zip(e8, h8)]
    rate = 0.8 * capacity / mean_steps
    nreq = args.serve_point_requests + len(probes)
    with nbg.Server(slots_per_group=args.serve_slots, chunk_steps=args.serve_chunk) as srv:
        infos, wall = serve_stream(nbg, srv, pool + probes, rate, nreq, args.seed + 101, args.serve_timeout,
                                   fixed_tail=len(probes))
        st = srv.stats()
    ok = [i for i in infos if i["rc"] == 0]
    lat = np.array([i["latency_ms"] for i in ok]) if ok else np.zeros(1)
    per_n = {}
    for nb in sorted({i["n"] for i in ok}):
        l = np.array([i["latency_ms"] for i in ok if i["n"] == nb])
        per_n[str(nb)] = {"requests": int(len(l)), "p50_ms": float(np.percentile(l, 50)),
                          "p99_ms": float(np.percentile(l, 99))}
    pr = np.array([i["latency_ms"] for i in ok if i.get("probe")])
    run = np.array([i["run_ms"] for i in ok if i.get("probe")])
    return {"workload": "serve_uneven", "requests": nreq, "completed": len(ok), "grad_fraction": 0.5,
            "tmax_days": "log-uniform 100..4000 (uncapped)",
            "load": {"rate_per_s": rate, "fraction_of_capacity": 0.8,
                     "capacity": "batch_uneven batched throughput, %.0f system-steps/s; mean request %.0f steps"
                                 % (capacity, mean_steps),
                     "wall_s": wall, "system_steps_per_s": sum(i["nsteps"] for i in ok) / wall,
                     "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                     "per_n": per_n, "chunks": st["chunks"], "kernels": st["kernels"], "groups": st["groups"]},
            "class_8body_1600d": {"requests": int(len(pr)), "steps_each": [int(abs(round(1600.0 / h))) for h in h8],
                                  "p50_ms": float(np.percentile(pr, 50)) if len(pr) else None,
                                  "p99_ms": float(np.percentile(pr, 99)) if len(pr) else None,
                                  "run_p50_ms": float(np.percentile(run, 50)) if len(run) else None,
                                  "target_p99_ms": 50.0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="batch_3body",
                    choices=["batch_3body", "batch_8body", "batch_uneven", "plain_3body"])
    ap.add_argument("--nsys", type=int, default=None)
    ap.add_argument("--tmax", type=float, default=0.0,
                    help="integrate every system to this tmax instead of the workload's (small profiling cases)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--bodies", type=int, default=0,
                    help="batch_uneven: draw only systems of this body count (small profiling cases)")
    ap.add_argument("--chunk", type=int, default=0)
    ap.add_argument("--serial", action="store_true", help="one stream: no producer/consumer overlap")
    ap.add_argument("--noalloc", action="store_true",
                    help="time the allocation-free entry point (at most 128 systems) instead of the device-resident one")
    ap.add_argument("--kernel-timing", default="timed", choices=["timed", "separate"],
                    help="consumer duration from a CUDA-event pair around one launch per timed step, or from "
                         "event pairs around every launch in one extra pass")
    ap.add_argument("--spw", type=int, default=0, help="orbit producer systems per warp (0 = automatic)")
    ap.add_argument("--orbit-team", type=int, default=-1,
                    help="orbit producer form: -1 automatic, 0 one lane per system, 1 a team per system, 2 the wide "
                         "team form, 3 a team, wide when latency-bound")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="skip the autotuner (it picks chunk length and orbit-producer mapping before the warm-up)")
    ap.add_argument("--tune-steps", type=int, default=512,
                    help="steps per system of the shorter autotuner trial (the longer runs twice as many)")
    ap.add_argument("--ref-seconds", type=float, default=8.0)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--serve", action="store_true", help="serving: Poisson request streams of batch_uneven draws, then exit")
    ap.add_argument("--serve-rates", default="4,16,64,0", help="request rates per second (0 = all at once)")
    ap.add_argument("--serve-requests", type=int, default=256)
    ap.add_argument("--serve-pool", type=int, default=512)
    ap.add_argument("--serve-slots", type=int, default=256)
    ap.add_argument("--serve-chunk", type=int, default=32)
    ap.add_argument("--serve-tmax-max", type=float, default=0.0, help="cap on a request's tmax (0: none)")
    ap.add_argument("--serve-timeout", type=float, default=600.0)
    ap.add_argument("--secondary", default="batch_8body,batch_uneven,serve",
                    help="after the headline: one timed pass of each listed batch workload and the serving point "
                         "('none' to skip); single-GPU runs only")
    ap.add_argument("--serve-point-requests", type=int, default=64,
                    help="config-4 requests of the serving point (besides its 8-body 1600-day requests)")
    ap.add_argument("--serve-capacity", type=float, default=2.5e5,
                    help="system-steps/s taken as the GPU's capacity when batch_uneven is not measured first")
    ap.add_argument("--serve-probe", type=int, default=6,
                    help="8-body 1600-day gradient requests mixed into the serving point's load stream")
    ap.add_argument("--latency-table", action="store_true",
                    help="print the single-system step latency for 2..10 bodies (one lane / team producer), then exit")
    ap.add_argument("--fp64-probe", action="store_true",
                    help="print the measured FP64 rates (DFMA; DMMA alone; DMMA interleaved with DFMA), then exit")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    nbg = load_package()
    if args.impl == "reference":
        run_reference(args, nbg, rank)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    import torch
    torch.cuda.set_device(local_rank)
    if args.serve:
        run_serve(args, nbg)
        return
    if args.latency_table:
        print(json.dumps({"latency_table": latency_table(nbg, local_rank)}), flush=True)
        return
    if args.fp64_probe:
        ctx = nbg.Context(local_rank)
        dfma = ctx.fp64_peak_tflops()
        mma, _ = ctx.fp64_mma_peak_tflops(False)
        mixed, share = ctx.fp64_mma_peak_tflops(True)
        issue = {"%dw_%dc" % (w, c): ctx.fp64_warp_issue_cycles(w, c) for w in (1, 2, 4, 8) for c in (1, 8)}
        print(json.dumps({"fp64_probe": {"dfma_tflops": dfma, "dmma_tflops": mma, "dmma_plus_dfma_tflops": mixed,
                                         "dfma_share_of_mixed": share, "unit": "TFLOP/s (FMA = 2 flops)",
                                         "cycles_per_warp_dfma_one_block": issue}}), flush=True)
        return
    ctx = nbg.Context(local_rank)
    if args.chunk or args.serial:
        ctx.set_tuning(chunk_steps=args.chunk, overlap=0 if args.serial else -1)
    chunk = args.chunk or 64  # the library's default chunk length (not shortened at these sizes)
    if args.spw:
        ctx.set_orbit_lanes(args.spw)
    ctx.set_orbit_team(args.orbit_team)
    states, timings, hs, tms, nsteps = build_workload(nbg, args.workload, args.nsys, replica_seed(args.seed, rank),
                                                      args.tmax, args.bodies)
    total_ss = int(sum(nsteps))
    b = make_batch(nbg, states, timings, hs, tms)
    # device-resident inputs: a pristine copy and the working buffers
    dev0 = {k: torch.from_numpy(a.copy()).cuda() for k, a in b.arrays.items()}
    dev = {k: torch.empty_like(t) for k, t in dev0.items()}

    def reset():
        for k in dev:
            dev[k].copy_(dev0[k])

    tuning = None
    if not args.no_autotune and not (args.chunk or args.serial or args.spw or args.orbit_team != -1):
        reset()
        tuning = b.autotune_device(dev, ctx, trial_steps=args.tune_steps)
        chunk = tuning[0]["chunk_steps"]

    def step():
        reset()
        if args.noalloc:
            b.run_device_noalloc(dev, ctx)
        else:
            b.run_device(dev, ctx)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = ClockSampler(local_rank)
    clk.start()
    launches = 0
    host_ms = 0.0
    # per-kernel CUDA-event pairs on each kernel's own stream, summed over the
    # timed steps: the roofline's kernel durations come from the timed region
    # one event pair per timed step, around the Jacobian consumer's launch of
    # the middle chunk (the roofline kernel's duration, measured inside the
    # timed region): an event pair around every consumer launch slows the
    # overlapped streams by 8-10 % (measured), one pair per step does not
    ctx.set_profiling(3 if args.kernel_timing == "timed" else 0)
    kt = np.zeros(4)
    kn = np.zeros(2, dtype=np.int64)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step()
        launches += ctx.last_launch_count()
        host_ms += ctx.last_host_ms()
        kt += np.array(ctx.last_timing())
        kn += np.array(ctx.last_kernel_stats(), dtype=np.int64)
    e1.record()
    torch.cuda.synchronize()
    ctx.set_profiling(False)
    clocks = clk.stop()
    ms = reduce_max_ms(e0.elapsed_time(e1) / args.steps, dist)
    value = aggregate_value(total_ss, world, ms)

    # e2e through the host API with pinned buffers, copies inside the timed region
    bp = make_batch(nbg, states, timings, hs, tms, pinned=True)
    pristine = {k: a.copy() for k, a in bp.arrays.items()}
    in_keys = ("t", "x", "v", "m", "xerror", "verror", "jac_step", "jac_error", "dqdt", "jac_init", "count")
    out_keys = ("t", "x", "v", "xerror", "verror", "jac_step", "jac_error", "dqdt", "count", "tt", "dtdq0",
                "dtdelements")
    h2d = sum(bp.arrays[k].nbytes for k in in_keys)
    d2h = sum(bp.arrays[k].nbytes for k in out_keys)
    e2e_ms = []
    for it in range(1 + args.e2e_steps if args.e2e_steps > 0 else 0):
        for k in bp.arrays:
            bp.arrays[k][...] = pristine[k]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bp.run(ctx)
        torch.cuda.synchronize()
        if it > 0:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_val = total_ss * world / (np.mean(e2e_ms) * 1e-3) if e2e_ms else None

    if args.kernel_timing == "separate":
        # one more pass with the event pairs, after the timed region
        ctx.set_profiling(True)
        step()
        ctx.set_profiling(False)
        kt = np.array(ctx.last_timing()) * args.steps
        kn = np.array(ctx.last_kernel_stats(), dtype=np.int64) * args.steps
    # roofline of the Jacobian consumer, averaged over the timed steps
    total_ms, orbit_ms, transit_ms, jac_ms = kt / args.steps
    # the other kernels' summed durations, from one more pass timed per kernel
    # (not part of the timed region)
    ctx.set_profiling(1)
    step()
    ctx.set_profiling(0)
    _, orbit_ms, transit_ms, _ = ctx.last_timing()
    n_orbit, n_jac = (int(v) // args.steps for v in kn)
    flops = sum(flops_per_system_step(s.n) * ns for s, ns in zip(states, nsteps))
    peak = ctx.fp64_peak_tflops()
    achieved = flops / (jac_ms * 1e-3) / 1e12 if jac_ms > 0 else None
    # DRAM bytes per launch: ncu's per-system-step figure for this kernel and
    # workload times the system-steps one launch processes (chunk x systems)
    traffic = None
    prof_json = os.path.join(ROOT, "profiles", "jacobian_consumer_%s.json" % args.workload)
    if os.path.exists(prof_json):
        with open(prof_json) as f:
            per_unit = json.load(f).get("dram_bytes_per_system_step")
        if per_unit:
            traffic = per_unit * chunk * len(states)

    if rank == 0:
        line = {
            "metric": "system_steps_per_s", "value": value, "unit": "system-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded draws)",
            "config": {"workload": args.workload, "nsys": len(states), "system_steps_per_pass": total_ss,
                       "tmax_override": args.tmax or None,
                       "grad": True, "parallelism": "replicas" if world > 1 else "single",
                       "l2": "working set larger than L2 (operator records + jac_step)",
                       "chunk_steps": chunk,
                       "orbit_systems_per_warp": (args.spw or "auto") if tuning is None
                       else (tuning[0]["orbit_lanes"] or "auto"),
                       "orbit_team": ({-1: "auto", 0: "off", 1: "on", 2: "wide", 3: "on, wide when latency-bound"}
                                      [args.orbit_team] if tuning is None
                                      else {0: "off", 1: "on, wide when latency-bound"}[tuning[0]["orbit_team"]]),
                       "autotuner": None if tuning is None else {
                           "trial_steps_per_system": args.tune_steps,
                           "chosen": {k: tuning[0][k] for k in ("chunk_steps", "orbit_team", "producer_warps",
                                                                "producer_smem_kb")},
                           "candidates": [{k: (round(r[k], 2) if k == "ms" else r[k])
                                           for k in ("chunk_steps", "orbit_team", "producer_warps",
                                                     "producer_smem_kb", "ms")}
                                          for r in tuning]},
                       "streams": 1 if args.serial else 3},
            "e2e": {"value": e2e_val, "unit": "system-steps/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": float(np.mean(e2e_ms)) if e2e_ms else None},
            "gpu_launches": int(launches),
            "host_enqueue_ms_per_step": host_ms / args.steps,
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                         "kernel": "jacobian_chunk_kernel", "peak_source": "measured live (nbg_fp64_peak, DFMA)",
                         "launches": n_jac, "kernel_ms": jac_ms,
                         "kernel_ms_source": ("CUDA-event pair around one consumer launch (the middle chunk) per "
                                              "timed step, on its stream, scaled to the step's launches"
                                              if args.kernel_timing == "timed" else
                                              "CUDA-event pairs around every consumer launch of one extra pass"),
                         "orbit_ms": orbit_ms, "transit_ms": transit_ms,
                         "loop_ms": total_ms},
            "clocks": clocks,
        }
        if not args.no_cpu_baseline and world == 1:
            v, cores, used, t = cpu_baseline(nbg, states, timings, hs, tms, nsteps) if _same_n(states) else \
                (None, None, 0, 0.0)
            line["cpu_baseline"] = {"value": v, "unit": "system-steps/s", "cores": cores, "kind": "port",
                                    "sample": "%d systems of %s, %.1f s on %s host threads" %
                                              (used, args.workload, t, cores)}
        if world == 1 and args.secondary != "none":
            del dev, dev0
            torch.cuda.empty_cache()
            sec = {}
            for name in [w for w in args.secondary.split(",") if w]:
                if name == "serve":
                    cap = sec.get("batch_uneven", {}).get("value") or args.serve_capacity
                    sec[name] = measure_serving(nbg, args, cap)
                else:
                    sec[name] = measure_secondary(nbg, name, local_rank, args.seed, args.tune_steps)
            line["secondary"] = sec
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
