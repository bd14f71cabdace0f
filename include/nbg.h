/*
 * nbg.h -- C ABI of libnbg_cuda, the GB300 (sm_103a) implementation of
 * NbodyGradient.jl's AHL21 integration with forward Jacobian propagation and
 * transit timing.
 *
 * Conventions (all entry points):
 *   - Arrays are Julia column-major Float64 (double) unless noted, exactly as
 *     the reference State / TransitTiming hold them:
 *       x, v, xerror, verror : 3 x n           (x[k + 3 i])
 *       m                    : n
 *       jac_step, jac_error, jac_init : 7n x 7n (J[r + 7n c]; body i owns rows
 *                              7i..7i+6 ordered x, y, z, vx, vy, vz, m)
 *       dqdt                 : 7n
 *       pair                 : n x n uint8 (Julia Bool), pair[i + n j]
 *       tt                   : n x ntt
 *       dtdq0, dtdelements   : n x ntt x 7 x n   (A[j + n(c + ntt(k + 7p))])
 *       count                : n int64
 *   - Body indices are 0-based in this ABI (the Julia shim passes ti - 1).
 *   - Return value: 0 on success, a negative NBG_E* code on failure; the
 *     message is available from nbg_last_error() on the calling thread.
 *   - The library never keeps a caller pointer after a call returns, except
 *     the arrays given to nbg_batch_submit, which the batch uses until
 *     nbg_batch_wait has returned its run's result.
 *   - A context owns its CUDA streams (one, plus three per group of systems
 *     while the overlapped chunk pipeline is on) and its device buffers;
 *     calls on one context must not overlap.  Different contexts may be used
 *     from different threads.
 */
#ifndef NBG_H
#define NBG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NBG_OK 0
#define NBG_EINVAL (-1)       /* invalid argument                          */
#define NBG_ECUDA (-2)        /* CUDA runtime error                        */
#define NBG_ENOMEM (-3)       /* device allocation failed / budget exceeded */
#define NBG_EUNSUPPORTED (-4) /* outside the built configuration (n range) */
#define NBG_ENONFINITE (-5)   /* a system produced non-finite values        */
#define NBG_ETIMEOUT (-6)     /* a bounded wait ran out                     */
#define NBG_ECANCELLED (-7)   /* request cancelled                          */

#define NBG_MIN_BODIES 2
#define NBG_MAX_BODIES 10

/* Per-system status bits written by the batched entry points. */
#define NBG_STATUS_NONFINITE 1u     /* x, v or J not finite at the end          */
#define NBG_STATUS_NTT_OVERFLOW 2u  /* more transits than ntt (counted, dropped) */
#define NBG_STATUS_NEWTON_ITMAX 4u  /* a transit Newton search hit ITMAX = 20    */

typedef struct nbg_context nbg_context;

/* Create / destroy a context on CUDA device `device`.
 * Replaces: nothing in the reference (it is single-threaded Julia); the Julia
 * shim creates one context per session. */
int nbg_create(int device, nbg_context** out);
int nbg_destroy(nbg_context* ctx);

/* Copy the calling thread's last error message into buf (NUL-terminated).
 * No reference counterpart (the reference throws Julia exceptions; the shim
 * turns a non-zero return code into error(...) with this message). */
int nbg_last_error(char* buf, size_t len);

/* Library version (major * 10000 + minor * 100 + patch) and device facts
 * (no reference counterpart). */
int nbg_version(void);

typedef struct {
  char name[128];
  int sm_count;
  int cc_major, cc_minor;
  size_t total_mem;
  int min_bodies, max_bodies;
} nbg_device_info_t;
int nbg_device_info(int device, nbg_device_info_t* out);

/*
 * (intr::Integrator)(s::State{Float64}, tt::TransitTiming{Float64}; grad)
 * Replaces src/transits/Transits.jl:140-170 (called through :173-180) with
 * intr.scheme === ahl21!: integrates nsteps = |round(tmax/h)| AHL21 steps from
 * s.t = *t, detects transits of every body but ti across body ti, refines
 * them by Newton on partial steps (src/transits/timing.jl:3-109) and, when
 * grad != 0, propagates jac_step / jac_error / dqdt (ahl21.jl:5-95), fills
 * dtdq0 and computes dtdelements = dtdq0 * jac_init (timing.jl:112-123).
 *
 * In/out exactly as the reference mutates State and TransitTiming: x, v,
 * xerror, verror, jac_step, jac_error, dqdt, *t (set to t0 + nsteps * h),
 * tt, dtdq0, dtdelements and count.  Entries of tt / dtdq0 that no transit
 * of this call writes are left untouched; dtdelements is recomputed for
 * every transit 1..min(count, ntt) as the reference does.
 */
int nbg_integrate_transits(nbg_context* ctx, int n, int ti, double h, double tmax, int grad, double* t,
                           double* x, double* v, const double* m, double* xerror, double* verror,
                           double* jac_step, double* jac_error, double* dqdt, const uint8_t* pair,
                           const double* jac_init, int64_t ntt, double* tt, double* dtdq0, double* dtdelements,
                           int64_t* count);

/*
 * (intr::Integrator)(s::State{Float64}, ttbv::TransitParameters{Float64}; grad)
 * Replaces src/transits/Transits.jl:140-180 with a TransitParameters output
 * (Transits.jl:68-110) and the TransitParameters branch of findtransit!
 * (src/transits/timing.jl:82-98, dtbvdq! rows 1-3 at :155-193,
 * calc_dtdelements! at :126-138).  Same State arguments as
 * nbg_integrate_transits; the outputs carry a leading row index r = t,
 * v_sky, b_sky^2:
 *   ttbv                   : 3 x n x ntt          (A[r + 3(j + n c)])
 *   dtbvdq0, dtbvdelements : 3 x n x ntt x 7 x n  (A[r + 3(j + n(c + ntt(k + 7p)))])
 * Without grad, v_sky and b_sky^2 are those of the last Newton iterate's
 * state, as in the reference.
 */
int nbg_integrate_transit_parameters(nbg_context* ctx, int n, int ti, double h, double tmax, int grad, double* t,
                                     double* x, double* v, const double* m, double* xerror, double* verror,
                                     double* jac_step, double* jac_error, double* dqdt, const uint8_t* pair,
                                     const double* jac_init, int64_t ntt, double* ttbv, double* dtbvdq0,
                                     double* dtbvdelements, int64_t* count);

/*
 * (intr::Integrator)(s::State{Float64}, time::Float64; grad)
 * Replaces src/integrator/Integrator.jl:159-197 with intr.scheme === ahl21!:
 * nsteps = |round((time - s.t)/h)| steps of h * check_step(s.t, time), then,
 * when tmax = s.t + h nsteps differs from time, one step of time - tmax; s.t
 * is set to time.  x, v, xerror, verror, jac_step, jac_error and dqdt are
 * updated in place (jac_step / jac_error / dqdt only with grad; dqdt is that
 * of the last step, as in the reference).  intr(s; grad) (Integrator.jl:247)
 * is this call with time = s.t + intr.tmax.
 */
int nbg_integrate(nbg_context* ctx, int n, double h, double time, int grad, double* t, double* x, double* v,
                  const double* m, double* xerror, double* verror, double* jac_step, double* jac_error, double* dqdt,
                  const uint8_t* pair);

/*
 * (intr::Integrator)(s::State{Float64}, N::Int64; grad)
 * Replaces src/integrator/Integrator.jl:210-233: |N| steps of h (of -h when
 * N < 0); s.t advances by the compensated sum of the signed steps.
 */
int nbg_integrate_steps(nbg_context* ctx, int n, double h, int64_t nsteps, int grad, double* t, double* x,
                        double* v, const double* m, double* xerror, double* verror, double* jac_step,
                        double* jac_error, double* dqdt, const uint8_t* pair);

/*
 * init_nbody(ElementsIC(t0, H, elements)) for nsys systems on the GPU.
 * Replaces src/ics/init_nbody.jl:13-229 (with kepler_init.jl:66-210 and
 * kepler.jl:1-41) as called by State(ic) (src/integrator/Integrator.jl:82-103):
 * elements is each system's N x 7 column-major ElementsIC.elements (m, P,
 * t0, e cos w, e sin w, I, Omega), H its N x N hierarchy matrix (NULL: every
 * system fully nested, hierarchy([N, 1, ..., 1])), t0 its epoch; out: x, v
 * (3 x N) and jac_init (7N x 7N) per system, packed as the batched calls
 * pack them.  The element checks of InitialConditions.jl:71-77 stay with the
 * caller.  Host pointers (n, t0 always host).
 */
int nbg_batch_init_nbody(nbg_context* ctx, int nsys, const int32_t* n, const double* t0, const double* elements,
                         const double* H, double* x, double* v, double* jac_init);
/* The same with elements, H, x, v, jac_init in device memory. */
int nbg_batch_init_nbody_device(nbg_context* ctx, int nsys, const int32_t* n, const double* t0,
                                const double* elements, const double* H, double* x, double* v, double* jac_init);

/*
 * Batched form: nsys >= 1 independent systems integrated in one plan (an
 * empty batch returns NBG_EINVAL, as does every batched entry point).  Each
 * system's arrays are laid out exactly as for nbg_integrate_transits and
 * concatenated system after system in every packed buffer (so the offset of
 * system s in `x` is sum_{q<s} 3 n_q, in `jac_step` sum_{q<s} (7 n_q)^2, in
 * `tt` sum_{q<s} n_q ntt_q, in `dtdq0` sum_{q<s} 7 n_q^2 ntt_q, ...).
 * All pointers are host pointers.  status (may be NULL) receives one
 * NBG_STATUS_* word per system.  Outputs of every system are treated as
 * fresh TransitTiming arrays (count must be zero on entry).
 */
typedef struct {
  int32_t n;     /* bodies, NBG_MIN_BODIES..NBG_MAX_BODIES */
  int32_t ti;    /* 0-based transited body                  */
  int32_t grad;  /* 0 or 1                                  */
  int32_t ntt;   /* TransitTiming.ntt                       */
  double h;      /* Integrator.h                            */
  double tmax;   /* Integrator.tmax                         */
} nbg_system_desc;

int nbg_batch_integrate_transits(nbg_context* ctx, int nsys, const nbg_system_desc* desc, double* t, double* x,
                                 double* v, const double* m, double* xerror, double* verror, double* jac_step,
                                 double* jac_error, double* dqdt, const uint8_t* pair, const double* jac_init,
                                 double* tt, double* dtdq0, double* dtdelements, int64_t* count, uint32_t* status);

/*
 * Asynchronous batch: nbg_batch_integrate_transits in steps, so that the
 * caller's thread is free while a batch runs.  No reference counterpart (the
 * reference integrates one system per call on the caller's thread).
 *   nbg_batch_create   checks and copies nsys descriptors; binds the batch to
 *                      ctx.
 *   nbg_batch_submit   records the caller's packed host arrays (the arguments
 *                      of nbg_batch_integrate_transits after desc, same
 *                      layout and rules); nothing runs yet.
 *   nbg_batch_run      starts nbg_batch_integrate_transits on a library host
 *                      thread and returns at once.  Until nbg_batch_wait has
 *                      returned the run's result, the arrays belong to the
 *                      batch and ctx takes no other call.
 *   nbg_batch_wait     waits up to timeout_ms (< 0: no limit); NBG_ETIMEOUT
 *                      while the run continues, else the run's result, with
 *                      its message from nbg_last_error on the waiting thread.
 *   nbg_batch_destroy  waits for a started run, then frees the batch.
 * After nbg_batch_wait has returned the result, the batch may be submitted
 * (new arrays or the same) and run again.
 */
typedef struct nbg_batch nbg_batch;
int nbg_batch_create(nbg_context* ctx, int nsys, const nbg_system_desc* desc, nbg_batch** out);
int nbg_batch_submit(nbg_batch* b, double* t, double* x, double* v, const double* m, double* xerror, double* verror,
                     double* jac_step, double* jac_error, double* dqdt, const uint8_t* pair, const double* jac_init,
                     double* tt, double* dtdq0, double* dtdelements, int64_t* count, uint32_t* status);
int nbg_batch_run(nbg_batch* b);
int nbg_batch_wait(nbg_batch* b, int32_t timeout_ms);
int nbg_batch_destroy(nbg_batch* b);

/*
 * nbg_integrate_transit_parameters for nsys systems in one plan (arguments
 * as nbg_batch_integrate_transits; ttbv / dtbvdq0 / dtbvdelements packed
 * with 3 n ntt and 3 n ntt 7 n doubles per system).  No reference
 * counterpart (the reference loops in Julia).
 */
int nbg_batch_integrate_transit_parameters(nbg_context* ctx, int nsys, const nbg_system_desc* desc, double* t,
                                           double* x, double* v, const double* m, double* xerror, double* verror,
                                           double* jac_step, double* jac_error, double* dqdt, const uint8_t* pair,
                                           const double* jac_init, double* ttbv, double* dtbvdq0,
                                           double* dtbvdelements, int64_t* count, uint32_t* status);

/*
 * (intr::Integrator)(s::State{Float64}, o::CartesianOutput{Float64})
 * Replaces src/outputs/Outputs.jl:26-49: nstep steps (with gradient) of
 * h * check_step(s.t, tmax), saving the state at the start of every step:
 * out_t[i] = s.t + h i, out_x / out_v (3 x N per step) and, unless out_jac is
 * NULL, out_jac (7N x 7N per step) -- the t, x, v and jac_step of
 * o.states[i + 1].  The State is advanced in place; s.t = t0 + h nstep.  The
 * records stream to the host chunk by chunk while the integration runs.  The
 * reference's optional JLD2 file is the caller's to write.
 */
int nbg_integrate_cartesian(nbg_context* ctx, int n, double h, double tmax, int64_t nstep, double* t, double* x,
                            double* v, const double* m, double* xerror, double* verror, double* jac_step,
                            double* jac_error, double* dqdt, const uint8_t* pair, double* out_t, double* out_x,
                            double* out_v, double* out_jac);

/*
 * nbg_integrate for nsys systems in one plan: desc[s].tmax is system s's
 * target time (the `time` of intr(s, time)), desc[s].h its step and
 * desc[s].grad its flag (ti and ntt are ignored); arrays packed as for
 * nbg_batch_integrate_transits.  No reference counterpart (the reference
 * loops in Julia).
 */
int nbg_batch_integrate(nbg_context* ctx, int nsys, const nbg_system_desc* desc, double* t, double* x, double* v,
                        const double* m, double* xerror, double* verror, double* jac_step, double* jac_error,
                        double* dqdt, const uint8_t* pair);

/*
 * Same as nbg_batch_integrate_transits, but every array pointer (and desc)
 * is a DEVICE pointer of the context's device, already resident in HBM
 * (desc_host and status stay host pointers).  Used when the caller keeps
 * systems on the GPU between calls.
 */
int nbg_batch_integrate_transits_device(nbg_context* ctx, int nsys, const nbg_system_desc* desc_host, double* t,
                                        double* x, double* v, const double* m, double* xerror, double* verror,
                                        double* jac_step, double* jac_error, double* dqdt, const uint8_t* pair,
                                        const double* jac_init, double* tt, double* dtdq0, double* dtdelements,
                                        int64_t* count, uint32_t* status);

/*
 * Allocation-free form of nbg_batch_integrate_transits_device (no
 * counterpart in the reference): same arguments, same results, but the call
 * allocates no device memory.  It is meant for callers that cannot let a
 * library allocate while they run -- a sampler or pipeline that reserves the
 * GPU's memory for itself and hands over only its own buffers, or a loop that
 * must not pay the device-wide synchronisation of cudaMalloc / cudaFree when
 * a larger batch arrives (the other entry points grow a per-context buffer
 * cache that way).
 *
 * All working memory comes from one fixed array of NBG_NOALLOC_SCRATCH_BYTES
 * in the library, per device.  A call whose working set does not fit even at
 * one integration step per chunk, or that passes more than
 * NBG_NOALLOC_MAX_SYSTEMS systems, is rejected with NBG_ENOMEM / NBG_EINVAL
 * and a message naming the sizes; larger batches fit by shortening the
 * chunk, at some speed.
 *
 * Every call looks up the array's device address (cudaGetSymbolAddress) with
 * the context's device current.  Under CUDA's lazy module loading (the
 * default) the first call on a device loads the library's module there and
 * reserves the 64 MiB array at that moment: a caller that reserves the rest
 * of the GPU's memory for itself must make one call (any small batch) before
 * doing so, or that first lookup fails with NBG_ECUDA (out of memory); make
 * that first call before any stream capture on the device, too.  With
 * CUDA_MODULE_LOADING=EAGER every context reserves the array when it is
 * created, whether it calls this entry point or not.  The host bookkeeping
 * (about 90 KB) belongs to the context and is allocated by nbg_create.
 *
 * Speed: the call runs every kernel on the context's one stream, without the
 * producer / consumer overlap of the other batched entry points, and its
 * chunk shrinks when the working set would not fit; expect it to be slower
 * than nbg_batch_integrate_transits_device on the same batch (measured: 128
 * 3-body systems, 2000 steps, 473 ms against 326 ms, 1.45 times as long).
 *
 * Every call on a device shares
 * the one array and finds the previous call's contents in it (the call
 * clears what must start at zero itself).  Calls that overlap on the GPU --
 * from two threads, two contexts or two streams of the same device -- race
 * on the array and corrupt each other's results: serialise them.  The call
 * returns when its results are in the caller's arrays.
 */
#define NBG_NOALLOC_SCRATCH_BYTES (64u * 1024u * 1024u)
#define NBG_NOALLOC_MAX_SYSTEMS 128
int nbg_batch_integrate_transits_noalloc(nbg_context* ctx, int nsys, const nbg_system_desc* desc_host, double* t,
                                         double* x, double* v, const double* m, double* xerror, double* verror,
                                         double* jac_step, double* jac_error, double* dqdt, const uint8_t* pair,
                                         const double* jac_init, double* tt, double* dtdq0, double* dtdelements,
                                         int64_t* count, uint32_t* status);

/*
 * Request server: continuous batching of single-system requests.
 *
 * Replaces: the same (intr::Integrator)(s::State{Float64}, tt::TransitTiming;
 * grad) call as nbg_integrate_transits (src/transits/Transits.jl:140-180),
 * issued as independent requests from any number of host threads.  A request
 * is a State plus a fresh TransitTiming (count = 0, tt / dtdq0 / dtdelements
 * zero).  Requests with the same body count, grad flag and pair pattern share
 * a group of device-resident slots; each group advances all its slots by
 * chunk_steps steps per chunk on its own CUDA stream, and a request that
 * arrives while others run takes a free slot at the next chunk boundary of
 * its group (its first step runs in that chunk).  A slot holds its system's
 * state and jac_step on the device from admission to its last step.
 * Admission is by HBM footprint: half of hbm_budget_bytes is an output arena
 * from which each admitted request takes its tt / dtdq0 / dtdelements block
 * (a request waits while the arena is full); the other half holds the groups'
 * slot buffers (a request whose new group does not fit fails NBG_ENOMEM).
 * Results are bitwise the same whether a request runs alone or among others.
 * Requests not yet admitted when the server stops are cancelled
 * (NBG_ECANCELLED); admitted ones run to completion.  nbg_server_cancel
 * withdraws one request at any time before its last chunk is queued.
 */
typedef struct nbg_server nbg_server;

typedef struct {
  int32_t slots_per_group;   /* slots per (n, grad, pair pattern) group; 0 = 256 (rounded up to 32) */
  int32_t chunk_steps;       /* steps per chunk; 0 = 32                                   */
  int32_t max_inflight;      /* chunks a group may have queued on the GPU; 0 = 2          */
  int32_t orbit_lanes;       /* orbit producer systems per warp (1..32); 0 = 32           */
  uint64_t hbm_budget_bytes; /* device memory the server may hold; 0 = a quarter of free  */
  int32_t orbit_team;        /* -1 or 0 (the zero-initialised default) = automatic; see
                                nbg_set_orbit_team (1: always, -2 never)              */
  int32_t reserved;
} nbg_server_config;

typedef struct {
  int64_t id;
  int32_t n, grad;
  int64_t nsteps;
  double queue_ms;   /* enqueue -> admitted into a slot                    */
  double run_ms;     /* admitted -> results in the server's host buffer    */
  double latency_ms; /* enqueue -> results in the server's host buffer     */
  uint32_t status;   /* NBG_STATUS_* bits                                  */
  int32_t rc;        /* NBG_OK or the request's error code                 */
} nbg_request_info;

typedef struct {
  int64_t submitted, admitted, completed, failed, running, pending;
  int64_t chunks, kernels;   /* chunk launches and kernel launches so far */
  uint64_t hbm_groups;       /* bytes held by the groups' slot buffers     */
  uint64_t hbm_outputs_in_use; /* bytes of the output arena in use         */
  uint64_t hbm_budget;
  int32_t groups, pad;
} nbg_server_stats_t;

/* Start a server (and its host thread) on CUDA device `device`; cfg may be NULL. */
int nbg_server_start(int device, const nbg_server_config* cfg, nbg_server** out);

/* Queue one request; the arrays are copied before the call returns.  desc
 * as for the batched calls; t0 is s.t.  jac_step, jac_error, jac_init and
 * dqdt may be NULL when desc->grad == 0.  *id receives the request id. */
int nbg_server_enqueue(nbg_server* srv, const nbg_system_desc* desc, double t0, const double* x, const double* v,
                       const double* m, const double* xerror, const double* verror, const double* jac_step,
                       const double* jac_error, const double* dqdt, const uint8_t* pair, const double* jac_init,
                       int64_t* id);

/* Wait up to timeout_ms (< 0: no limit) for the next completed request not
 * yet collected; NBG_ETIMEOUT if none completes in time. */
int nbg_server_wait_any(nbg_server* srv, int32_t timeout_ms, int64_t* id);

/* Wait up to timeout_ms (< 0: no limit) for request `id`, copy its results
 * into the (non-NULL) output arrays -- the State fields as updated by the
 * integration, s.t, and the TransitTiming tt, dtdq0, dtdelements and count
 * -- and release it.  info (may be NULL) receives its latency and status.
 * Returns the request's own error code if it failed. */
int nbg_server_poll(nbg_server* srv, int64_t id, int32_t timeout_ms, double* t, double* x, double* v,
                    double* xerror, double* verror, double* jac_step, double* jac_error, double* dqdt, double* tt,
                    double* dtdq0, double* dtdelements, int64_t* count, nbg_request_info* info);

int nbg_server_stats(nbg_server* srv, nbg_server_stats_t* out);

/* Withdraw request `id` (no reference counterpart: the reference has no
 * request queue).  A request not yet admitted leaves its queue; a running one
 * is retired at the next chunk boundary of its group, its slot and output
 * memory freed; nbg_server_poll of either returns NBG_ECANCELLED.  Returns
 * NBG_OK when the cancellation took effect, NBG_EINVAL for an unknown or
 * already collected id, or for a request that has finished or whose last
 * chunk is already queued (its result stands and is collected as usual). */
int nbg_server_cancel(nbg_server* srv, int64_t id);

/* Cancel requests not yet admitted (their nbg_server_poll returns
 * NBG_ECANCELLED), finish the running ones, wait for threads still inside
 * nbg_server_wait_any / nbg_server_poll to return (a wait_any with nothing
 * left to collect returns NBG_ECANCELLED), then free the server.  Requests
 * not collected by then are freed with it. */
int nbg_server_stop(nbg_server* srv);

/* Tuning knobs of a context (no reference counterpart).  Results do not
 * depend on them.
 * chunk_steps: integration steps per producer/consumer chunk (default 64,
 *   shortened for batches whose per-chunk operator records would pass
 *   4 GiB; 0 keeps the current value);
 * overlap: 1 (default) runs the orbit producer on its own stream one chunk
 *   ahead of the transit searches, operator kernels and Jacobian consumer
 *   (three streams per group of systems); 0 runs everything on one stream;
 *   a negative value keeps the current setting. */
int nbg_set_tuning(nbg_context* ctx, int chunk_steps, int overlap);

/* Device time (ms) of the last batched call's integration, measured with
 * CUDA events on the context's stream: total (chunk loop), and -- when
 * profiling is on -- the summed durations of the orbit-producer, transit-
 * search and Jacobian-consumer launches.  No counterpart in the reference. */
int nbg_last_timing(nbg_context* ctx, double* total_ms, double* orbit_ms, double* transit_ms, double* jacobian_ms);

/*
 * Autotuner (no counterpart in the reference).  Times two short trial
 * integrations of this batch -- every system's first min(nsteps, T) steps
 * for T = trial_steps and 2 trial_steps, on device copies (the caller's
 * arrays are not modified) -- for each candidate mapping: steps per chunk
 * {64, 128} x orbit producer form {one lane per system, team of lanes} x
 * producer block layout {one warp; four warps holding 200 KB of shared
 * memory, operator and search blocks 32 KB} (nbg_set_producer_layout).  The
 * two trial times give the loop's fill and drain and its time per step with
 * the whole batch active.  For a batch of uneven length (its shortest system
 * under half its longest) two more trials run only the systems with its
 * longest chains (steps times 2N - 3, at most 32) for the chain's time per
 * step, and the predicted time sums, step by step, the whole batch's time
 * per step scaled by the Jacobian work still active, never below the
 * chain's; for an even batch it extrapolates the two trials
 * to the longest system.  trial_ms reports the trials' times.  Before the
 * timed trials, untimed runs launch every kernel form the candidates use
 * (one-lane and team producers; for an uneven batch also the chain set's wide
 * form and team searches), so that no trial carries a kernel's first-launch
 * module loading.  The fastest candidate is kept on the
 * context (as nbg_set_tuning / nbg_set_orbit_team / nbg_set_orbit_lanes
 * would).  Arrays as for nbg_batch_integrate_transits_device.  report (may
 * be NULL) receives up to report_len candidates; *nreport (may be NULL)
 * their number.  Results of later calls do not depend on the choice.
 */
typedef struct {
  int32_t chunk_steps, orbit_team, orbit_lanes;
  int32_t producer_warps, producer_smem_kb, pad;
  double ms;                 /* predicted chunk-loop time of the full batch   */
  double system_steps_per_s; /* the batch's system-steps / that time          */
  double trial_ms[4];        /* the trials: whole batch T and 2T steps; its
                                longest systems alone T and 2T (0: not run)  */
} nbg_tuning_result;
int nbg_autotune_device(nbg_context* ctx, int nsys, const nbg_system_desc* desc_host, double* t, double* x, double* v,
                        const double* m, double* xerror, double* verror, double* jac_step, double* jac_error,
                        double* dqdt, const uint8_t* pair, const double* jac_init, int trial_steps,
                        nbg_tuning_result* report, int report_len, int* nreport);

/* Systems per warp of the orbit producer (1..32; 0 = automatic: about two
 * warps per SM).  A tuning knob; results do not depend on it. */
int nbg_set_orbit_lanes(nbg_context* ctx, int systems_per_warp);

/* Form of the orbit producer for groups without kick pairs: -1 automatic
 * (default: one lane per system up to four bodies and a team of N/2 lanes
 * per system from N = 5 on, each in its wide form in latency-bound chunks),
 * 0 one lane per system, 1 a team for every N, 2 the wide team form for
 * every N, 3 a team for every N, wide in latency-bound chunks.  A team runs
 * the Kepler sweeps and phisalpha!'s pair loops level by level (pairs with
 * equal i + j share no body and run in parallel), which keeps every body's
 * sequence of updates and so gives bitwise the same results.  The wide form
 * runs each pair solve on two lanes, each evaluating one of its independent
 * parts (the sine and cosine series, the Newton update's numerator and
 * denominator, G3 and H1): bitwise the same results with fewer FP64
 * instructions on the system's warp.  A chunk is latency-bound when at most
 * max(32, SMs / 2) of its group's systems still run.  A tuning knob; no
 * counterpart in the reference. */
int nbg_set_orbit_team(nbg_context* ctx, int mode);

/* Block layout of the orbit producer (a tuning knob; no counterpart in the
 * reference; results do not depend on it): warps_per_block (1..4)
 * independent producer warps per block, each block holding smem_kb KB of
 * shared memory (0..220), and guard_kb KB (0..100) requested by every
 * operator-record and transit-search block.  Blocks cannot share an SM when
 * their shared memory exceeds the SM's 227 KB, so smem_kb = 200 with
 * guard_kb = 32 keeps the throughput kernels off the SMs that run the
 * latency-bound producer.  Default 1, 0, 0. */
int nbg_set_producer_layout(nbg_context* ctx, int warps_per_block, int smem_kb, int guard_kb);

/* Profiling (no reference counterpart).
 * Record an event pair around kernel launches (0: off, the default; 1: every
 * orbit-producer, transit, operator and Jacobian launch; 2: the Jacobian
 * consumer's launches; 3: one consumer launch per group and call, its
 * middle chunk, with nbg_last_timing's jacobian_ms scaled to all the
 * consumer launches -- event pairs delay the overlapped streams, and one
 * pair per call perturbs them least). */
int nbg_set_profiling(nbg_context* ctx, int on);

/* Launch counts of the last call, per kernel kind (no reference
 * counterpart; measurement helpers, as the two below). */
int nbg_last_kernel_stats(nbg_context* ctx, int64_t* orbit_launches, int64_t* jacobian_launches);

/* Number of kernels launched by the last call. */
int64_t nbg_last_launch_count(nbg_context* ctx);

/* Host (wall-clock) time the last batched call spent enqueueing its chunk
 * loop -- the launch overhead a CUDA graph of the loop could save.  No
 * counterpart in the reference; a measurement helper. */
int nbg_last_host_time(nbg_context* ctx, double* enqueue_ms);

/* Measured FP64 FMA throughput of the context's device (TFLOP/s, FMA = 2
 * flops): the roofline denominator for the FP64-bound kernels.  No
 * counterpart in the reference; a measurement helper. */
int nbg_fp64_peak(nbg_context* ctx, double* tflops);

/* Measured FP64 tensor-core throughput of the context's device (TFLOP/s, one
 * mma.sync m8n8k4 f64 = 512 flops), after checking one exact product against
 * the documented fragment layout (NBG_EUNSUPPORTED if it differs).  With
 * with_dfma != 0 every DMMA is interleaved with 8 independent DFMAs of the
 * same warp and *tflops counts both; *dfma_share (may be NULL) is the DFMA
 * part of those flops.  Compared with nbg_fp64_peak this shows whether the
 * tensor path adds FP64 throughput beside the FMA pipe.  No counterpart in
 * the reference; a measurement helper. */
int nbg_fp64_mma_peak(nbg_context* ctx, int with_dfma, double* tflops, double* dfma_share);

/* FP64 issue interval of one warp: `warps` warps (1..32) of a single block,
 * each running `chains` (1, 2, 4 or 8) independent DFMA chains, timed with
 * clock64; *cycles_per_dfma is the slowest warp's SM cycles per warp-DFMA.
 * Shows the per-warp issue limit that bounds a one-system step's latency.
 * No counterpart in the reference; a measurement helper. */
int nbg_fp64_warp_issue(nbg_context* ctx, int warps, int chains, double* cycles_per_dfma);

#ifdef __cplusplus
}
#endif

#endif /* NBG_H */
