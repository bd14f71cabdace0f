// nbg_cuda.cu -- libnbg_cuda: kernels, orchestration and the C ABI (include/nbg.h).
//
// Build: nbodygradient.jl_gb300/build.py compiles this file and nbg_inst.cu
// once per body count with nvcc -gencode arch=compute_103a,code=sm_103a
// --fmad=false -O3 and links them into libnbg_cuda.so.  --fmad=false keeps
// every scalar product and sum separately rounded as in the Julia
// reference; the kernels use fma() explicitly where a fused product is
// intended (the BLAS-like operator products).
#include <cuda_runtime.h>

#include <algorithm>
#include <deque>
#include <thread>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <tuple>
#include <string>
#include <vector>

#include "../../include/nbg.h"
#include "nbg_internal.cuh"

using namespace nbg;

// Every group of a batch (and of the request server) runs on three streams of
// its own; with the driver's default of 8 hardware work queues, streams share
// queues and a group's latency-bound producer waits behind another group's
// long consumer kernel (measured: the uneven 2048-system batch 203 s -> 94 s
// per pass with 32 queues).  The library asks for 32 when it is loaded, before
// the process creates its CUDA context, unless the caller has set the
// variable itself; a context that already exists keeps its setting.
__attribute__((constructor)) static void nbg_request_work_queues() {
  setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0);
}

// ===================================================================== kernels

// Gather the caller-layout arrays of one group's systems into its SoA state.
__global__ void pack_state_kernel(int N, int S, const int* sysidx, const SysOff* off, const double* x,
                                  const double* v, const double* xe, const double* ve, const double* m,
                                  const double* dqdt, const long long* count, double* gx, double* gv, double* gxe,
                                  double* gve, double* gm, double* gdq, long long* gcnt) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S) return;
  const int gs = sysidx[s];
  if (gs < 0) return;
  const SysOff o = off[gs];
  for (int q = 0; q < 3 * N; q++) {
    gx[q * S + s] = x[o.x + q];
    gv[q * S + s] = v[o.x + q];
    gxe[q * S + s] = xe[o.x + q];
    gve[q * S + s] = ve[o.x + q];
  }
  for (int q = 0; q < N; q++) {
    gm[q * S + s] = m[o.m + q];
    gcnt[q * S + s] = count[o.cnt + q];
  }
  for (int q = 0; q < 7 * N; q++) gdq[q * S + s] = dqdt[o.dqdt + q];
}

__global__ void unpack_state_kernel(int N, int S, int grad, const int* sysidx, const SysOff* off, double* x,
                                    double* v, double* xe, double* ve, double* dqdt, long long* count,
                                    const double* gx, const double* gv, const double* gxe, const double* gve,
                                    const double* gdq, const long long* gcnt) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S) return;
  const int gs = sysidx[s];
  if (gs < 0) return;
  const SysOff o = off[gs];
  for (int q = 0; q < 3 * N; q++) {
    x[o.x + q] = gx[q * S + s];
    v[o.x + q] = gv[q * S + s];
    xe[o.x + q] = gxe[q * S + s];
    ve[o.x + q] = gve[q * S + s];
  }
  for (int q = 0; q < N; q++) count[o.cnt + q] = gcnt[q * S + s];
  if (grad)
    for (int q = 0; q < 7 * N; q++) dqdt[o.dqdt + q] = gdq[q * S + s];
}

// jac_step / jac_error non-mass rows <-> internal [S][6N][7N]; also checks
// that the mass rows are unit rows with zero error (bad[0] set otherwise).
__global__ void pack_jac_kernel(int N, int S, const int* sysidx, const SysOff* off, const double* J,
                                const double* E, double* Jint, double* Eint, int* bad) {
  const int M = 7 * N, R6 = 6 * N;
  const long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long tot = (long long)S * M * M;
  if (f >= tot) return;
  const int s = (int)(f / ((long long)M * M));
  const int rem = (int)(f % ((long long)M * M));
  const int c = rem / M, r = rem % M;  // full row r, column c
  const int gs = sysidx[s];
  if (gs < 0) return;
  const long long base = off[gs].J;
  const double jv = J[base + r + (long long)M * c];
  const double ev = E[base + r + (long long)M * c];
  if (r % 7 == 6) {
    if (jv != ((r == c) ? 1.0 : 0.0) || ev != 0.0) atomicOr(bad, 1);
    return;
  }
  const int rn = (r / 7) * 6 + r % 7;
  Jint[((size_t)s * R6 + rn) * M + c] = jv;
  Eint[((size_t)s * R6 + rn) * M + c] = ev;
  (void)R6;
}

__global__ void unpack_jac_kernel(int N, int S, const int* sysidx, const SysOff* off, double* J, double* E,
                                  const double* Jint, const double* Eint) {
  const int M = 7 * N, R6 = 6 * N;
  const long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long tot = (long long)S * R6 * M;
  if (f >= tot) return;
  const int s = (int)(f / ((long long)R6 * M));
  const int rem = (int)(f % ((long long)R6 * M));
  const int rn = rem / M, c = rem % M;
  const int gs = sysidx[s];
  if (gs < 0) return;
  const int r = (rn / 6) * 7 + rn % 6;
  const long long base = off[gs].J;
  J[base + r + (long long)M * c] = Jint[((size_t)s * R6 + rn) * M + c];
  E[base + r + (long long)M * c] = Eint[((size_t)s * R6 + rn) * M + c];
}

// calc_dtdelements! (timing.jl:112-123): one thread per output entry of one
// system; transits beyond min(count, ntt) are left untouched.  Systems are
// list[y] (or y itself without a list); with after_dtdq0 a system's output
// block follows its dtdq0 block in the dtdq0 array.
__global__ void dtdelements_kernel(int nsys, const int* list, const SysOff* off, const double* dtdq0,
                                   const double* jac_init, double* dtdel, const long long* count, int after_dtdq0) {
  const int y = blockIdx.y + gridDim.y * blockIdx.z;
  if (y >= nsys) return;
  const int gs = list ? list[y] : y;
  const SysOff o = off[gs];
  if (!o.grad) return;
  const int n = o.n, ntt = o.ntt, M = 7 * n, nr = o.nr > 1 ? o.nr : 1;
  const long long tot = (long long)nr * n * ntt * 7 * n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    // e = r + nr (j + n (c + ntt (l + 7 k)))
    const int r = (int)(e % nr);
    const long long e1 = e / nr;
    const int j = (int)(e1 % n);
    const long long c = (e1 / n) % ntt;
    const int l = (int)((e1 / ((long long)n * ntt)) % 7);
    const int k = (int)(e1 / ((long long)n * ntt * 7));
    const long long cnt = count[o.cnt + j];
    if (c >= cnt || c >= ntt) continue;
    double acc = 0.0;
    for (int p = 0; p < n; p++)
      for (int q = 0; q < 7; q++)
        acc = acc + dtdq0[o.dq + r + nr * (j + (long long)n * (c + (long long)ntt * (q + 7LL * p)))] *
                        jac_init[o.J + (7 * p + q) + (long long)M * (7 * k + l)];
    dtdel[o.dq + (after_dtdq0 ? tot : 0) + e] = acc;
  }
}

// ================================================================ host side


namespace {
thread_local std::string g_last_error;
}  // namespace

namespace nbg {

int set_error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

long long steps_of(double h, double tmax) {
  double q = std::nearbyint(tmax / h);  // round(Int64, tmax/h): ties to even
  long long n = (long long)q;
  return n < 0 ? -n : n;
}

// check_step (src/integrator/Integrator.jl:249-259)
double check_step(double t0, double tmax) {
  auto sgn = [](double x) { return x > 0 ? 1.0 : (x < 0 ? -1.0 : x); };
  if (std::fabs(tmax) > std::fabs(t0)) return sgn(tmax);
  if (sgn(tmax) != sgn(t0)) return sgn(tmax);
  return -1.0 * sgn(tmax);
}

void launch_pack_state(int N, int S, const int* sysidx, const SysOff* off, const double* x, const double* v,
                       const double* xe, const double* ve, const double* m, const double* dqdt,
                       const long long* count, const GroupArgs& g, cudaStream_t st) {
  pack_state_kernel<<<(S + 127) / 128, 128, 0, st>>>(N, S, sysidx, off, x, v, xe, ve, m, dqdt, count, g.x, g.v,
                                                      g.xe, g.ve, g.m, g.dqdt, g.count);
}

void launch_unpack_state(int N, int S, int grad, const int* sysidx, const SysOff* off, double* x, double* v,
                         double* xe, double* ve, double* dqdt, long long* count, const GroupArgs& g,
                         cudaStream_t st) {
  unpack_state_kernel<<<(S + 127) / 128, 128, 0, st>>>(N, S, grad, sysidx, off, x, v, xe, ve, dqdt, count, g.x,
                                                        g.v, g.xe, g.ve, g.dqdt, g.count);
}

void launch_pack_jac(int N, int S, const int* sysidx, const SysOff* off, const double* J, const double* E,
                     const GroupArgs& g, int* bad, cudaStream_t st) {
  const long long tot = (long long)S * 49 * N * N;
  pack_jac_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(N, S, sysidx, off, J, E, g.Jint, g.Eint, bad);
}

void launch_unpack_jac(int N, int S, const int* sysidx, const SysOff* off, double* J, double* E,
                       const GroupArgs& g, cudaStream_t st) {
  const long long tot = (long long)S * 42 * N * N;
  unpack_jac_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(N, S, sysidx, off, J, E, g.Jint, g.Eint);
}

void launch_dtdelements(int nlist, const int* list, const SysOff* off, const double* dtdq0, const double* jac_init,
                        double* dtdel, const long long* count, bool after_dtdq0, cudaStream_t st) {
  if (nlist <= 0) return;
  dim3 grid(8, std::min(nlist, 65535), (nlist + 65534) / 65535);
  dtdelements_kernel<<<grid, 256, 0, st>>>(nlist, list, off, dtdq0, jac_init, dtdel, count, after_dtdq0 ? 1 : 0);
}

}  // namespace nbg

namespace {

struct Buf {
  void* p = nullptr;
  size_t bytes = 0;
};

constexpr int kNaMax = NBG_NOALLOC_MAX_SYSTEMS;

// Host bookkeeping of nbg_batch_integrate_transits_noalloc (about 90 KB): one
// per context, allocated with the context, so that the call itself allocates
// nothing and needs little of its caller's stack.
struct NoallocPlan {
  SysOff off[kNaMax];
  long long offtt[kNaMax], offdq[kNaMax], nsteps[kNaMax];
  double hsig[kNaMax], t0[kNaMax], tout[kNaMax];
  uint8_t pair[kNaMax * NBG_MAX_BODIES * NBG_MAX_BODIES];
  int order[kNaMax];                 // systems by group, longest first within a group
  int ngroups, gstart[kNaMax + 1];   // group q owns order[gstart[q] .. gstart[q+1])
  int gN[kNaMax], ggrad[kNaMax], gof[kNaMax];
  unsigned long long gkick[kNaMax];
  long long gmax[kNaMax];
  GroupArgs g[kNaMax];
  // per-group staging of the scalars copied to the device, and the status read back
  int sidx[kNaMax], vntt[kNaMax], vti[kNaMax];
  double vt0[kNaMax], vh[kNaMax], vhI[kNaMax];
  long long vns[kNaMax];
  unsigned sv[kNaMax];
};

}  // namespace

struct nbg_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::map<std::string, Buf> pool;
  int chunk_steps = 64;
  int overlap = 1;  // orbit producer on its own stream, one chunk ahead of the rest
  int orbit_spw = 0;  // 0: automatic
  int orbit_team = -1;  // -1: automatic (teams for N >= 5), 0: one lane per system, 1: teams for every N
  int prod_warps = 1, prod_smem_kb = 0, guard_smem_kb = 0;  // orbit producer block layout
  int sm_count = 0;
  double last_total_ms = 0, last_orbit_ms = 0, last_jac_ms = 0, last_transit_ms = 0, last_ops_ms = 0;
  double last_host_ms = 0;  // host time spent enqueueing the chunk loop
  long long last_launches = 0, last_orbit_launches = 0, last_jac_launches = 0;
  int profile = 0;
  std::vector<cudaEvent_t> prof_events;  // pairs around each timed launch
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // overlap mode: per group q, a producer stream, an operator / Jacobian
  // stream and a transit-search stream (gstreams[3q .. 3q+2])
  std::vector<cudaStream_t> gstreams;
  // the same for the groups of a batch whose systems run longest: streams of
  // the device's highest priority (their blocks are dispatched first)
  std::vector<cudaStream_t> hstreams;
  std::vector<cudaEvent_t> sync_events;  // cross-stream ordering, no timing
  NoallocPlan* noalloc = nullptr;         // host plan of the allocation-free entry point

  int sync_event(size_t i, cudaEvent_t* out) {
    while (sync_events.size() <= i) {
      cudaEvent_t e;
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
        return set_error(NBG_ECUDA, "cudaEventCreateWithFlags failed");
      sync_events.push_back(e);
    }
    *out = sync_events[i];
    return NBG_OK;
  }

  int event(size_t i, cudaEvent_t* out) {
    while (prof_events.size() <= i) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) return set_error(NBG_ECUDA, "cudaEventCreate failed");
      prof_events.push_back(e);
    }
    *out = prof_events[i];
    return NBG_OK;
  }

  // Grow-only device buffer cache keyed by name.
  template <class T>
  int get(const char* name, size_t count, T** out) {
    size_t bytes = std::max<size_t>(count * sizeof(T), 16);
    Buf& b = pool[name];
    if (b.bytes < bytes) {
      if (b.p) cudaFree(b.p);
      b.p = nullptr;
      b.bytes = 0;
      cudaError_t e = cudaMalloc(&b.p, bytes);
      if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(NBG_ENOMEM, "cudaMalloc(%zu bytes) for %s: %s", bytes, name, cudaGetErrorString(e));
      }
      b.bytes = bytes;
    }
    *out = (T*)b.p;
    return NBG_OK;
  }
};

namespace {

typedef int (*LaunchFn)(const GroupArgs&, int, cudaStream_t);
typedef int (*SeedFn)(const GroupArgs&, cudaStream_t);
const LaunchFn kOrbit[NBG_MAX_BODIES + 1] = {nullptr, nullptr, launch_orbit<2>, launch_orbit<3>, launch_orbit<4>,
                                             launch_orbit<5>, launch_orbit<6>, launch_orbit<7>, launch_orbit<8>,
                                             launch_orbit<9>, launch_orbit<10>};
const LaunchFn kJac[NBG_MAX_BODIES + 1] = {nullptr, nullptr, launch_jac<2>, launch_jac<3>, launch_jac<4>,
                                           launch_jac<5>, launch_jac<6>, launch_jac<7>, launch_jac<8>,
                                           launch_jac<9>, launch_jac<10>};
const LaunchFn kTransit[NBG_MAX_BODIES + 1] = {nullptr, nullptr, launch_transit<2>, launch_transit<3>,
                                               launch_transit<4>, launch_transit<5>, launch_transit<6>,
                                               launch_transit<7>, launch_transit<8>, launch_transit<9>,
                                               launch_transit<10>};
const LaunchFn kOps[NBG_MAX_BODIES + 1] = {nullptr, nullptr, launch_operators<2>, launch_operators<3>,
                                           launch_operators<4>, launch_operators<5>, launch_operators<6>,
                                           launch_operators<7>, launch_operators<8>, launch_operators<9>,
                                           launch_operators<10>};
const SeedFn kSeed[NBG_MAX_BODIES + 1] = {nullptr, nullptr, launch_seed<2>, launch_seed<3>, launch_seed<4>,
                                          launch_seed<5>, launch_seed<6>, launch_seed<7>, launch_seed<8>,
                                          launch_seed<9>, launch_seed<10>};

}  // namespace

namespace nbg {
int launch_group_orbit(int N, const GroupArgs& g, int chunk, cudaStream_t st) { return kOrbit[N](g, chunk, st); }
int launch_group_transit(int N, const GroupArgs& g, int chunk, cudaStream_t st) { return kTransit[N](g, chunk, st); }
int launch_group_operators(int N, const GroupArgs& g, int chunk, cudaStream_t st) { return kOps[N](g, chunk, st); }
int launch_group_jacobian(int N, const GroupArgs& g, int chunk, cudaStream_t st) { return kJac[N](g, chunk, st); }
int launch_group_seed(int N, const GroupArgs& g, cudaStream_t st) { return kSeed[N](g, st); }
}  // namespace nbg

namespace {

}  // namespace

namespace nbg {
// Team producer (a team of lanes per system) for kick-free groups: automatic
// from five bodies on, where the level-parallel sweeps shorten the step's
// critical path by 1.4x (N = 5) to 2.6x (N = 10).
// Modes (nbg_set_orbit_team): -1 automatic, 0 one lane, 1 team, 2 wide
// team always, 3 team with the wide form in latency-bound chunks.
bool use_team(int mode, int N, unsigned long long kick) {
  if (kick) return false;
  return mode > 0 || (mode < 0 && N >= 5);
}

// The wide team form (two lanes per pair solve): always in mode 2, in the
// latency-bound chunks (few systems running) in modes -1 and 3.
bool use_wide(int mode, bool latency_bound, unsigned long long kick) {
  if (kick) return false;
  return mode == 2 || ((mode < 0 || mode == 3) && latency_bound);
}
}  // namespace nbg

namespace {

// A plain integration (no transit timing) of one system: the steps
// intr(s, time) or intr(s, N) takes (Integrator.jl:159-233).
struct PlainSpec {
  long long nsteps;  // steps in all, the fractional last step included
  double h;          // signed step
  double hlast;      // length of the last step (h unless it is fractional)
  double tout;       // s.t after the call
};

// CartesianOutput destination of one system (host arrays, nsteps entries
// each): t, x (3 x N), v (3 x N), jac_step (7N x 7N, may be null).
struct TrajOut {
  double *t, *x, *v, *jac;
};

struct GroupPlan {
  int N, grad;
  unsigned long long kick;
  std::vector<int> systems;  // global indices, longest first
  long long max_steps = 0;
};

// Core of every entry point.  All array pointers are device pointers in the
// caller's packed layout; desc / t0 / pair are host copies.
// plain: null for transit timing (intr(s, tt)); otherwise one PlainSpec per
// system, no transit detection and no tt / dtdq0 / dtdelements (those
// pointers and jac_init may be null; d_count must hold nsys*n zeros).
int run_batch(nbg_context* ctx, int nsys, const nbg_system_desc* desc, const double* t_host,
              const uint8_t* pair_host, double* d_t, double* d_x, double* d_v, const double* d_m, double* d_xe,
              double* d_ve, double* d_J, double* d_E, double* d_dqdt, const double* d_jinit, double* d_tt,
              double* d_dq0, double* d_dtdel, long long* d_count, uint32_t* status_host,
              const PlainSpec* plain = nullptr, int tbv = 0, const TrajOut* traj = nullptr) {
  const int nr = tbv ? 3 : 1;  // rows per transit of the outputs
  cudaStream_t st = ctx->stream;
  ctx->last_launches = 0;
  ctx->last_orbit_ms = ctx->last_jac_ms = ctx->last_transit_ms = ctx->last_ops_ms = 0;
  // ---- offsets and groups
  std::vector<SysOff> off(nsys);
  std::vector<long long> nsteps(nsys);
  std::vector<double> hsig(nsys);
  long long ax = 0, am = 0, aJ = 0, adq = 0, ap = 0, att = 0, adq0 = 0, acn = 0;
  std::map<std::tuple<int, int, unsigned long long>, GroupPlan> groups;
  for (int s = 0; s < nsys; s++) {
    const nbg_system_desc& d = desc[s];
    if (d.n < NBG_MIN_BODIES || d.n > NBG_MAX_BODIES)
      return set_error(NBG_EUNSUPPORTED, "system %d: n = %d outside the built range %d..%d", s, d.n, NBG_MIN_BODIES,
                       NBG_MAX_BODIES);
    if (d.ti < 0 || d.ti >= d.n) return set_error(NBG_EINVAL, "system %d: ti = %d not in 0..%d", s, d.ti, d.n - 1);
    if (d.ntt < 1) return set_error(NBG_EINVAL, "system %d: ntt = %d < 1", s, d.ntt);
    if (!(d.h != 0.0) || !std::isfinite(d.h) || !std::isfinite(d.tmax))
      return set_error(NBG_EINVAL, "system %d: h = %g, tmax = %g", s, d.h, d.tmax);
    const int n = d.n, M = 7 * n;
    SysOff& o = off[s];
    o.x = ax; o.m = am; o.J = aJ; o.dqdt = adq; o.pair = ap; o.tt = att; o.dq = adq0; o.cnt = acn;
    o.n = n; o.ntt = d.ntt; o.grad = d.grad ? 1 : 0; o.nr = nr;
    ax += 3 * n; am += n; aJ += (long long)M * M; adq += M; ap += (long long)n * n;
    att += (long long)nr * n * d.ntt; adq0 += (long long)nr * n * d.ntt * 7 * n; acn += n;
    if (plain) {
      nsteps[s] = plain[s].nsteps;
      hsig[s] = plain[s].h;
    } else {
      nsteps[s] = steps_of(d.h, d.tmax);
      hsig[s] = d.h * check_step(t_host[s], d.tmax + t_host[s]);
    }
    unsigned long long kick = 0;
    for (int i = 0; i < n - 1; i++)
      for (int j = i + 1; j < n; j++)
        if (pair_host[o.pair + i + (long long)n * j]) kick |= 1ull << pair_bit(i, j, n);
    GroupPlan& gp = groups[std::make_tuple(n, o.grad, kick)];
    gp.N = n; gp.grad = o.grad; gp.kick = kick;
    gp.systems.push_back(s);
    gp.max_steps = std::max(gp.max_steps, nsteps[s]);
  }
  SysOff* d_off;
  int rc;
  if ((rc = ctx->get("off", (size_t)nsys, &d_off))) return rc;
  NBG_CUDA(cudaMemcpyAsync(d_off, off.data(), sizeof(SysOff) * nsys, cudaMemcpyHostToDevice, st));
  long long* d_offtt;
  long long* d_offdq;
  if ((rc = ctx->get("offtt", (size_t)nsys, &d_offtt))) return rc;
  if ((rc = ctx->get("offdq", (size_t)nsys, &d_offdq))) return rc;
  {
    std::vector<long long> a(nsys), b(nsys);
    for (int s = 0; s < nsys; s++) { a[s] = off[s].tt; b[s] = off[s].dq; }
    NBG_CUDA(cudaMemcpyAsync(d_offtt, a.data(), sizeof(long long) * nsys, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(d_offdq, b.data(), sizeof(long long) * nsys, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaStreamSynchronize(st));  // host vectors a, b go out of scope
  }
  // Steps per chunk: the context's setting, shortened (not below 8) where a
  // group's operator records for one chunk would pass 4 GiB per buffer half.
  int K = std::max(1, ctx->chunk_steps);
  for (auto& kv : groups) {
    const GroupPlan& gp = kv.second;
    if (!gp.grad) continue;
    int npk = 0;
    for (int i = 0; i < gp.N - 1; i++)
      for (int j = i + 1; j < gp.N; j++)
        if (!((gp.kick >> pair_bit(i, j, gp.N)) & 1)) npk++;
    const double per_step = 8.0 * step_record_size(gp.N, npk, gp.kick != 0) * (((gp.systems.size() + 31) / 32) * 32);
    const int kmax = (int)std::min(4096.0, std::floor(4294967296.0 / per_step));
    K = std::min(K, std::max(std::min(K, 8), kmax));
  }
  // ---- per-group device state
  std::vector<GroupArgs> gargs;
  std::vector<GroupArgs> ghalf;  // the same groups on the second half of the per-chunk buffers
  int* d_bad;
  if ((rc = ctx->get("bad", 1, &d_bad))) return rc;
  NBG_CUDA(cudaMemsetAsync(d_bad, 0, sizeof(int), st));
  int gi = 0;
  std::vector<long long> gmaxsteps;
  std::vector<std::vector<long long>> gsteps;  // per group, its systems' step counts, longest first
  for (auto& kv : groups) {
    GroupPlan& gp = kv.second;
    std::stable_sort(gp.systems.begin(), gp.systems.end(),
                     [&](int a, int b) { return nsteps[a] > nsteps[b]; });
    const int N = gp.N, nsg = (int)gp.systems.size();
    const int S = ((nsg + 31) / 32) * 32;
    GroupArgs g;
    memset(&g, 0, sizeof(g));
    g.N = N; g.S = S; g.nsys = nsg; g.grad = gp.grad; g.K = K; g.kick = gp.kick; g.tbv = tbv;
    // Orbit producer lanes per warp.  A warp's FP64 instruction occupies its
    // SM sub-partition's FP64 pipe for the same time at any lane count, and
    // one producer warp per sub-partition runs its chain at the same speed
    // whatever its lane count; with the overlapped streams, full warps leave
    // the most FP64 issue slots to the kernels running beside the producer.
    // Without overlap a small batch is spread over about two warps per SM.
    g.team = use_team(ctx->orbit_team, N, gp.kick) && ctx->orbit_spw == 0;
    g.pwarps = ctx->prod_warps;
    g.prod_smem = ctx->prod_smem_kb * 1024;
    g.guard_smem = ctx->guard_smem_kb * 1024;
    if (ctx->orbit_spw > 0) {
      g.spw = ctx->orbit_spw;
    } else if (ctx->overlap) {
      g.spw = 32;
    } else {
      int target = std::max(1, 2 * ctx->sm_count);
      int want = (nsg + target - 1) / target, spw = 1;
      while (spw < want && spw < 32) spw *= 2;
      g.spw = spw;
    }
    int npk = 0;
    for (int i = 0; i < N - 1; i++)
      for (int j = i + 1; j < N; j++)
        if (!((gp.kick >> pair_bit(i, j, N)) & 1)) npk++;
    g.npk = npk;
    g.R = step_record_size(N, npk, gp.kick != 0);
    char nm[64];
    auto name = [&](const char* f) { snprintf(nm, sizeof(nm), "g%d_%s", gi, f); return nm; };
#define GET(field, cnt) if ((rc = ctx->get(name(#field), (size_t)(cnt), &g.field))) return rc
    GET(x, 3 * N * S); GET(v, 3 * N * S); GET(xe, 3 * N * S); GET(ve, 3 * N * S); GET(m, N * S);
    GET(dqdt, 7 * N * S); GET(gsave, N * S); GET(count, N * S); GET(t0, S); GET(h, S); GET(hI, S);
    GET(nsteps, S); GET(ntt, S); GET(ti, S); GET(sysidx, S); GET(status, S);
    double* hlast = nullptr;
    if (plain) {
      if ((rc = ctx->get(name("hlast"), (size_t)S, &hlast))) return rc;
      g.hlast = hlast;
      g.notransit = 1;
    }
    g.task_cap = K * (N - 1) * S;
    // Per-chunk buffers (the transit queue, the captures and the records) are
    // double-buffered in overlap mode: chunk c uses half c % 2.
    const size_t nf = (size_t)g.task_cap * (12 * N + 2), ni = (size_t)g.task_cap * 3;
    const size_t nrec = (size_t)K * g.R * S, ntrec = (size_t)K * (N - 1) * trec_size(N, tbv) * S;
    const size_t nflag = (size_t)K * (N - 1) * S, ncap = (size_t)K * 2 * npk * PCAP * S + 1;
    const size_t nsnap = (size_t)K * snap_count(gp.kick != 0) * 3 * N * S;
    const int nb = ctx->overlap ? 2 : 1;
    GET(task_f, nb * nf); GET(task_i, nb * ni); GET(task_count, nb);
    size_t ntxv = 0, ntJ = 0;
    if (traj) {
      bool jac = false;
      for (int q2 = 0; q2 < nsg; q2++) jac = jac || traj[gp.systems[q2]].jac;
      ntxv = (size_t)S * K * 6 * N;
      ntJ = jac ? (size_t)S * K * 49 * N * N : 0;
      if ((rc = ctx->get(name("trajxv"), nb * ntxv, &g.trajxv))) return rc;
      if (ntJ && (rc = ctx->get(name("trajJ"), nb * ntJ, &g.trajJ))) return rc;
    }
    g.tgrid = std::min(((g.task_cap + 31) / 32) * 32, std::max(1, ctx->sm_count) * 4 * 32);
    if (gp.grad) {
      GET(steprec, nb * nrec); GET(trec, nb * ntrec); GET(tflag, nb * nflag); GET(tscratch, (size_t)g.R * g.tgrid);
      GET(pcap, nb * ncap); GET(xsnap, nb * nsnap);
      GET(Jint, (size_t)S * 6 * N * 7 * N); GET(Eint, (size_t)S * 6 * N * 7 * N);
    }
#undef GET
    g.tt = d_tt; g.off_tt = d_offtt; g.dtdq0 = d_dq0; g.off_dq = d_offdq;
    // host-side scalars
    std::vector<int> sidx(S, -1), vntt(S, 1), vti(S, 0);
    std::vector<double> vt0(S, 0.0), vh(S, 0.0), vhI(S, 0.0), vhl(S, 0.0);
    std::vector<long long> vns(S, 0);
    for (int q = 0; q < nsg; q++) {
      int s = gp.systems[q];
      sidx[q] = s; vntt[q] = desc[s].ntt; vti[q] = desc[s].ti;
      vt0[q] = t_host[s]; vh[q] = hsig[s]; vhI[q] = desc[s].h; vns[q] = nsteps[s];
      if (plain) vhl[q] = plain[s].hlast;
    }
    if (plain) NBG_CUDA(cudaMemcpyAsync(hlast, vhl.data(), sizeof(double) * S, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(g.sysidx, sidx.data(), sizeof(int) * S, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(g.ntt, vntt.data(), sizeof(int) * S, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(g.ti, vti.data(), sizeof(int) * S, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(g.t0, vt0.data(), sizeof(double) * S, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(g.h, vh.data(), sizeof(double) * S, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(g.hI, vhI.data(), sizeof(double) * S, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(g.nsteps, vns.data(), sizeof(long long) * S, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaMemsetAsync(g.status, 0, sizeof(unsigned) * S, st));
    NBG_CUDA(cudaStreamSynchronize(st));
    // gather state
    int pb = (S + 127) / 128;
    pack_state_kernel<<<pb, 128, 0, st>>>(N, S, g.sysidx, d_off, d_x, d_v, d_xe, d_ve, d_m, d_dqdt, d_count, g.x,
                                          g.v, g.xe, g.ve, g.m, g.dqdt, g.count);
    ctx->last_launches++;
    if (gp.grad) {
      long long tot = (long long)S * 49 * N * N;
      pack_jac_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(N, S, g.sysidx, d_off, d_J, d_E, g.Jint, g.Eint,
                                                                     d_bad);
      ctx->last_launches++;
    }
    gargs.push_back(g);
    {
      GroupArgs h1 = g;
      h1.task_f += nf; h1.task_i += ni; h1.task_count += 1;
      if (g.trajxv) h1.trajxv += ntxv;
      if (g.trajJ) h1.trajJ += ntJ;
      if (gp.grad) { h1.steprec += nrec; h1.trec += ntrec; h1.tflag += nflag; h1.pcap += ncap; h1.xsnap += nsnap; }
      ghalf.push_back(h1);
    }
    gmaxsteps.push_back(gp.max_steps);
    gsteps.emplace_back();
    for (int sidx : gp.systems) gsteps.back().push_back(nsteps[sidx]);
    gi++;
  }
  NBG_CUDA(cudaGetLastError());
  int bad = 0;
  NBG_CUDA(cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaStreamSynchronize(st));
  if (bad)
    return set_error(NBG_EUNSUPPORTED,
                     "jac_step mass rows must be unit rows with zero jac_error (true for every State the reference "
                     "builds and integrates)");
  for (auto& g : gargs) {
    kSeed[g.N](g, st);
    ctx->last_launches++;
  }
  // ---- chunk loop
  long long max_steps = 0;
  for (auto& kv : groups) max_steps = std::max(max_steps, kv.second.max_steps);
  const long long nchunks = (max_steps + K - 1) / K;
  // CartesianOutput: after a chunk's consumer, its recorded states go to the
  // callers' arrays (stream-ordered before the buffer half is reused)
  std::vector<std::vector<std::pair<int, int>>> gtraj(gargs.size());  // (system, slot) per group
  if (traj) {
    int qg = 0;
    for (auto& kv : groups) {
      for (int q2 = 0; q2 < (int)kv.second.systems.size(); q2++) gtraj[qg].emplace_back(kv.second.systems[q2], q2);
      qg++;
    }
  }
  auto copy_traj = [&](size_t q, const GroupArgs& g, long long c, cudaStream_t s2) -> int {
    if (!traj) return NBG_OK;
    const int N = g.N, M = 7 * N;
    for (auto& ss : gtraj[q]) {
      const TrajOut& o = traj[ss.first];
      const long long k0 = c * K, kn = std::min<long long>(K, nsteps[ss.first] - k0);
      if (kn <= 0) continue;
      const double* src = g.trajxv + (size_t)ss.second * K * 6 * N;
      NBG_CUDA(cudaMemcpy2DAsync(o.x + k0 * 3 * N, sizeof(double) * 3 * N, src, sizeof(double) * 6 * N,
                                 sizeof(double) * 3 * N, (size_t)kn, cudaMemcpyDeviceToHost, s2));
      NBG_CUDA(cudaMemcpy2DAsync(o.v + k0 * 3 * N, sizeof(double) * 3 * N, src + 3 * N, sizeof(double) * 6 * N,
                                 sizeof(double) * 3 * N, (size_t)kn, cudaMemcpyDeviceToHost, s2));
      if (o.jac && g.trajJ)
        NBG_CUDA(cudaMemcpyAsync(o.jac + k0 * M * M, g.trajJ + (size_t)ss.second * K * M * M,
                                 sizeof(double) * kn * M * M, cudaMemcpyDeviceToHost, s2));
    }
    return NBG_OK;
  };
  // profiling: an event pair around every launch (level 1), every Jacobian
  // consumer launch (2), or one consumer launch per group -- its middle
  // chunk (3)
  std::vector<std::pair<int, size_t>> prof;  // (kind, first event index)
  size_t nev = 0;
  bool sample_now = false;  // level 3: this launch is the group's sampled one
  long long sampled = 0;
  auto skip = [&](int kind) {
    return !ctx->profile || (ctx->profile >= 2 && kind != 1) || (ctx->profile == 3 && !sample_now);
  };
  auto timed = [&](int kind, auto&& launch) -> int {
    if (skip(kind)) return launch();
    cudaEvent_t a, b;
    int r;
    if ((r = ctx->event(nev, &a)) || (r = ctx->event(nev + 1, &b))) return r;
    cudaEventRecord(a, st);
    r = launch();
    cudaEventRecord(b, st);
    prof.emplace_back(kind, nev);
    nev += 2;
    return r;
  };
  // the same on another stream: the event pair brackets the launch on the
  // stream it is launched on
  auto timed_on = [&](cudaStream_t s2, int kind, auto&& launch) -> int {
    if (skip(kind)) return launch();
    cudaEvent_t a, b;
    int r;
    if ((r = ctx->event(nev, &a)) || (r = ctx->event(nev + 1, &b))) return r;
    cudaEventRecord(a, s2);
    r = launch();
    cudaEventRecord(b, s2);
    prof.emplace_back(kind, nev);
    nev += 2;
    return r;
  };
  // The transit searches of a chunk take the team form once few of the
  // group's systems still run (the long tail of an uneven batch, where the
  // searches are latency-bound); while many run, one lane per search keeps
  // every lane busy.  The same kernels' results either way (bitwise).
  //
  // In the same tail the group's orbit producer runs on SMs of its own: its
  // blocks ask for 210 KB of shared memory, and from the first tail chunk on
  // every operator-record and search block asks for at least 18 KB, so that
  // no other block fits beside a producer block (every consumer block needs
  // 24 KB or more).  A producer warp then has its SM's FP64 pipe to itself
  // instead of sharing it with the throughput kernels of the other groups;
  // while many systems run, the layout stays the autotuner's.
  const int tail_max = std::max(32, ctx->sm_count / 2);
  bool tail_any = false;
  auto active_at = [&](size_t q, long long c) -> long long {
    const std::vector<long long>& st_q = gsteps[q];
    const long long first = c * K;
    // systems with steps left at this chunk: a prefix of the longest-first list
    long long lo = 0, hi = (long long)st_q.size();
    while (lo < hi) {
      const long long mid = (lo + hi) / 2;
      if (st_q[mid] > first) lo = mid + 1;
      else hi = mid;
    }
    return lo;
  };
  auto search_args = [&](size_t q, const GroupArgs& g, long long c) {
    GroupArgs gx = g;
    gx.search_team = (active_at(q, c) <= tail_max) ? 1 : 0;
    if (tail_any) gx.guard_smem = std::max(gx.guard_smem, 18 * 1024);
    return gx;
  };
  auto orbit_args = [&](size_t q, const GroupArgs& g, long long c) {
    GroupArgs gx = g;
    const bool tail = active_at(q, c) <= tail_max;
    if (tail) gx.prod_smem = std::max(gx.prod_smem, 210 * 1024);
    gx.wide = use_wide(ctx->orbit_team, tail, g.kick) ? 1 : 0;
    return gx;
  };
  auto ops_args = [&](const GroupArgs& g) {
    GroupArgs gx = g;
    if (tail_any) gx.guard_smem = std::max(gx.guard_smem, 18 * 1024);
    return gx;
  };
  ctx->last_orbit_launches = ctx->last_jac_launches = 0;
  NBG_CUDA(cudaEventRecord(ctx->ev0, st));
  const auto host0 = std::chrono::steady_clock::now();
  if (!ctx->overlap) {
    for (long long c = 0; c < nchunks; c++) {
      for (size_t q = 0; q < gargs.size(); q++) {
        const GroupArgs& g = gargs[q];
        if (c * K >= gmaxsteps[q]) continue;
        NBG_CUDA(cudaMemsetAsync(g.task_count, 0, sizeof(int), st));
        if ((rc = timed(0, [&] { return kOrbit[g.N](orbit_args(q, g, c), (int)c, st); }))) return rc;
        if (!g.notransit && (rc = timed(2, [&] { return kTransit[g.N](search_args(q, g, c), (int)c, st); })))
          return rc;
        ctx->last_launches += g.notransit ? 1 : 2;
        ctx->last_orbit_launches++;
        if (g.grad) {
          if ((rc = timed(3, [&] { return kOps[g.N](g, (int)c, st); }))) return rc;
          sample_now = (c == ((gmaxsteps[q] + K - 1) / K) / 2);
          sampled += (ctx->profile == 3 && sample_now) ? 1 : 0;
          if ((rc = timed(1, [&] { return kJac[g.N](g, (int)c, st); }))) return rc;
          ctx->last_launches += 3;
          ctx->last_jac_launches++;
        }
        if ((rc = copy_traj(q, g, c, st))) return rc;
      }
    }
  } else {
    // Three streams per group.  sp runs the group's orbit producer, chunk
    // after chunk; once the producer has finished chunk c, stt runs chunk
    // c's transit searches while sw runs its operator kernels, and then
    // (after the searches) its Jacobian consumer.  Chunk c + 2 reuses chunk
    // c's buffer half, so the producer waits for chunk c's consumer before it
    // starts chunk c + 2.  The producer thus runs one chunk ahead, and the
    // latency-bound producer and search warps share the SMs with the
    // throughput-bound operator and Jacobian kernels.  With a stream triple of
    // its own, every group (body count, grad, pair pattern) progresses
    // independently: its chunk chain is not held up by another group's.
    //
    // In a batch of several groups, the groups whose longest chain is at
    // least half the batch's longest get streams of the highest priority:
    // their blocks are dispatched before the other groups' as SMs free up, so
    // that the long chains' pipelines are not held back by the short groups'
    // throughput work (the results do not depend on it).  A chain's length
    // is its longest system's steps times 2N - 3, the pair solves on the
    // critical path of a team step.
    const size_t ng = gargs.size();
    auto chain_len = [&](size_t q) { return (double)gmaxsteps[q] * (2.0 * gargs[q].N - 3.0); };
    double longest_all = 0.0;
    for (size_t q = 0; q < ng; q++) longest_all = std::max(longest_all, chain_len(q));
    std::vector<cudaStream_t> gstr(3 * ng);
    {
      size_t nlo = 0, nhi = 0;
      int prio_lo = 0, prio_hi = 0;
      NBG_CUDA(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
      for (size_t q = 0; q < ng; q++) {
        const bool hi = ng > 1 && 2.0 * chain_len(q) >= longest_all;
        std::vector<cudaStream_t>& pool = hi ? ctx->hstreams : ctx->gstreams;
        size_t& used = hi ? nhi : nlo;
        while (pool.size() < used + 3) {
          cudaStream_t s2;
          NBG_CUDA(cudaStreamCreateWithPriority(&s2, cudaStreamNonBlocking, hi ? prio_hi : prio_lo));
          pool.push_back(s2);
        }
        for (int r = 0; r < 3; r++) gstr[3 * q + r] = pool[used + r];
        used += 3;
      }
    }
    cudaEvent_t evs;
    if ((rc = ctx->sync_event(0, &evs))) return rc;
    NBG_CUDA(cudaEventRecord(evs, st));
    for (size_t q = 0; q < 3 * ng; q++) NBG_CUDA(cudaStreamWaitEvent(gstr[q], evs, 0));  // after the packing
    // Each group is enqueued at its own pace: at most kAhead of its chunks are
    // queued on the GPU, and the host adds a group's next chunk once one of
    // its queued chunks has completed (an event per chunk, polled).  Groups of
    // short or cheap systems thus run ahead and finish, instead of being held
    // to the slowest group's pace by a launch queue that the slowest group
    // keeps full.
    constexpr int kAhead = 4;
    std::vector<long long> next_chunk(ng, 0), nch(ng);
    std::vector<std::deque<long long>> queued(ng);
    for (size_t q = 0; q < ng; q++) nch[q] = (gmaxsteps[q] + K - 1) / K;
    auto chunk_event = [&](size_t q, long long c, cudaEvent_t* ev) {
      return ctx->sync_event(8 + 6 * ng + (kAhead + 1) * q + (size_t)(c % (kAhead + 1)), ev);
    };
    size_t remaining = 0;
    for (size_t q = 0; q < ng; q++) remaining += nch[q] > 0 ? 1 : 0;
    while (remaining > 0) {
      bool progressed = false;
      for (size_t q = 0; q < ng; q++) {
        while (!queued[q].empty()) {
          cudaEvent_t evq;
          if ((rc = chunk_event(q, queued[q].front(), &evq))) return rc;
          const cudaError_t e = cudaEventQuery(evq);
          if (e == cudaErrorNotReady) break;
          if (e != cudaSuccess) return set_error(NBG_ECUDA, "chunk failed: %s", cudaGetErrorString(e));
          queued[q].pop_front();
        }
        if (next_chunk[q] >= nch[q] || (int)queued[q].size() >= kAhead) continue;
        const long long c = next_chunk[q]++;
        if (next_chunk[q] == nch[q]) remaining--;
        progressed = true;
        const int par = (int)(c & 1);
        const GroupArgs& g = par ? ghalf[q] : gargs[q];
        cudaStream_t sp = gstr[3 * q], sw = gstr[3 * q + 1], stt = gstr[3 * q + 2];
        cudaEvent_t ev_orb, ev_done, ev_tr;
        if ((rc = ctx->sync_event(2 + 6 * q + par, &ev_orb)) || (rc = ctx->sync_event(4 + 6 * q + par, &ev_done)) ||
            (rc = ctx->sync_event(6 + 6 * q + par, &ev_tr)))
          return rc;
        if (c >= 2) NBG_CUDA(cudaStreamWaitEvent(sp, ev_done, 0));
        NBG_CUDA(cudaMemsetAsync(g.task_count, 0, sizeof(int), sp));
        if (active_at(q, c) <= tail_max) tail_any = true;
        if ((rc = timed_on(sp, 0, [&] { return kOrbit[g.N](orbit_args(q, g, c), (int)c, sp); }))) return rc;
        NBG_CUDA(cudaEventRecord(ev_orb, sp));
        NBG_CUDA(cudaStreamWaitEvent(stt, ev_orb, 0));
        NBG_CUDA(cudaStreamWaitEvent(sw, ev_orb, 0));
        if (!g.notransit && (rc = timed_on(stt, 2, [&] { return kTransit[g.N](search_args(q, g, c), (int)c, stt); })))
          return rc;
        NBG_CUDA(cudaEventRecord(ev_tr, stt));
        ctx->last_launches += g.notransit ? 1 : 2;
        ctx->last_orbit_launches++;
        if (g.grad) {
          if ((rc = timed_on(sw, 3, [&] { return kOps[g.N](ops_args(g), (int)c, sw); }))) return rc;
          NBG_CUDA(cudaStreamWaitEvent(sw, ev_tr, 0));
          sample_now = (c == ((gmaxsteps[q] + K - 1) / K) / 2);
          sampled += (ctx->profile == 3 && sample_now) ? 1 : 0;
          if ((rc = timed_on(sw, 1, [&] { return kJac[g.N](g, (int)c, sw); }))) return rc;
          ctx->last_launches += 3;
          ctx->last_jac_launches++;
        } else {
          NBG_CUDA(cudaStreamWaitEvent(sw, ev_tr, 0));
        }
        if ((rc = copy_traj(q, g, c, sw))) return rc;
        NBG_CUDA(cudaEventRecord(ev_done, sw));
        cudaEvent_t evq;
        if ((rc = chunk_event(q, c, &evq))) return rc;
        NBG_CUDA(cudaEventRecord(evq, sw));
        queued[q].push_back(c);
      }
      if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    // join: everything after runs on st (an event recorded on a stream and
    // waited on at once may be re-recorded for the next stream)
    for (size_t q = 0; q < 3 * ng; q++) {
      cudaEvent_t ej;
      if ((rc = ctx->sync_event(1, &ej))) return rc;
      NBG_CUDA(cudaEventRecord(ej, gstr[q]));
      NBG_CUDA(cudaStreamWaitEvent(st, ej, 0));
    }
  }
  NBG_CUDA(cudaGetLastError());
  NBG_CUDA(cudaEventRecord(ctx->ev1, st));
  ctx->last_host_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - host0).count();
  // ---- outputs
  for (auto& g : gargs) {
    int pb = (g.S + 127) / 128;
    unpack_state_kernel<<<pb, 128, 0, st>>>(g.N, g.S, g.grad, g.sysidx, d_off, d_x, d_v, d_xe, d_ve, d_dqdt, d_count,
                                            g.x, g.v, g.xe, g.ve, g.dqdt, g.count);
    ctx->last_launches++;
    if (g.grad) {
      long long tot = (long long)g.S * 42 * g.N * g.N;
      unpack_jac_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(g.N, g.S, g.sysidx, d_off, d_J, d_E, g.Jint,
                                                                       g.Eint);
      ctx->last_launches++;
    }
  }
  if (!plain) {
    dim3 grid(8, std::min(nsys, 65535), (nsys + 65534) / 65535);
    dtdelements_kernel<<<grid, 256, 0, st>>>(nsys, nullptr, d_off, d_dq0, d_jinit, d_dtdel, d_count, 0);
    ctx->last_launches++;
  }
  // s.t = t0 + nsteps * h (Transits.jl:161 at the last step); the plain
  // drivers set it themselves (Integrator.jl:196, :228)
  {
    std::vector<double> tout(nsys);
    for (int s = 0; s < nsys; s++)
      tout[s] = plain ? plain[s].tout : (nsteps[s] > 0 ? t_host[s] + (double)nsteps[s] * hsig[s] : t_host[s]);
    NBG_CUDA(cudaMemcpyAsync(d_t, tout.data(), sizeof(double) * nsys, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaStreamSynchronize(st));
  }
  NBG_CUDA(cudaGetLastError());
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  ctx->last_total_ms = ms;
  for (auto& pr : prof) {
    float e = 0;
    cudaEventElapsedTime(&e, ctx->prof_events[pr.second], ctx->prof_events[pr.second + 1]);
    (pr.first == 1 ? ctx->last_jac_ms : pr.first == 2 ? ctx->last_transit_ms
                                      : pr.first == 3 ? ctx->last_ops_ms : ctx->last_orbit_ms) += e;
  }
  // level 3: the sampled launches stand for all of them
  if (ctx->profile == 3 && sampled > 0) ctx->last_jac_ms *= (double)ctx->last_jac_launches / (double)sampled;
  if (status_host) {
    std::fill(status_host, status_host + nsys, 0u);
    for (auto& g : gargs) {
      std::vector<unsigned> sv(g.S);
      std::vector<int> si(g.S);
      NBG_CUDA(cudaMemcpy(sv.data(), g.status, sizeof(unsigned) * g.S, cudaMemcpyDeviceToHost));
      NBG_CUDA(cudaMemcpy(si.data(), g.sysidx, sizeof(int) * g.S, cudaMemcpyDeviceToHost));
      for (int q = 0; q < g.S; q++)
        if (si[q] >= 0) status_host[si[q]] = sv[q];
    }
  }
  return NBG_OK;
}

}  // namespace

// ====================================================== allocation-free call
//
// nbg_batch_integrate_transits_noalloc runs the same kernels in the same
// order as run_batch, but takes every device buffer from the fixed scratch
// array of nbg_noalloc.cu (bump allocation, 256-byte aligned) and keeps its
// host bookkeeping in the context's NoallocPlan.  The steps per chunk (and the transit
// kernel's thread count) shrink until the working set fits; neither changes
// the arithmetic of any system.

cudaError_t nbg_noalloc_scratch(int device, unsigned char** out);  // nbg_noalloc.cu

namespace {

struct ScratchArena {
  unsigned char* base;  // nullptr: measure only
  size_t used;
  template <class T>
  void take(T** out, size_t count) {
    const size_t bytes = std::max<size_t>(count * sizeof(T), 16);
    const size_t at = (used + 255) / 256 * 256;
    used = at + bytes;
    *out = base ? (T*)(base + at) : nullptr;
  }
};

// Carves the device buffers of every group for chunk length K and transit
// grid cap tcap; with a.base == nullptr it only measures.
void noalloc_layout(NoallocPlan& P, ScratchArena& a, int nsys, int K, int tcap, SysOff** d_off,
                    long long** d_offtt, long long** d_offdq, int** d_bad) {
  a.take(d_off, (size_t)nsys);
  a.take(d_offtt, (size_t)nsys);
  a.take(d_offdq, (size_t)nsys);
  a.take(d_bad, 1);
  for (int q = 0; q < P.ngroups; q++) {
    GroupArgs& g = P.g[q];
    const int N = g.N, S = g.S;
    g.K = K;
    g.task_cap = K * (N - 1) * S;
    g.tgrid = std::min(((g.task_cap + 31) / 32) * 32, tcap);
    a.take(&g.x, 3 * N * S); a.take(&g.v, 3 * N * S); a.take(&g.xe, 3 * N * S); a.take(&g.ve, 3 * N * S);
    a.take(&g.m, N * S); a.take(&g.dqdt, 7 * N * S); a.take(&g.gsave, N * S); a.take(&g.count, N * S);
    a.take(&g.t0, S); a.take(&g.h, S); a.take(&g.hI, S); a.take(&g.nsteps, S); a.take(&g.ntt, S);
    a.take(&g.ti, S); a.take(&g.sysidx, S); a.take(&g.status, S);
    a.take(&g.task_f, (size_t)g.task_cap * (12 * N + 2)); a.take(&g.task_i, (size_t)g.task_cap * 3);
    a.take(&g.task_count, 1);
    if (g.grad) {
      a.take(&g.steprec, (size_t)K * g.R * S); a.take(&g.trec, (size_t)K * (N - 1) * trec_size(N, 0) * S);
      a.take(&g.tflag, (size_t)K * (N - 1) * S); a.take(&g.tscratch, (size_t)g.R * g.tgrid);
      a.take(&g.pcap, (size_t)K * 2 * g.npk * PCAP * S + 1);
      a.take(&g.xsnap, (size_t)K * snap_count(g.kick != 0) * 3 * N * S);
      a.take(&g.Jint, (size_t)S * 6 * N * 7 * N); a.take(&g.Eint, (size_t)S * 6 * N * 7 * N);
    }
  }
}

int run_batch_noalloc(nbg_context* ctx, NoallocPlan& P, int nsys, const nbg_system_desc* desc, double* d_t,
                      double* d_x, double* d_v, const double* d_m, double* d_xe, double* d_ve, double* d_J,
                      double* d_E, double* d_dqdt, const uint8_t* d_pair, const double* d_jinit, double* d_tt,
                      double* d_dq0, double* d_dtdel, long long* d_count, uint32_t* status_host) {
  cudaStream_t st = ctx->stream;
  ctx->last_launches = 0;
  ctx->last_orbit_ms = ctx->last_jac_ms = ctx->last_transit_ms = ctx->last_ops_ms = 0;
  ctx->last_orbit_launches = ctx->last_jac_launches = 0;
  // ---- offsets, steps, groups (host, no heap)
  long long ax = 0, am = 0, aJ = 0, adq = 0, ap = 0, att = 0, adq0 = 0, acn = 0;
  for (int s = 0; s < nsys; s++) {
    const nbg_system_desc& d = desc[s];
    if (d.n < NBG_MIN_BODIES || d.n > NBG_MAX_BODIES)
      return set_error(NBG_EUNSUPPORTED, "system %d: n = %d outside the built range %d..%d", s, d.n, NBG_MIN_BODIES,
                       NBG_MAX_BODIES);
    if (d.ti < 0 || d.ti >= d.n) return set_error(NBG_EINVAL, "system %d: ti = %d not in 0..%d", s, d.ti, d.n - 1);
    if (d.ntt < 1) return set_error(NBG_EINVAL, "system %d: ntt = %d < 1", s, d.ntt);
    if (!(d.h != 0.0) || !std::isfinite(d.h) || !std::isfinite(d.tmax))
      return set_error(NBG_EINVAL, "system %d: h = %g, tmax = %g", s, d.h, d.tmax);
    const int n = d.n, M = 7 * n;
    SysOff& o = P.off[s];
    o.x = ax; o.m = am; o.J = aJ; o.dqdt = adq; o.pair = ap; o.tt = att; o.dq = adq0; o.cnt = acn;
    o.n = n; o.ntt = d.ntt; o.grad = d.grad ? 1 : 0; o.nr = 0;
    P.offtt[s] = att;
    P.offdq[s] = adq0;
    ax += 3 * n; am += n; aJ += (long long)M * M; adq += M; ap += (long long)n * n;
    att += (long long)n * d.ntt; adq0 += (long long)n * d.ntt * 7 * n; acn += n;
  }
  // start times and pair flags steer the plan: bring them to the host
  NBG_CUDA(cudaMemcpyAsync(P.t0, d_t, sizeof(double) * nsys, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(P.pair, d_pair, (size_t)ap, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaStreamSynchronize(st));
  P.ngroups = 0;
  int* gof = P.gof;
  for (int s = 0; s < nsys; s++) {
    const int n = desc[s].n;
    P.nsteps[s] = steps_of(desc[s].h, desc[s].tmax);
    P.hsig[s] = desc[s].h * check_step(P.t0[s], desc[s].tmax + P.t0[s]);
    unsigned long long kick = 0;
    for (int i = 0; i < n - 1; i++)
      for (int j = i + 1; j < n; j++)
        if (P.pair[P.off[s].pair + i + (long long)n * j]) kick |= 1ull << pair_bit(i, j, n);
    int q = 0;
    while (q < P.ngroups && !(P.gN[q] == n && P.ggrad[q] == P.off[s].grad && P.gkick[q] == kick)) q++;
    if (q == P.ngroups) {
      P.gN[q] = n; P.ggrad[q] = P.off[s].grad; P.gkick[q] = kick; P.gmax[q] = 0;
      P.ngroups++;
    }
    gof[s] = q;
    P.gmax[q] = std::max(P.gmax[q], P.nsteps[s]);
  }
  // order: by group, then by steps (longest first, stable)
  int pos = 0;
  for (int q = 0; q < P.ngroups; q++) {
    P.gstart[q] = pos;
    for (int s = 0; s < nsys; s++)
      if (gof[s] == q) {
        int k = pos++;
        while (k > P.gstart[q] && P.nsteps[P.order[k - 1]] < P.nsteps[s]) {
          P.order[k] = P.order[k - 1];
          k--;
        }
        P.order[k] = s;
      }
  }
  P.gstart[P.ngroups] = pos;
  for (int q = 0; q < P.ngroups; q++) {
    GroupArgs& g = P.g[q];
    memset(&g, 0, sizeof(g));
    const int N = P.gN[q], nsg = P.gstart[q + 1] - P.gstart[q];
    g.N = N; g.S = ((nsg + 31) / 32) * 32; g.nsys = nsg; g.grad = P.ggrad[q]; g.kick = P.gkick[q];
    if (ctx->orbit_spw > 0) {
      g.spw = ctx->orbit_spw;
    } else {
      int target = std::max(1, 2 * ctx->sm_count);
      int want = (nsg + target - 1) / target, spw = 1;
      while (spw < want && spw < 32) spw *= 2;
      g.spw = spw;
    }
    int npk = 0;
    for (int i = 0; i < N - 1; i++)
      for (int j = i + 1; j < N; j++)
        if (!((g.kick >> pair_bit(i, j, N)) & 1)) npk++;
    g.npk = npk;
    g.R = step_record_size(N, npk, g.kick != 0);
  }
  // ---- fit the working set: longest chunk first, then the widest transit grid
  SysOff* d_off;
  long long *d_offtt, *d_offdq;
  int* d_bad;
  const size_t limit = (size_t)NBG_NOALLOC_SCRATCH_BYTES;
  int K = 0, tcap = 0;
  size_t need_min = 0;
  for (int k = std::max(1, ctx->chunk_steps); k >= 1 && !K; k = (k > 1 ? k / 2 : 0))
    for (int tc = 1024; tc >= 32 && !K; tc /= 2) {
      ScratchArena a{nullptr, 0};
      noalloc_layout(P, a, nsys, k, tc, &d_off, &d_offtt, &d_offdq, &d_bad);
      need_min = a.used;
      if (a.used <= limit) { K = k; tcap = tc; }
    }
  if (!K)
    return set_error(NBG_ENOMEM,
                     "nbg_batch_integrate_transits_noalloc: these %d systems need %zu bytes of device scratch even "
                     "at one step per chunk; the fixed scratch holds %zu bytes (NBG_NOALLOC_SCRATCH_BYTES)",
                     nsys, need_min, limit);
  unsigned char* base = nullptr;
  {
    cudaError_t e = nbg_noalloc_scratch(ctx->device, &base);
    if (e != cudaSuccess)
      return set_error(NBG_ECUDA, "cudaGetSymbolAddress of the no-allocation scratch on device %d: %s", ctx->device,
                       cudaGetErrorString(e));
  }
  {
    ScratchArena a{base, 0};
    noalloc_layout(P, a, nsys, K, tcap, &d_off, &d_offtt, &d_offdq, &d_bad);
  }
  NBG_CUDA(cudaMemcpyAsync(d_off, P.off, sizeof(SysOff) * nsys, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemcpyAsync(d_offtt, P.offtt, sizeof(long long) * nsys, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemcpyAsync(d_offdq, P.offdq, sizeof(long long) * nsys, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemsetAsync(d_bad, 0, sizeof(int), st));
  // ---- per-group state: scalars through one stack staging area per group
  for (int q = 0; q < P.ngroups; q++) {
    GroupArgs& g = P.g[q];
    const int N = g.N, S = g.S;
    g.tt = d_tt; g.off_tt = d_offtt; g.dtdq0 = d_dq0; g.off_dq = d_offdq;
    int *sidx = P.sidx, *vntt = P.vntt, *vti = P.vti;
    double *vt0 = P.vt0, *vh = P.vh, *vhI = P.vhI;
    long long* vns = P.vns;
    for (int r = 0; r < S; r++) {
      sidx[r] = -1; vntt[r] = 1; vti[r] = 0; vt0[r] = vh[r] = vhI[r] = 0.0; vns[r] = 0;
    }
    for (int r = 0; r < g.nsys; r++) {
      const int s = P.order[P.gstart[q] + r];
      sidx[r] = s; vntt[r] = desc[s].ntt; vti[r] = desc[s].ti;
      vt0[r] = P.t0[s]; vh[r] = P.hsig[s]; vhI[r] = desc[s].h; vns[r] = P.nsteps[s];
    }
    NBG_CUDA(cudaMemcpyAsync(g.sysidx, sidx, sizeof(int) * S, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(g.ntt, vntt, sizeof(int) * S, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(g.ti, vti, sizeof(int) * S, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(g.t0, vt0, sizeof(double) * S, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(g.h, vh, sizeof(double) * S, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(g.hI, vhI, sizeof(double) * S, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(g.nsteps, vns, sizeof(long long) * S, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaMemsetAsync(g.status, 0, sizeof(unsigned) * S, st));
    NBG_CUDA(cudaStreamSynchronize(st));  // the next group reuses the staging arrays
    const int pb = (S + 127) / 128;
    pack_state_kernel<<<pb, 128, 0, st>>>(N, S, g.sysidx, d_off, d_x, d_v, d_xe, d_ve, d_m, d_dqdt, d_count, g.x,
                                          g.v, g.xe, g.ve, g.m, g.dqdt, g.count);
    ctx->last_launches++;
    if (g.grad) {
      const long long tot = (long long)S * 49 * N * N;
      pack_jac_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(N, S, g.sysidx, d_off, d_J, d_E, g.Jint, g.Eint,
                                                                     d_bad);
      ctx->last_launches++;
    }
  }
  NBG_CUDA(cudaGetLastError());
  int bad = 0;
  NBG_CUDA(cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaStreamSynchronize(st));
  if (bad)
    return set_error(NBG_EUNSUPPORTED,
                     "jac_step mass rows must be unit rows with zero jac_error (true for every State the reference "
                     "builds and integrates)");
  for (int q = 0; q < P.ngroups; q++) {
    kSeed[P.g[q].N](P.g[q], st);
    ctx->last_launches++;
  }
  // ---- chunk loop
  long long max_steps = 0;
  for (int q = 0; q < P.ngroups; q++) max_steps = std::max(max_steps, P.gmax[q]);
  const long long nchunks = (max_steps + K - 1) / K;
  int rc;
  NBG_CUDA(cudaEventRecord(ctx->ev0, st));
  for (long long c = 0; c < nchunks; c++) {
    for (int q = 0; q < P.ngroups; q++) {
      const GroupArgs& g = P.g[q];
      if (c * K >= P.gmax[q]) continue;
      NBG_CUDA(cudaMemsetAsync(g.task_count, 0, sizeof(int), st));
      if ((rc = kOrbit[g.N](g, (int)c, st))) return rc;
      if ((rc = kTransit[g.N](g, (int)c, st))) return rc;
      ctx->last_launches += 2;
      ctx->last_orbit_launches++;
      if (g.grad) {
        if ((rc = kOps[g.N](g, (int)c, st))) return rc;
        if ((rc = kJac[g.N](g, (int)c, st))) return rc;
        ctx->last_launches += 3;
        ctx->last_jac_launches++;
      }
    }
  }
  NBG_CUDA(cudaGetLastError());
  NBG_CUDA(cudaEventRecord(ctx->ev1, st));
  // ---- outputs
  for (int q = 0; q < P.ngroups; q++) {
    const GroupArgs& g = P.g[q];
    const int pb = (g.S + 127) / 128;
    unpack_state_kernel<<<pb, 128, 0, st>>>(g.N, g.S, g.grad, g.sysidx, d_off, d_x, d_v, d_xe, d_ve, d_dqdt, d_count,
                                            g.x, g.v, g.xe, g.ve, g.dqdt, g.count);
    ctx->last_launches++;
    if (g.grad) {
      const long long tot = (long long)g.S * 42 * g.N * g.N;
      unpack_jac_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(g.N, g.S, g.sysidx, d_off, d_J, d_E, g.Jint,
                                                                       g.Eint);
      ctx->last_launches++;
    }
  }
  {
    dim3 grid(8, nsys, 1);
    dtdelements_kernel<<<grid, 256, 0, st>>>(nsys, nullptr, d_off, d_dq0, d_jinit, d_dtdel, d_count, 0);
    ctx->last_launches++;
  }
  // s.t = t0 + nsteps * h (Transits.jl:161 at the last step)
  for (int s = 0; s < nsys; s++)
    P.tout[s] = P.nsteps[s] > 0 ? P.t0[s] + (double)P.nsteps[s] * P.hsig[s] : P.t0[s];
  NBG_CUDA(cudaMemcpyAsync(d_t, P.tout, sizeof(double) * nsys, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaStreamSynchronize(st));
  NBG_CUDA(cudaGetLastError());
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  ctx->last_total_ms = ms;
  if (status_host) {
    std::fill(status_host, status_host + nsys, 0u);
    for (int q = 0; q < P.ngroups; q++) {
      const GroupArgs& g = P.g[q];
      unsigned* sv = P.sv;
      NBG_CUDA(cudaMemcpy(sv, g.status, sizeof(unsigned) * g.S, cudaMemcpyDeviceToHost));
      for (int r = 0; r < g.nsys; r++) status_host[P.order[P.gstart[q] + r]] = sv[r];
    }
  }
  return NBG_OK;
}

}  // namespace

// FP64 FMA throughput probe: CHAINS independent FMA chains per thread, full
// warps, several blocks per SM.  Every index stays inside the grid-sized
// output buffer.
constexpr int PEAK_CHAINS = 8;
__global__ void fp64_peak_kernel(double* out, int iters) {
  double a[PEAK_CHAINS];
  const double b = 1.0000001 + 1e-9 * threadIdx.x, c = 1e-7;
#pragma unroll
  for (int k = 0; k < PEAK_CHAINS; k++) a[k] = 1.0 + k * 1e-3;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < PEAK_CHAINS; k++) a[k] = fma(a[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < PEAK_CHAINS; k++) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Single-block FP64 issue probe: `warps` warps of one block run CH
// independent DFMA chains each and time them with clock64; cyc[w] is warp
// w's cycle count.  One block, so every warp shares one SM.  out holds
// blockDim doubles, cyc one entry per warp.
template <int CH>
__global__ void fp64_issue_kernel(double* out, long long* cyc, int iters) {
  double a[CH];
  const double b = 1.0000001 + 1e-9 * threadIdx.x, c = 1e-7;
#pragma unroll
  for (int k = 0; k < CH; k++) a[k] = 1.0 + k * 1e-3;
  __syncthreads();
  const long long t0 = clock64();
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < CH; k++) a[k] = fma(a[k], b, c);
  }
  const long long t1 = clock64();
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < CH; k++) s += a[k];
  out[threadIdx.x] = s;
  if ((threadIdx.x & 31) == 0) cyc[threadIdx.x >> 5] = t1 - t0;
}

// FP64 tensor-core (DMMA) probes: mma.sync m8n8k4 with f64 operands, one
// 8x4 by 4x8 product into an 8x8 accumulator per warp instruction (256 FMAs).
// Fragments (PTX ISA, mma.m8n8k4 .f64): lane l holds A[l/4][l%4],
// B[l%4][l/4] and C[l/4][2(l%4)], C[l/4][2(l%4)+1].
__device__ __forceinline__ void dmma_8x8x4(double& c0, double& c1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(c0), "+d"(c1)
               : "d"(a), "d"(b));
}

// One product of exactly representable small operands: err[lane] = the
// difference of this lane's two accumulator entries from the exact result
// (0 when the fragment layout above holds).  One warp, 32 outputs.
__global__ void fp64_mma_check_kernel(double* err) {
  const int l = threadIdx.x & 31, g = l >> 2, t = l & 3;
  auto A = [](int r, int k) { return (r + 1) + 0.5 * k; };
  auto B = [](int k, int n) { return (k + 1) * (double)(n - 3); };
  auto C = [](int r, int n) { return (double)(r * n); };
  double c0 = C(g, 2 * t), c1 = C(g, 2 * t + 1);
  dmma_8x8x4(c0, c1, A(g, t), B(t, g));
  double e0 = C(g, 2 * t), e1 = C(g, 2 * t + 1);
  for (int k = 0; k < 4; k++) {
    e0 += A(g, k) * B(k, 2 * t);
    e1 += A(g, k) * B(k, 2 * t + 1);
  }
  err[l] = fabs(c0 - e0) + fabs(c1 - e1);
}

// Throughput: MMA_CHAINS independent accumulators per warp; with dfma != 0
// every DMMA is followed by PEAK_CHAINS independent DFMAs of the same warp,
// so the two pipes' rates add up when they are separate units and share one
// rate when they are one.  Every index stays inside the grid-sized buffer.
constexpr int MMA_CHAINS = 4;
__global__ void fp64_mma_peak_kernel(double* out, int iters, int dfma) {
  const int l = threadIdx.x & 31;
  const double a = 1.0 + 1e-3 * l, b = 1.0 - 1e-3 * l;
  double c[MMA_CHAINS][2];
#pragma unroll
  for (int k = 0; k < MMA_CHAINS; k++) c[k][0] = c[k][1] = 1e-3 * k;
  double f[PEAK_CHAINS];
#pragma unroll
  for (int k = 0; k < PEAK_CHAINS; k++) f[k] = 1.0 + k * 1e-3;
  const double fb = 1.0000001 + 1e-9 * threadIdx.x, fc = 1e-7;
  if (dfma) {
    for (int it = 0; it < iters; it++) {
#pragma unroll
      for (int k = 0; k < MMA_CHAINS; k++) dmma_8x8x4(c[k][0], c[k][1], a, b);
#pragma unroll
      for (int k = 0; k < PEAK_CHAINS; k++) f[k] = fma(f[k], fb, fc);
    }
  } else {
    for (int it = 0; it < iters; it++) {
#pragma unroll
      for (int k = 0; k < MMA_CHAINS; k++) dmma_8x8x4(c[k][0], c[k][1], a, b);
    }
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < MMA_CHAINS; k++) s += c[k][0] + c[k][1];
#pragma unroll
  for (int k = 0; k < PEAK_CHAINS; k++) s += f[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// ===================================================================== C ABI

extern "C" {

int nbg_version(void) { return 100; }

int nbg_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return NBG_EINVAL;
  snprintf(buf, len, "%s", g_last_error.c_str());
  return NBG_OK;
}

int nbg_device_info(int device, nbg_device_info_t* out) {
  if (!out) return set_error(NBG_EINVAL, "out is NULL");
  cudaDeviceProp p;
  NBG_CUDA(cudaGetDeviceProperties(&p, device));
  memset(out, 0, sizeof(*out));
  snprintf(out->name, sizeof(out->name), "%s", p.name);
  out->sm_count = p.multiProcessorCount;
  out->cc_major = p.major;
  out->cc_minor = p.minor;
  out->total_mem = p.totalGlobalMem;
  out->min_bodies = NBG_MIN_BODIES;
  out->max_bodies = NBG_MAX_BODIES;
  return NBG_OK;
}

int nbg_create(int device, nbg_context** out) {
  if (!out) return set_error(NBG_EINVAL, "out is NULL");
  *out = nullptr;
  int ndev = 0;
  NBG_CUDA(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) return set_error(NBG_EINVAL, "device %d not in 0..%d", device, ndev - 1);
  NBG_CUDA(cudaSetDevice(device));
  nbg_context* c = new nbg_context();
  c->device = device;
  c->noalloc = new NoallocPlan();
  {
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, device) == cudaSuccess) c->sm_count = p.multiProcessorCount;
  }
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
    delete c;
    return set_error(NBG_ECUDA, "stream/event creation failed");
  }
  *out = c;
  return NBG_OK;
}

int nbg_destroy(nbg_context* ctx) {
  if (!ctx) return NBG_OK;
  cudaSetDevice(ctx->device);
  // every stream of the context is idle before its buffers are freed
  cudaStreamSynchronize(ctx->stream);
  for (cudaStream_t s2 : ctx->gstreams) cudaStreamSynchronize(s2);
  for (cudaStream_t s2 : ctx->hstreams) cudaStreamSynchronize(s2);
  for (auto& kv : ctx->pool)
    if (kv.second.p) cudaFree(kv.second.p);
  cudaEventDestroy(ctx->ev0);
  cudaEventDestroy(ctx->ev1);
  for (auto e : ctx->prof_events) cudaEventDestroy(e);
  for (auto e : ctx->sync_events) cudaEventDestroy(e);
  for (cudaStream_t s2 : ctx->gstreams) cudaStreamDestroy(s2);
  for (cudaStream_t s2 : ctx->hstreams) cudaStreamDestroy(s2);
  cudaStreamDestroy(ctx->stream);
  delete ctx->noalloc;
  delete ctx;
  return NBG_OK;
}

int nbg_set_tuning(nbg_context* ctx, int chunk_steps, int overlap) {
  if (!ctx) return set_error(NBG_EINVAL, "ctx is NULL");
  if (chunk_steps < 0 || chunk_steps > 4096) return set_error(NBG_EINVAL, "chunk_steps = %d", chunk_steps);
  if (chunk_steps) ctx->chunk_steps = chunk_steps;
  if (overlap >= 0) ctx->overlap = overlap;
  return NBG_OK;
}

int nbg_set_orbit_lanes(nbg_context* ctx, int systems_per_warp) {
  if (!ctx) return set_error(NBG_EINVAL, "ctx is NULL");
  if (systems_per_warp < 0 || systems_per_warp > 32)
    return set_error(NBG_EINVAL, "systems_per_warp = %d not in 0..32", systems_per_warp);
  ctx->orbit_spw = systems_per_warp;
  return NBG_OK;
}

int nbg_set_producer_layout(nbg_context* ctx, int warps_per_block, int smem_kb, int guard_kb) {
  if (!ctx) return set_error(NBG_EINVAL, "ctx is NULL");
  if (warps_per_block < 1 || warps_per_block > PROD_MAX_WARPS)
    return set_error(NBG_EINVAL, "warps_per_block = %d not in 1..%d", warps_per_block, PROD_MAX_WARPS);
  if (smem_kb < 0 || smem_kb > 220 || guard_kb < 0 || guard_kb > 100)
    return set_error(NBG_EINVAL, "smem_kb = %d (0..220), guard_kb = %d (0..100)", smem_kb, guard_kb);
  ctx->prod_warps = warps_per_block;
  ctx->prod_smem_kb = smem_kb;
  ctx->guard_smem_kb = guard_kb;
  return NBG_OK;
}

int nbg_set_orbit_team(nbg_context* ctx, int mode) {
  if (!ctx) return set_error(NBG_EINVAL, "ctx is NULL");
  if (mode < -1 || mode > 3) return set_error(NBG_EINVAL, "mode = %d not in -1..3", mode);
  ctx->orbit_team = mode;
  return NBG_OK;
}

int nbg_set_profiling(nbg_context* ctx, int on) {
  if (!ctx) return set_error(NBG_EINVAL, "ctx is NULL");
  if (on < 0 || on > 3) return set_error(NBG_EINVAL, "profiling level %d not in 0..3", on);
  ctx->profile = on;
  return NBG_OK;
}

int nbg_last_kernel_stats(nbg_context* ctx, int64_t* orbit_launches, int64_t* jacobian_launches) {
  if (!ctx) return set_error(NBG_EINVAL, "ctx is NULL");
  if (orbit_launches) *orbit_launches = ctx->last_orbit_launches;
  if (jacobian_launches) *jacobian_launches = ctx->last_jac_launches;
  return NBG_OK;
}

int nbg_last_timing(nbg_context* ctx, double* total_ms, double* orbit_ms, double* transit_ms, double* jacobian_ms) {
  if (!ctx) return set_error(NBG_EINVAL, "ctx is NULL");
  if (total_ms) *total_ms = ctx->last_total_ms;
  if (orbit_ms) *orbit_ms = ctx->last_orbit_ms + ctx->last_ops_ms;
  if (transit_ms) *transit_ms = ctx->last_transit_ms;
  if (jacobian_ms) *jacobian_ms = ctx->last_jac_ms;
  return NBG_OK;
}

int64_t nbg_last_launch_count(nbg_context* ctx) { return ctx ? ctx->last_launches : -1; }

int nbg_last_host_time(nbg_context* ctx, double* enqueue_ms) {
  if (!ctx || !enqueue_ms) return set_error(NBG_EINVAL, "NULL argument");
  *enqueue_ms = ctx->last_host_ms;
  return NBG_OK;
}

int nbg_fp64_peak(nbg_context* ctx, double* tflops) {
  if (!ctx || !tflops) return set_error(NBG_EINVAL, "NULL argument");
  NBG_CUDA(cudaSetDevice(ctx->device));
  cudaDeviceProp p;
  NBG_CUDA(cudaGetDeviceProperties(&p, ctx->device));
  const int threads = 256, blocks = p.multiProcessorCount * 4, iters = 20000;
  double* out;
  int rc;
  if ((rc = ctx->get("peak", (size_t)threads * blocks, &out))) return rc;
  fp64_peak_kernel<<<blocks, threads, 0, ctx->stream>>>(out, 100);
  NBG_CUDA(cudaGetLastError());
  float best = 1e30f;
  for (int rep = 0; rep < 3; rep++) {
    NBG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    fp64_peak_kernel<<<blocks, threads, 0, ctx->stream>>>(out, iters);
    NBG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    NBG_CUDA(cudaEventSynchronize(ctx->ev1));
    float ms = 0;
    NBG_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    best = std::min(best, ms);
  }
  *tflops = 2.0 * (double)blocks * threads * iters * PEAK_CHAINS / (best * 1e-3) / 1e12;
  return NBG_OK;
}

int nbg_fp64_warp_issue(nbg_context* ctx, int warps, int chains, double* cycles_per_dfma) {
  if (!ctx || !cycles_per_dfma) return set_error(NBG_EINVAL, "NULL argument");
  if (warps < 1 || warps > 32) return set_error(NBG_EINVAL, "warps = %d not in 1..32", warps);
  if (chains != 1 && chains != 2 && chains != 4 && chains != 8)
    return set_error(NBG_EINVAL, "chains = %d not 1, 2, 4 or 8", chains);
  NBG_CUDA(cudaSetDevice(ctx->device));
  double* out;
  long long* cyc;
  int rc;
  if ((rc = ctx->get("issue_out", (size_t)32 * warps, &out))) return rc;
  if ((rc = ctx->get("issue_cyc", (size_t)warps, &cyc))) return rc;
  const int iters = 2000;
  for (int pass = 0; pass < 2; pass++) {  // the first pass warms the instruction cache
    const int it = pass ? iters : 10;
    switch (chains) {
      case 1: fp64_issue_kernel<1><<<1, 32 * warps, 0, ctx->stream>>>(out, cyc, it); break;
      case 2: fp64_issue_kernel<2><<<1, 32 * warps, 0, ctx->stream>>>(out, cyc, it); break;
      case 4: fp64_issue_kernel<4><<<1, 32 * warps, 0, ctx->stream>>>(out, cyc, it); break;
      default: fp64_issue_kernel<8><<<1, 32 * warps, 0, ctx->stream>>>(out, cyc, it); break;
    }
    NBG_CUDA(cudaGetLastError());
  }
  long long h[32];
  NBG_CUDA(cudaMemcpyAsync(h, cyc, sizeof(long long) * warps, cudaMemcpyDeviceToHost, ctx->stream));
  NBG_CUDA(cudaStreamSynchronize(ctx->stream));
  long long mx = 0;
  for (int w = 0; w < warps; w++) mx = std::max(mx, h[w]);
  *cycles_per_dfma = (double)mx / ((double)iters * chains);
  return NBG_OK;
}

int nbg_fp64_mma_peak(nbg_context* ctx, int with_dfma, double* tflops, double* dfma_share) {
  if (!ctx || !tflops) return set_error(NBG_EINVAL, "NULL argument");
  NBG_CUDA(cudaSetDevice(ctx->device));
  cudaDeviceProp p;
  NBG_CUDA(cudaGetDeviceProperties(&p, ctx->device));
  const int threads = 256, blocks = p.multiProcessorCount * 4, iters = 4000;
  double* out;
  int rc;
  if ((rc = ctx->get("peak", (size_t)threads * blocks, &out))) return rc;
  fp64_mma_check_kernel<<<1, 32, 0, ctx->stream>>>(out);
  NBG_CUDA(cudaGetLastError());
  double err[32];
  NBG_CUDA(cudaMemcpyAsync(err, out, sizeof(err), cudaMemcpyDeviceToHost, ctx->stream));
  NBG_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int l = 0; l < 32; l++)
    if (err[l] != 0.0) return set_error(NBG_EUNSUPPORTED, "DMMA fragment check: lane %d off by %g", l, err[l]);
  fp64_mma_peak_kernel<<<blocks, threads, 0, ctx->stream>>>(out, 20, with_dfma);
  NBG_CUDA(cudaGetLastError());
  float best = 1e30f;
  for (int rep = 0; rep < 3; rep++) {
    NBG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    fp64_mma_peak_kernel<<<blocks, threads, 0, ctx->stream>>>(out, iters, with_dfma);
    NBG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    NBG_CUDA(cudaEventSynchronize(ctx->ev1));
    float ms = 0;
    NBG_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    best = std::min(best, ms);
  }
  const double warps = (double)blocks * threads / 32.0;
  const double mma_flops = warps * iters * MMA_CHAINS * 512.0;
  const double fma_flops = with_dfma ? 2.0 * (double)blocks * threads * iters * PEAK_CHAINS : 0.0;
  *tflops = (mma_flops + fma_flops) / (best * 1e-3) / 1e12;
  if (dfma_share) *dfma_share = fma_flops / (mma_flops + fma_flops);
  return NBG_OK;
}

static int batch_host_device(nbg_context* ctx, int nsys, const nbg_system_desc* desc, double* t, double* x,
                             double* v, const double* m, double* xerror, double* verror, double* jac_step,
                             double* jac_error, double* dqdt, const uint8_t* pair, const double* jac_init, double* tt,
                             double* dtdq0, double* dtdelements, int64_t* count, uint32_t* status, bool copy_outputs_in,
                             int tbv = 0) {
  const int nr = tbv ? 3 : 1;
  if (!ctx) return set_error(NBG_EINVAL, "ctx is NULL");
  if (nsys <= 0 || !desc) return set_error(NBG_EINVAL, "nsys = %d", nsys);
  NBG_CUDA(cudaSetDevice(ctx->device));
  long long ax = 0, am = 0, aJ = 0, adq = 0, ap = 0, att = 0, adq0 = 0;
  for (int s = 0; s < nsys; s++) {
    int n = desc[s].n, M = 7 * n;
    if (n < NBG_MIN_BODIES || n > NBG_MAX_BODIES)
      return set_error(NBG_EUNSUPPORTED, "system %d: n = %d outside %d..%d", s, n, NBG_MIN_BODIES, NBG_MAX_BODIES);
    if (desc[s].ntt < 1) return set_error(NBG_EINVAL, "system %d: ntt = %d", s, desc[s].ntt);
    ax += 3 * n; am += n; aJ += (long long)M * M; adq += M; ap += (long long)n * n;
    att += (long long)nr * n * desc[s].ntt; adq0 += (long long)nr * n * desc[s].ntt * 7 * n;
  }
  if (!copy_outputs_in)
    for (long long q = 0; q < am; q++)
      if (count[q] != 0) return set_error(NBG_EINVAL, "batched calls need fresh TransitTiming outputs (count == 0)");
  cudaStream_t st = ctx->stream;
  double *d_t, *d_x, *d_v, *d_m, *d_xe, *d_ve, *d_J, *d_E, *d_dq, *d_ji, *d_tt, *d_dq0, *d_del;
  long long* d_cnt;
  int rc;
#define GETB(ptr, nm, cnt) if ((rc = ctx->get(nm, (size_t)(cnt), &ptr))) return rc
  GETB(d_t, "u_t", nsys); GETB(d_x, "u_x", ax); GETB(d_v, "u_v", ax); GETB(d_m, "u_m", am);
  GETB(d_xe, "u_xe", ax); GETB(d_ve, "u_ve", ax); GETB(d_J, "u_J", aJ); GETB(d_E, "u_E", aJ);
  GETB(d_dq, "u_dq", adq); GETB(d_ji, "u_ji", aJ); GETB(d_tt, "u_tt", att); GETB(d_dq0, "u_dq0", adq0);
  GETB(d_del, "u_del", adq0); GETB(d_cnt, "u_cnt", am);
#undef GETB
  NBG_CUDA(cudaMemcpyAsync(d_t, t, sizeof(double) * nsys, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemcpyAsync(d_x, x, sizeof(double) * ax, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemcpyAsync(d_v, v, sizeof(double) * ax, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemcpyAsync(d_m, m, sizeof(double) * am, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemcpyAsync(d_xe, xerror, sizeof(double) * ax, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemcpyAsync(d_ve, verror, sizeof(double) * ax, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemcpyAsync(d_J, jac_step, sizeof(double) * aJ, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemcpyAsync(d_E, jac_error, sizeof(double) * aJ, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemcpyAsync(d_dq, dqdt, sizeof(double) * adq, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemcpyAsync(d_ji, jac_init, sizeof(double) * aJ, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemcpyAsync(d_cnt, count, sizeof(long long) * am, cudaMemcpyHostToDevice, st));
  if (copy_outputs_in) {
    NBG_CUDA(cudaMemcpyAsync(d_tt, tt, sizeof(double) * att, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(d_dq0, dtdq0, sizeof(double) * adq0, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(d_del, dtdelements, sizeof(double) * adq0, cudaMemcpyHostToDevice, st));
  } else {
    NBG_CUDA(cudaMemsetAsync(d_tt, 0, sizeof(double) * att, st));
    NBG_CUDA(cudaMemsetAsync(d_dq0, 0, sizeof(double) * adq0, st));
    NBG_CUDA(cudaMemsetAsync(d_del, 0, sizeof(double) * adq0, st));
  }
  rc = run_batch(ctx, nsys, desc, t, pair, d_t, d_x, d_v, d_m, d_xe, d_ve, d_J, d_E, d_dq, d_ji, d_tt, d_dq0, d_del,
                 d_cnt, status, nullptr, tbv);
  if (rc) return rc;
  NBG_CUDA(cudaMemcpyAsync(t, d_t, sizeof(double) * nsys, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(x, d_x, sizeof(double) * ax, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(v, d_v, sizeof(double) * ax, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(xerror, d_xe, sizeof(double) * ax, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(verror, d_ve, sizeof(double) * ax, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(jac_step, d_J, sizeof(double) * aJ, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(jac_error, d_E, sizeof(double) * aJ, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(dqdt, d_dq, sizeof(double) * adq, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(count, d_cnt, sizeof(long long) * am, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(tt, d_tt, sizeof(double) * att, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(dtdq0, d_dq0, sizeof(double) * adq0, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(dtdelements, d_del, sizeof(double) * adq0, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaStreamSynchronize(st));
  return NBG_OK;
}

// Plain integration of nsys systems (host arrays, the packed layout of the
// batched calls; no transit arrays).
// NBG_ENONFINITE (after every output has been written) when a system ended
// with a non-finite x, v or jac_step: the entry points without a status array
// report it this way; the reference lets the values propagate silently.
static int nonfinite_error(int nsys, const uint32_t* status) {
  for (int s = 0; s < nsys; s++)
    if (status[s] & NBG_STATUS_NONFINITE)
      return set_error(NBG_ENONFINITE, "system %d: x, v or jac_step is not finite at the end of the integration "
                                       "(outputs written as computed)", s);
  return NBG_OK;
}

static int plain_host(nbg_context* ctx, int nsys, const nbg_system_desc* desc, const PlainSpec* spec, double* t,
                      double* x, double* v, const double* m, double* xerror, double* verror, double* jac_step,
                      double* jac_error, double* dqdt, const uint8_t* pair, const TrajOut* traj = nullptr) {
  if (!ctx) return set_error(NBG_EINVAL, "ctx is NULL");
  if (nsys <= 0 || !desc) return set_error(NBG_EINVAL, "nsys = %d", nsys);
  if (!t || !x || !v || !m || !xerror || !verror || !jac_step || !jac_error || !dqdt || !pair)
    return set_error(NBG_EINVAL, "NULL array argument");
  NBG_CUDA(cudaSetDevice(ctx->device));
  long long ax = 0, am = 0, aJ = 0, adq = 0;
  for (int s = 0; s < nsys; s++) {
    const int n = desc[s].n, M = 7 * n;
    if (n < NBG_MIN_BODIES || n > NBG_MAX_BODIES)
      return set_error(NBG_EUNSUPPORTED, "system %d: n = %d outside %d..%d", s, n, NBG_MIN_BODIES, NBG_MAX_BODIES);
    ax += 3 * n; am += n; aJ += (long long)M * M; adq += M;
  }
  cudaStream_t st = ctx->stream;
  double *d_t, *d_x, *d_v, *d_m, *d_xe, *d_ve, *d_J, *d_E, *d_dq;
  long long* d_cnt;
  int rc;
#define GETB(ptr, nm, cnt) if ((rc = ctx->get(nm, (size_t)(cnt), &ptr))) return rc
  GETB(d_t, "p_t", nsys); GETB(d_x, "p_x", ax); GETB(d_v, "p_v", ax); GETB(d_m, "p_m", am);
  GETB(d_xe, "p_xe", ax); GETB(d_ve, "p_ve", ax); GETB(d_J, "p_J", aJ); GETB(d_E, "p_E", aJ);
  GETB(d_dq, "p_dq", adq); GETB(d_cnt, "p_cnt", am);
#undef GETB
  NBG_CUDA(cudaMemcpyAsync(d_x, x, sizeof(double) * ax, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemcpyAsync(d_v, v, sizeof(double) * ax, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemcpyAsync(d_m, m, sizeof(double) * am, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemcpyAsync(d_xe, xerror, sizeof(double) * ax, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemcpyAsync(d_ve, verror, sizeof(double) * ax, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemcpyAsync(d_J, jac_step, sizeof(double) * aJ, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemcpyAsync(d_E, jac_error, sizeof(double) * aJ, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemcpyAsync(d_dq, dqdt, sizeof(double) * adq, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemsetAsync(d_cnt, 0, sizeof(long long) * am, st));
  std::vector<uint32_t> stv(nsys, 0u);
  rc = run_batch(ctx, nsys, desc, t, pair, d_t, d_x, d_v, d_m, d_xe, d_ve, d_J, d_E, d_dq, nullptr, nullptr, nullptr,
                 nullptr, d_cnt, stv.data(), spec, 0, traj);
  if (rc) return rc;
  NBG_CUDA(cudaMemcpyAsync(t, d_t, sizeof(double) * nsys, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(x, d_x, sizeof(double) * ax, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(v, d_v, sizeof(double) * ax, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(xerror, d_xe, sizeof(double) * ax, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(verror, d_ve, sizeof(double) * ax, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(jac_step, d_J, sizeof(double) * aJ, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(jac_error, d_E, sizeof(double) * aJ, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(dqdt, d_dq, sizeof(double) * adq, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaStreamSynchronize(st));
  return nonfinite_error(nsys, stv.data());
}

// intr(s, time) (Integrator.jl:159-197): nsteps = |round((time - t0)/h)|
// steps of h * check_step(t0, time), then one step of time - tmax when
// tmax = t0 + h nsteps falls short of time; s.t = time.
static PlainSpec spec_to_time(double t0, double h, double time) {
  PlainSpec p;
  long long n = (long long)std::nearbyint((time - t0) / h);
  if (n < 0) n = -n;
  const double hs = h * check_step(t0, time);
  const double tmax = t0 + (hs * (double)n);
  p.nsteps = n;
  p.h = hs;
  p.hlast = hs;
  if (tmax != time) {
    p.nsteps = n + 1;
    p.hlast = time - tmax;
  }
  p.tout = time;
  return p;
}

int nbg_integrate(nbg_context* ctx, int n, double h, double time, int grad, double* t, double* x, double* v,
                  const double* m, double* xerror, double* verror, double* jac_step, double* jac_error, double* dqdt,
                  const uint8_t* pair) {
  if (!t) return set_error(NBG_EINVAL, "NULL array argument");
  if (!(h != 0.0) || !std::isfinite(h) || !std::isfinite(time) || !std::isfinite(t[0]))
    return set_error(NBG_EINVAL, "h = %g, time = %g, t = %g", h, time, t[0]);
  nbg_system_desc d;
  d.n = n; d.ti = 0; d.grad = grad ? 1 : 0; d.ntt = 1; d.h = h; d.tmax = time;
  const PlainSpec p = spec_to_time(t[0], h, time);
  return plain_host(ctx, 1, &d, &p, t, x, v, m, xerror, verror, jac_step, jac_error, dqdt, pair);
}

int nbg_integrate_steps(nbg_context* ctx, int n, double h, int64_t nsteps, int grad, double* t, double* x,
                        double* v, const double* m, double* xerror, double* verror, double* jac_step,
                        double* jac_error, double* dqdt, const uint8_t* pair) {
  if (!t) return set_error(NBG_EINVAL, "NULL array argument");
  if (!(h != 0.0) || !std::isfinite(h) || !std::isfinite(t[0])) return set_error(NBG_EINVAL, "h = %g", h);
  if (nsteps < -(1LL << 40) || nsteps > (1LL << 40)) return set_error(NBG_EINVAL, "nsteps = %lld", (long long)nsteps);
  // intr(s, N) (Integrator.jl:210-233): a negative N steps backward; s.t
  // advances by a compensated sum of the signed step
  PlainSpec p;
  const double hs = nsteps < 0 ? -h : h;
  p.nsteps = nsteps < 0 ? -nsteps : nsteps;
  p.h = hs;
  p.hlast = hs;
  double ts = t[0], e = 0.0;
  for (long long q = 0; q < p.nsteps; q++) {
    e = e + hs;
    const double tn = ts + e;
    e = (ts - tn) + e;
    ts = tn;
  }
  p.tout = ts;
  nbg_system_desc d;
  d.n = n; d.ti = 0; d.grad = grad ? 1 : 0; d.ntt = 1; d.h = h; d.tmax = hs * (double)p.nsteps;
  return plain_host(ctx, 1, &d, &p, t, x, v, m, xerror, verror, jac_step, jac_error, dqdt, pair);
}

int nbg_integrate_cartesian(nbg_context* ctx, int n, double h, double tmax, int64_t nstep, double* t, double* x,
                            double* v, const double* m, double* xerror, double* verror, double* jac_step,
                            double* jac_error, double* dqdt, const uint8_t* pair, double* out_t, double* out_x,
                            double* out_v, double* out_jac) {
  if (!t || !out_t || !out_x || !out_v) return set_error(NBG_EINVAL, "NULL array argument");
  if (!(h != 0.0) || !std::isfinite(h) || !std::isfinite(tmax) || !std::isfinite(t[0]))
    return set_error(NBG_EINVAL, "h = %g, tmax = %g", h, tmax);
  if (nstep < 0 || nstep > (1LL << 32)) return set_error(NBG_EINVAL, "nstep = %lld", (long long)nstep);
  // (intr::Integrator)(s, o::CartesianOutput) (Outputs.jl:26-49): nstep grad
  // steps of h * check_step(t0, intr.tmax); the state before step i is saved,
  // with s.t = t0 + h (i - 1); afterwards s.t = t0 + h nstep
  const double t0 = t[0];
  PlainSpec p;
  p.h = h * check_step(t0, tmax);
  p.hlast = p.h;
  p.nsteps = nstep;
  p.tout = nstep > 0 ? t0 + (p.h * (double)nstep) : t0;
  for (long long i = 0; i < nstep; i++) out_t[i] = (i == 0) ? t0 : t0 + (p.h * (double)i);
  nbg_system_desc d;
  d.n = n; d.ti = 0; d.grad = 1; d.ntt = 1; d.h = h; d.tmax = tmax;
  TrajOut o{out_t, out_x, out_v, out_jac};
  return plain_host(ctx, 1, &d, &p, t, x, v, m, xerror, verror, jac_step, jac_error, dqdt, pair, &o);
}

int nbg_batch_integrate(nbg_context* ctx, int nsys, const nbg_system_desc* desc, double* t, double* x, double* v,
                        const double* m, double* xerror, double* verror, double* jac_step, double* jac_error,
                        double* dqdt, const uint8_t* pair) {
  if (nsys <= 0 || !desc || !t) return set_error(NBG_EINVAL, "nsys = %d", nsys);
  std::vector<nbg_system_desc> d(desc, desc + nsys);
  std::vector<PlainSpec> p(nsys);
  for (int s = 0; s < nsys; s++) {
    if (!(d[s].h != 0.0) || !std::isfinite(d[s].h) || !std::isfinite(d[s].tmax) || !std::isfinite(t[s]))
      return set_error(NBG_EINVAL, "system %d: h = %g, time = %g", s, d[s].h, d[s].tmax);
    d[s].ti = 0;
    d[s].ntt = 1;
    p[s] = spec_to_time(t[s], d[s].h, d[s].tmax);
  }
  return plain_host(ctx, nsys, d.data(), p.data(), t, x, v, m, xerror, verror, jac_step, jac_error, dqdt, pair);
}

int nbg_integrate_transits(nbg_context* ctx, int n, int ti, double h, double tmax, int grad, double* t, double* x,
                           double* v, const double* m, double* xerror, double* verror, double* jac_step,
                           double* jac_error, double* dqdt, const uint8_t* pair, const double* jac_init, int64_t ntt,
                           double* tt, double* dtdq0, double* dtdelements, int64_t* count) {
  if (!t || !x || !v || !m || !xerror || !verror || !jac_step || !jac_error || !dqdt || !pair || !jac_init || !tt ||
      !dtdq0 || !dtdelements || !count)
    return set_error(NBG_EINVAL, "NULL array argument");
  if (ntt < 1 || ntt > (1LL << 30)) return set_error(NBG_EINVAL, "ntt = %lld", (long long)ntt);
  nbg_system_desc d;
  d.n = n; d.ti = ti; d.grad = grad ? 1 : 0; d.ntt = (int32_t)ntt; d.h = h; d.tmax = tmax;
  if (n < NBG_MIN_BODIES || n > NBG_MAX_BODIES)
    return set_error(NBG_EUNSUPPORTED, "n = %d outside %d..%d", n, NBG_MIN_BODIES, NBG_MAX_BODIES);
  if (ti < 0 || ti >= n) return set_error(NBG_EINVAL, "ti = %d not in 0..%d", ti, n - 1);
  uint32_t st1 = 0;
  const int rc = batch_host_device(ctx, 1, &d, t, x, v, m, xerror, verror, jac_step, jac_error, dqdt, pair, jac_init,
                                   tt, dtdq0, dtdelements, count, &st1, true);
  return rc ? rc : nonfinite_error(1, &st1);
}

static void* ctx_scratch(void* c, const char* name, size_t bytes) {
  unsigned char* p = nullptr;
  if (((nbg_context*)c)->get(name, bytes, &p)) return nullptr;
  return p;
}

int nbg_batch_init_nbody_device(nbg_context* ctx, int nsys, const int32_t* n, const double* t0,
                                const double* elements, const double* H, double* x, double* v, double* jac_init) {
  if (!ctx) return set_error(NBG_EINVAL, "ctx is NULL");
  if (nsys <= 0 || !n || !t0 || !elements || !x || !v || !jac_init) return set_error(NBG_EINVAL, "NULL argument");
  NBG_CUDA(cudaSetDevice(ctx->device));
  return init_nbody_device(ctx->device, ctx->stream, nsys, n, t0, elements, H, x, v, jac_init, ctx_scratch, ctx);
}

int nbg_batch_init_nbody(nbg_context* ctx, int nsys, const int32_t* n, const double* t0, const double* elements,
                         const double* H, double* x, double* v, double* jac_init) {
  if (!ctx) return set_error(NBG_EINVAL, "ctx is NULL");
  if (nsys <= 0 || !n || !t0 || !elements || !x || !v || !jac_init) return set_error(NBG_EINVAL, "NULL argument");
  NBG_CUDA(cudaSetDevice(ctx->device));
  long long ael = 0, aH = 0, ax = 0, aJ = 0;
  for (int s = 0; s < nsys; s++) {
    if (n[s] < NBG_MIN_BODIES || n[s] > NBG_MAX_BODIES)
      return set_error(NBG_EUNSUPPORTED, "system %d: n = %d outside %d..%d", s, n[s], NBG_MIN_BODIES, NBG_MAX_BODIES);
    ael += 7LL * n[s]; aH += (long long)n[s] * n[s]; ax += 3LL * n[s]; aJ += 49LL * n[s] * n[s];
  }
  cudaStream_t st = ctx->stream;
  double *d_el, *d_H = nullptr, *d_x, *d_v, *d_J;
  int rc;
  if ((rc = ctx->get("i_el", (size_t)ael, &d_el)) || (rc = ctx->get("i_x", (size_t)ax, &d_x)) ||
      (rc = ctx->get("i_v", (size_t)ax, &d_v)) || (rc = ctx->get("i_J", (size_t)aJ, &d_J)))
    return rc;
  if (H && (rc = ctx->get("i_H", (size_t)aH, &d_H))) return rc;
  NBG_CUDA(cudaMemcpyAsync(d_el, elements, sizeof(double) * ael, cudaMemcpyHostToDevice, st));
  if (H) NBG_CUDA(cudaMemcpyAsync(d_H, H, sizeof(double) * aH, cudaMemcpyHostToDevice, st));
  if ((rc = init_nbody_device(ctx->device, st, nsys, n, t0, d_el, d_H, d_x, d_v, d_J, ctx_scratch, ctx))) return rc;
  NBG_CUDA(cudaMemcpyAsync(x, d_x, sizeof(double) * ax, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(v, d_v, sizeof(double) * ax, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaMemcpyAsync(jac_init, d_J, sizeof(double) * aJ, cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaStreamSynchronize(st));
  return NBG_OK;
}

int nbg_integrate_transit_parameters(nbg_context* ctx, int n, int ti, double h, double tmax, int grad, double* t,
                                     double* x, double* v, const double* m, double* xerror, double* verror,
                                     double* jac_step, double* jac_error, double* dqdt, const uint8_t* pair,
                                     const double* jac_init, int64_t ntt, double* ttbv, double* dtbvdq0,
                                     double* dtbvdelements, int64_t* count) {
  if (!t || !x || !v || !m || !xerror || !verror || !jac_step || !jac_error || !dqdt || !pair || !jac_init ||
      !ttbv || !dtbvdq0 || !dtbvdelements || !count)
    return set_error(NBG_EINVAL, "NULL array argument");
  if (ntt < 1 || ntt > (1LL << 30)) return set_error(NBG_EINVAL, "ntt = %lld", (long long)ntt);
  if (n < NBG_MIN_BODIES || n > NBG_MAX_BODIES)
    return set_error(NBG_EUNSUPPORTED, "n = %d outside %d..%d", n, NBG_MIN_BODIES, NBG_MAX_BODIES);
  if (ti < 0 || ti >= n) return set_error(NBG_EINVAL, "ti = %d not in 0..%d", ti, n - 1);
  nbg_system_desc d;
  d.n = n; d.ti = ti; d.grad = grad ? 1 : 0; d.ntt = (int32_t)ntt; d.h = h; d.tmax = tmax;
  uint32_t st1 = 0;
  const int rc = batch_host_device(ctx, 1, &d, t, x, v, m, xerror, verror, jac_step, jac_error, dqdt, pair, jac_init,
                                   ttbv, dtbvdq0, dtbvdelements, count, &st1, true, 1);
  return rc ? rc : nonfinite_error(1, &st1);
}

int nbg_batch_integrate_transit_parameters(nbg_context* ctx, int nsys, const nbg_system_desc* desc, double* t,
                                           double* x, double* v, const double* m, double* xerror, double* verror,
                                           double* jac_step, double* jac_error, double* dqdt, const uint8_t* pair,
                                           const double* jac_init, double* ttbv, double* dtbvdq0,
                                           double* dtbvdelements, int64_t* count, uint32_t* status) {
  return batch_host_device(ctx, nsys, desc, t, x, v, m, xerror, verror, jac_step, jac_error, dqdt, pair, jac_init,
                           ttbv, dtbvdq0, dtbvdelements, count, status, false, 1);
}

int nbg_batch_integrate_transits(nbg_context* ctx, int nsys, const nbg_system_desc* desc, double* t, double* x,
                                 double* v, const double* m, double* xerror, double* verror, double* jac_step,
                                 double* jac_error, double* dqdt, const uint8_t* pair, const double* jac_init,
                                 double* tt, double* dtdq0, double* dtdelements, int64_t* count, uint32_t* status) {
  return batch_host_device(ctx, nsys, desc, t, x, v, m, xerror, verror, jac_step, jac_error, dqdt, pair, jac_init, tt,
                           dtdq0, dtdelements, count, status, false);
}

int nbg_batch_integrate_transits_device(nbg_context* ctx, int nsys, const nbg_system_desc* desc, double* t,
                                        double* x, double* v, const double* m, double* xerror, double* verror,
                                        double* jac_step, double* jac_error, double* dqdt, const uint8_t* pair,
                                        const double* jac_init, double* tt, double* dtdq0, double* dtdelements,
                                        int64_t* count, uint32_t* status) {
  if (!ctx) return set_error(NBG_EINVAL, "ctx is NULL");
  if (nsys <= 0 || !desc) return set_error(NBG_EINVAL, "nsys = %d", nsys);
  NBG_CUDA(cudaSetDevice(ctx->device));
  // the orchestration needs start times and pair flags on the host
  long long ap = 0;
  for (int s = 0; s < nsys; s++) {
    if (desc[s].n < NBG_MIN_BODIES || desc[s].n > NBG_MAX_BODIES)
      return set_error(NBG_EUNSUPPORTED, "system %d: n = %d", s, desc[s].n);
    ap += (long long)desc[s].n * desc[s].n;
  }
  std::vector<double> th(nsys);
  std::vector<uint8_t> ph(ap);
  NBG_CUDA(cudaMemcpy(th.data(), t, sizeof(double) * nsys, cudaMemcpyDeviceToHost));
  NBG_CUDA(cudaMemcpy(ph.data(), pair, ap, cudaMemcpyDeviceToHost));
  return run_batch(ctx, nsys, desc, th.data(), ph.data(), t, x, v, m, xerror, verror, jac_step, jac_error, dqdt,
                   jac_init, tt, dtdq0, dtdelements, (long long*)count, status);
}

int nbg_autotune_device(nbg_context* ctx, int nsys, const nbg_system_desc* desc, double* t, double* x, double* v,
                        const double* m, double* xerror, double* verror, double* jac_step, double* jac_error,
                        double* dqdt, const uint8_t* pair, const double* jac_init, int trial_steps,
                        nbg_tuning_result* report, int report_len, int* nreport) {
  if (!ctx) return set_error(NBG_EINVAL, "ctx is NULL");
  if (nsys <= 0 || !desc) return set_error(NBG_EINVAL, "nsys = %d", nsys);
  if (trial_steps < 8 || trial_steps > 100000) return set_error(NBG_EINVAL, "trial_steps = %d", trial_steps);
  NBG_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  // Trials per candidate, on copies: every system's first min(nsteps, T)
  // steps for T = trial_steps and 2 trial_steps give the loop's fill and
  // drain and its time per step with the whole batch active (close to affine
  // in T).  A batch of uneven length is not all active to its end: once its
  // short systems have finished, a step costs what its longest systems'
  // chains cost.  For such a batch two more trials run the longest systems
  // alone (T and 2T steps) for the chain's time per step, and the loop time
  // is modelled step by step as the larger of the whole-batch cost scaled by
  // the work still active (systems weighted by their Jacobian work per step)
  // and the chain cost.
  std::vector<nbg_system_desc> td1(desc, desc + nsys), td2(desc, desc + nsys);
  long long ax = 0, am = 0, aJ = 0, adq = 0, ap = 0, att = 0, adq0 = 0, steps = 0, longest = 0;
  bool any_team = false;
  for (int s = 0; s < nsys; s++) {
    const int n = desc[s].n, M = 7 * n;
    if (n < NBG_MIN_BODIES || n > NBG_MAX_BODIES) return set_error(NBG_EUNSUPPORTED, "system %d: n = %d", s, n);
    if (!(desc[s].h != 0.0) || !std::isfinite(desc[s].h) || !std::isfinite(desc[s].tmax) || desc[s].ntt < 1)
      return set_error(NBG_EINVAL, "system %d: h = %g, tmax = %g, ntt = %d", s, desc[s].h, desc[s].tmax, desc[s].ntt);
    const long long full = steps_of(desc[s].h, desc[s].tmax);
    const double sg = desc[s].tmax < 0 ? -1.0 : 1.0;
    td1[s].tmax = sg * std::fabs(desc[s].h) * (double)std::min<long long>(full, trial_steps);
    td2[s].tmax = sg * std::fabs(desc[s].h) * (double)std::min<long long>(full, 2LL * trial_steps);
    steps += full;
    longest = std::max(longest, full);
    any_team = any_team || n >= 4;
    ax += 3 * n; am += n; aJ += (long long)M * M; adq += M; ap += (long long)n * n;
    att += (long long)n * desc[s].ntt; adq0 += (long long)n * desc[s].ntt * 7 * n;
  }
  if (steps == 0) return set_error(NBG_EINVAL, "the batch has no steps to time");
  // the step distribution: (steps, weight) sorted by steps, and the chain set
  std::vector<std::pair<long long, double>> dist(nsys);
  long long shortest = longest;
  double wtot = 0.0;
  for (int s = 0; s < nsys; s++) {
    const int n = desc[s].n, P = n * (n - 1) / 2;
    const double w = 7.0 * n * (264.0 * P + 18.0 * n * n + 87.0 * n);  // consumer flops per system-step
    dist[s] = {steps_of(desc[s].h, desc[s].tmax), w};
    shortest = std::min(shortest, dist[s].first);
    wtot += w;
  }
  std::sort(dist.begin(), dist.end());
  const bool uneven = longest > 0 && (double)shortest < 0.5 * (double)longest;
  // the chain set: the systems with the longest chains (at most 32), the rest shortened to zero steps
  std::vector<nbg_system_desc> tc1(td1), tc2(td2);
  if (uneven) {
    std::vector<int> ord(nsys);
    for (int s = 0; s < nsys; s++) ord[s] = s;
    // longest chains first: steps times 2N - 3, the pair solves on the critical path of a team step
    auto chain = [&](int q) { return (double)steps_of(desc[q].h, desc[q].tmax) * (2.0 * desc[q].n - 3.0); };
    std::sort(ord.begin(), ord.end(), [&](int a, int b) { return chain(a) > chain(b); });
    const int nchain = std::min(32, std::max(1, nsys / 64));
    for (int q = nchain; q < nsys; q++) {
      tc1[ord[q]].tmax = 0.0;
      tc2[ord[q]].tmax = 0.0;
    }
  }
  std::vector<double> th(nsys);
  std::vector<uint8_t> ph(ap);
  NBG_CUDA(cudaMemcpy(th.data(), t, sizeof(double) * nsys, cudaMemcpyDeviceToHost));
  NBG_CUDA(cudaMemcpy(ph.data(), pair, ap, cudaMemcpyDeviceToHost));
  double *c_t, *c_x, *c_v, *c_xe, *c_ve, *c_J, *c_E, *c_dq, *c_tt, *c_dq0, *c_del;
  long long* c_cnt;
  int rc;
#define GETT(ptr, nm, cnt) if ((rc = ctx->get(nm, (size_t)(cnt), &ptr))) return rc
  GETT(c_t, "a_t", nsys); GETT(c_x, "a_x", ax); GETT(c_v, "a_v", ax); GETT(c_xe, "a_xe", ax); GETT(c_ve, "a_ve", ax);
  GETT(c_J, "a_J", aJ); GETT(c_E, "a_E", aJ); GETT(c_dq, "a_dq", adq); GETT(c_tt, "a_tt", att);
  GETT(c_dq0, "a_dq0", adq0); GETT(c_del, "a_del", adq0); GETT(c_cnt, "a_cnt", am);
#undef GETT
  auto reset = [&]() -> int {
    NBG_CUDA(cudaMemcpyAsync(c_t, t, sizeof(double) * nsys, cudaMemcpyDeviceToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(c_x, x, sizeof(double) * ax, cudaMemcpyDeviceToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(c_v, v, sizeof(double) * ax, cudaMemcpyDeviceToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(c_xe, xerror, sizeof(double) * ax, cudaMemcpyDeviceToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(c_ve, verror, sizeof(double) * ax, cudaMemcpyDeviceToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(c_J, jac_step, sizeof(double) * aJ, cudaMemcpyDeviceToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(c_E, jac_error, sizeof(double) * aJ, cudaMemcpyDeviceToDevice, st));
    NBG_CUDA(cudaMemcpyAsync(c_dq, dqdt, sizeof(double) * adq, cudaMemcpyDeviceToDevice, st));
    NBG_CUDA(cudaMemsetAsync(c_cnt, 0, sizeof(long long) * am, st));
    NBG_CUDA(cudaMemsetAsync(c_tt, 0, sizeof(double) * att, st));
    NBG_CUDA(cudaMemsetAsync(c_dq0, 0, sizeof(double) * adq0, st));
    NBG_CUDA(cudaMemsetAsync(c_del, 0, sizeof(double) * adq0, st));
    return NBG_OK;
  };
  struct Cand { int chunk, team, spw, pw, smem, guard; };
  std::vector<Cand> cands;
  for (int chunk : {64, 128})
    for (int team : {0, 1}) {
      if (team && !any_team) continue;
      // producer blocks of one warp anywhere, or of four warps holding their
      // SM's shared memory so that consumer, operator and search blocks run
      // on the other SMs
      cands.push_back({chunk, team, 0, 1, 0, 0});
      cands.push_back({chunk, team, 0, 4, 200, 32});
    }
  const int save_chunk = ctx->chunk_steps, save_team = ctx->orbit_team, save_spw = ctx->orbit_spw;
  const int save_pw = ctx->prod_warps, save_sm = ctx->prod_smem_kb, save_gd = ctx->guard_smem_kb;
  const int save_prof = ctx->profile;
  ctx->profile = 0;
  int best = -1, nrep = 0;
  double best_ms = 1e300;
  std::vector<double> cand_ms;
  rc = NBG_OK;
  // Untimed warm-up.  The first run of a batch allocates the context's
  // buffers (grow-only, so at the longest chunk of the candidates), and with
  // lazy module loading (the CUDA default) the first launch of each kernel
  // loads it.  Every kernel a candidate can launch runs once here: the
  // one-lane producer, the team producer and, for an uneven batch, the chain
  // set, whose groups take the wide form and the team searches.  Otherwise the
  // first trial to allocate or to use a kernel would carry that cost, and the
  // difference of two trial lengths would understate a step's time.
  int wchunk = 0;
  for (const Cand& cd : cands) wchunk = std::max(wchunk, cd.chunk);
  for (int wteam : {0, 3}) {
    if (wteam && !any_team) continue;
    ctx->chunk_steps = wchunk;
    ctx->orbit_team = wteam;
    ctx->orbit_spw = cands[0].spw;
    ctx->prod_warps = cands[0].pw;
    ctx->prod_smem_kb = cands[0].smem;
    ctx->guard_smem_kb = cands[0].guard;
    for (int r = 0; r < (uneven ? 2 : 1) && !rc; r++) {
      if ((rc = reset())) break;
      rc = run_batch(ctx, nsys, r == 0 ? td1.data() : tc1.data(), th.data(), ph.data(), c_t, c_x, c_v, m, c_xe, c_ve,
                     c_J, c_E, c_dq, jac_init, c_tt, c_dq0, c_del, c_cnt, nullptr);
    }
  }
  for (size_t q = 1; q <= cands.size() && !rc; q++) {
    const Cand& cd = cands[q - 1];
    ctx->chunk_steps = cd.chunk;
    ctx->orbit_team = cd.team ? 3 : 0;  // a team, wide in latency-bound chunks
    ctx->orbit_spw = cd.spw;
    ctx->prod_warps = cd.pw;
    ctx->prod_smem_kb = cd.smem;
    ctx->guard_smem_kb = cd.guard;
    double tms[4] = {0.0, 0.0, 0.0, 0.0};
    const int ntrials = uneven ? 4 : 2;
    for (int r = 0; r < ntrials && !rc; r++) {
      if ((rc = reset())) break;
      const nbg_system_desc* dd = r == 0 ? td1.data() : r == 1 ? td2.data() : r == 2 ? tc1.data() : tc2.data();
      rc = run_batch(ctx, nsys, dd, th.data(), ph.data(), c_t, c_x, c_v, m, c_xe, c_ve, c_J, c_E, c_dq, jac_init, c_tt,
                     c_dq0, c_del, c_cnt, nullptr);
      tms[r] = ctx->last_total_ms;
    }
    if (rc) break;
    const double T1 = std::min<long long>(longest, trial_steps), T2 = std::min<long long>(longest, 2LL * trial_steps);
    const double slope = (T2 > T1) ? std::max(0.0, (tms[1] - tms[0]) / (T2 - T1)) : 0.0;
    double ms = (T2 > T1) ? tms[0] + slope * ((double)longest - T1) : tms[1];
    if (uneven && T2 > T1) {
      const double fill = std::max(0.0, tms[0] - slope * T1);
      const double chain = std::max(0.0, (tms[3] - tms[2]) / (T2 - T1));
      // The time per step falls from `slope` with the whole batch active in
      // proportion to the Jacobian work still active (fraction f), but never
      // below `chain`, the step of the longest chains running alone.
      // walk the steps: between consecutive system lengths the active work is constant
      double model = fill, active = wtot;
      long long k = 0;
      size_t at = 0;
      while (at < dist.size() && k < longest) {
        while (at < dist.size() && dist[at].first <= k) active -= dist[at++].second;
        const long long next = at < dist.size() ? dist[at].first : longest;
        const double f = std::max(0.0, active / wtot);
        model += (double)(next - k) * std::max(slope * f, chain);
        k = next;
      }
      ms = model;
    }
    if (report && nrep < report_len) {
      memset(&report[nrep], 0, sizeof(report[nrep]));
      report[nrep].chunk_steps = cd.chunk;
      report[nrep].orbit_team = cd.team;
      report[nrep].orbit_lanes = cd.spw;
      report[nrep].producer_warps = cd.pw;
      report[nrep].producer_smem_kb = cd.smem;
      report[nrep].ms = ms;
      report[nrep].system_steps_per_s = (double)steps / (ms * 1e-3);
      for (int r = 0; r < 4; r++) report[nrep].trial_ms[r] = tms[r];
    }
    nrep++;
    cand_ms.push_back(ms);
    if (ms < best_ms) {
      best_ms = ms;
      best = (int)q - 1;
    }
  }
  ctx->profile = save_prof;
  // the chosen candidate first in the report
  if (!rc && best > 0 && report && best < std::min(nrep, report_len)) std::swap(report[0], report[best]);
  if (rc || best < 0) {
    ctx->chunk_steps = save_chunk;
    ctx->orbit_team = save_team;
    ctx->orbit_spw = save_spw;
    ctx->prod_warps = save_pw;
    ctx->prod_smem_kb = save_sm;
    ctx->guard_smem_kb = save_gd;
    return rc ? rc : set_error(NBG_EINVAL, "autotune: no candidate ran");
  }
  ctx->chunk_steps = cands[best].chunk;
  ctx->orbit_team = cands[best].team ? 3 : 0;
  ctx->orbit_spw = cands[best].spw;
  ctx->prod_warps = cands[best].pw;
  ctx->prod_smem_kb = cands[best].smem;
  ctx->guard_smem_kb = cands[best].guard;
  if (nreport) *nreport = std::min(nrep, report_len);
  return NBG_OK;
}

int nbg_batch_integrate_transits_noalloc(nbg_context* ctx, int nsys, const nbg_system_desc* desc, double* t,
                                         double* x, double* v, const double* m, double* xerror, double* verror,
                                         double* jac_step, double* jac_error, double* dqdt, const uint8_t* pair,
                                         const double* jac_init, double* tt, double* dtdq0, double* dtdelements,
                                         int64_t* count, uint32_t* status) {
  if (!ctx) return set_error(NBG_EINVAL, "ctx is NULL");
  if (!desc) return set_error(NBG_EINVAL, "desc is NULL");
  if (nsys <= 0 || nsys > NBG_NOALLOC_MAX_SYSTEMS)
    return set_error(NBG_EINVAL, "nbg_batch_integrate_transits_noalloc: nsys = %d not in 1..%d (NBG_NOALLOC_MAX_SYSTEMS)",
                     nsys, NBG_NOALLOC_MAX_SYSTEMS);
  NBG_CUDA(cudaSetDevice(ctx->device));
  return run_batch_noalloc(ctx, *ctx->noalloc, nsys, desc, t, x, v, m, xerror, verror, jac_step, jac_error, dqdt, pair,
                           jac_init, tt, dtdq0, dtdelements, (long long*)count, status);
}

}  // extern "C"
