// nbg_server.cu -- the request server of libnbg_cuda: continuous batching of
// single-system integrate-plus-gradient requests (include/nbg.h,
// nbg_server_*).
//
// Requests of the same (body count, grad, pair pattern) share a *group*: a
// fixed set of C slots holding device-resident system state (structure of
// arrays, as in the batched entry points), the Jacobian columns and the
// per-chunk operator records.  Every group has its own CUDA stream and its
// own chunk counter.  One host thread runs all groups:
//
//   for every group with room on the GPU (< max_inflight chunks queued):
//     admit   -- pending requests of the group take free slots when their
//                output block fits the HBM output arena; their inputs are
//                copied from pinned host memory and scattered into the slots
//     chunk   -- orbit producer, transit searches, operator records and
//                Jacobian consumer for K steps of every active slot; a slot
//                admitted at chunk c0 runs its step k in chunk c0 + k / K
//     retire  -- slots whose last step ran in this chunk are gathered back
//                into their request's layout, dtdelements is formed and the
//                results are copied to the request's pinned host buffer
//   completed chunks (CUDA events) hand their retired requests to pollers.
//
// Each group runs the batched path's three-stream pipeline: admission and
// the orbit producer on one stream, one chunk ahead of the transit searches
// (a second stream) and the operator records, Jacobian consumer and
// retirement (a third); the per-chunk buffers alternate between two halves.
// A slot retired at chunk c is refilled at chunk c + 2 or later, whose
// producer stream waits for chunk c's retirement, so every hand-over is
// stream-ordered and the host never waits for the GPU.  Groups run
// concurrently on their streams.
// Each lane's arithmetic depends on its own system only, so a request's
// results are bitwise the same alone or among any other requests.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <atomic>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "../../include/nbg.h"
#include "nbg_arena.hpp"
#include "nbg_internal.cuh"

using namespace nbg;

namespace {

typedef std::chrono::steady_clock Clock;

// One admitted request's per-slot settings, uploaded to the device.
struct AdmitRec {
  SysOff off;
  long long kbase, nsteps;
  double t0, h, hI;
  int slot, ntt, ti, pad;
};

__global__ void admit_kernel(int n, const AdmitRec* recs, SysOff* d_off, long long* kbase, long long* off_tt,
                             long long* off_dq, int* mask, GroupArgs g) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const AdmitRec r = recs[i];
  const int s = r.slot;
  d_off[s] = r.off;
  kbase[s] = r.kbase;
  off_tt[s] = r.off.tt;
  off_dq[s] = r.off.dq;
  g.nsteps[s] = r.nsteps;
  g.t0[s] = r.t0;
  g.h[s] = r.h;
  g.hI[s] = r.hI;
  g.ntt[s] = r.ntt;
  g.ti[s] = r.ti;
  g.status[s] = 0u;
  g.sysidx[s] = s;
  mask[s] = s;
}

__global__ void mark_kernel(int n, const int* list, int* mask) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) mask[list[i]] = list[i];
}

// kbase of a slot that holds no request.  A byte-wise fill of 0x3f makes it
// (cudaMemsetAsync), and it puts every chunk's first step of the slot far
// below zero, so kernels skip the slot whatever mix of old and new slot
// settings they read while a later chunk's admission rewrites them.
constexpr long long KBASE_FREE = 0x3f3f3f3f3f3f3f3fLL;

// Retirement: the slot is inactive (sysidx = -1) and its kbase leaves the
// request's steps.  Chunk c + 1's kernels may run while chunk c + 2 admits a
// new request into the slot (admit_kernel, on another stream): if one reads
// the new sysidx and nsteps beside the retired kbase, its first step is still
// negative and it skips the slot.
__global__ void deactivate_kernel(int n, const int* list, int* sysidx, long long* kbase) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    sysidx[list[i]] = -1;
    kbase[list[i]] = KBASE_FREE;
  }
}

// Cancellation of running requests (nbg_server_cancel), on the producer
// stream before chunk `first / K` is produced: the slot's step count is cut to
// the steps already run, so that this chunk's and every later chunk's kernels
// skip the slot (the producer queues no transit search for it) while the
// slot keeps its sysidx until its retirement on the consumer stream, as a
// finished request does.  Kernels of the previous chunk that read the cut
// count run fewer steps of a request whose results are discarded.
__global__ void truncate_kernel(int n, const int* list, long long* nsteps, const long long* kbase, long long first) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const int s = list[i];
    long long done = first - kbase[s];
    if (done < 0) done = 0;
    if (nsteps[s] > done) nsteps[s] = done;
  }
}

// Per-slot staging layout (doubles) of a request in the caller's layout:
// x, v, xerror, verror (3N each), m (N), dqdt (7N), count (N int64) and,
// with grad, jac_step, jac_error, jac_init (M^2 each).
struct StageLayout {
  size_t X, V, XE, VE, MM, DQ, CNT, JJ, EE, JI, stride;
  StageLayout(int N, int grad) {
    const size_t M = 7 * (size_t)N;
    X = 0; V = 3 * N; XE = 6 * N; VE = 9 * N; MM = 12 * N; DQ = 13 * N; CNT = 20 * N; JJ = 21 * N;
    EE = JJ + M * M; JI = EE + M * M;
    stride = grad ? JI + M * M : JJ;
  }
};

enum ReqState { REQ_PENDING = 0, REQ_RUNNING = 1, REQ_DONE = 2, REQ_FAILED = 3 };

struct Request {
  int64_t id = 0;
  nbg_system_desc d;
  double t0 = 0, hsig = 0;
  long long nsteps = 0;
  unsigned long long kick = 0;
  size_t stage_n = 0, heap_n = 0;  // doubles
  double* host = nullptr;          // pinned: [stage | tt, dtdq0, dtdelements | status]
  size_t host_cap = 0;
  size_t heap_off = 0;
  int group = -1, slot = -1;
  long long c_admit = 0, c_end = 0;
  Clock::time_point t_arr, t_adm, t_done;
  int state = REQ_PENDING;
  int rc = NBG_OK;
  std::string msg;  // error message of a failed request
  uint32_t status = 0;
  bool released = false;
  // nbg_server_cancel: set under the server mutex; read by the server thread
  std::atomic<bool> cancel{false};
  bool retiring = false;  // its last chunk and retirement are queued (under the mutex)
};

struct Inflight {
  cudaEvent_t ev;
  std::vector<Request*> retired;
  std::vector<Request*> cancelled;  // running requests retired early by nbg_server_cancel
};

struct Group {
  int N = 0, grad = 0, npk = 0;
  unsigned long long kick = 0;
  int C = 0;
  GroupArgs g;
  GroupArgs gh;  // g on the second half of the per-chunk buffers
  StageLayout lay{2, 0};
  double* stage = nullptr;
  SysOff* d_off = nullptr;
  long long *d_kbase = nullptr, *d_offtt = nullptr, *d_offdq = nullptr;
  int* d_mask = nullptr;    // admission mask (producer stream)
  int* d_mask_r = nullptr;  // retirement mask (consumer stream)
  int* d_bad = nullptr;
  AdmitRec* d_admit = nullptr;
  int* d_list = nullptr;
  int* d_list_c = nullptr;  // slots of cancelled requests (producer stream)
  unsigned char* ring = nullptr;  // pinned upload ring: entries of [C AdmitRec][C int]
  size_t ring_entry = 0;
  std::vector<cudaEvent_t> events;  // chunk completion, ring of max_inflight + 1
  cudaEvent_t ev_orb[2] = {nullptr, nullptr}, ev_tr[2] = {nullptr, nullptr};
  cudaStream_t st = nullptr;   // admission and orbit producer
  cudaStream_t sw = nullptr;   // operator records, Jacobian consumer, retirement
  cudaStream_t stt = nullptr;  // transit searches
  std::vector<void*> allocs;
  size_t bytes = 0;
  std::vector<Request*> slot_req;
  std::vector<long long> free_at;  // first chunk at which a retired slot may be refilled
  std::deque<Request*> pending;
  std::deque<Inflight> inflight;
  long long chunk = 0;
  int active = 0;
};

// Pinned host buffers, recycled by power-of-two size class.
struct PinnedPool {
  std::mutex mu;
  std::map<size_t, std::vector<void*>> free_;
  std::vector<void*> all;
  static size_t cls(size_t bytes) {
    size_t c = 4096;
    while (c < bytes) c <<= 1;
    return c;
  }
  void* get(size_t bytes, size_t* cap) {
    const size_t c = cls(bytes);
    *cap = c;
    std::lock_guard<std::mutex> lk(mu);
    auto& v = free_[c];
    if (!v.empty()) {
      void* p = v.back();
      v.pop_back();
      return p;
    }
    void* p = nullptr;
    if (cudaHostAlloc(&p, c, cudaHostAllocPortable) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    all.push_back(p);
    return p;
  }
  void put(void* p, size_t cap) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(mu);
    free_[cap].push_back(p);
  }
  void clear() {
    for (void* p : all) cudaFreeHost(p);
    all.clear();
    free_.clear();
  }
};

}  // namespace

struct nbg_server {
  int device = 0;
  nbg_server_config cfg;
  int sm_count = 0;
  std::thread thread;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stop = false;
  // shared with client threads (under mu)
  int64_t next_id = 1;
  std::unordered_map<int64_t, Request*> reqs;
  std::deque<Request*> incoming;
  std::deque<int64_t> done_ids;
  int fail_rc = NBG_OK;
  std::string fail_msg;
  nbg_server_stats_t stats;
  // threads inside nbg_server_wait_any / nbg_server_poll; nbg_server_stop
  // waits for them to leave before it frees anything they use
  int clients = 0;
  bool closing = false;  // the server thread has exited: waits end
  // server thread only
  std::vector<Group*> groups;
  std::map<std::tuple<int, int, unsigned long long>, int> group_of;
  double* heap = nullptr;
  Arena arena;
  size_t group_bytes = 0;
  PinnedPool pinned;

  void fail(int rc, const std::string& msg) {
    std::lock_guard<std::mutex> lk(mu);
    if (fail_rc == NBG_OK) {
      fail_rc = rc;
      fail_msg = msg;
    }
    cv_done.notify_all();
  }
};

namespace {

// Registers a thread inside nbg_server_wait_any / nbg_server_poll for its
// whole call (the poll's copies run outside the mutex).
struct ClientGuard {
  nbg_server* srv;
  explicit ClientGuard(nbg_server* s) : srv(s) {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->clients++;
  }
  ~ClientGuard() {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->clients--;
    srv->cv_done.notify_all();
  }
};

// Device buffers of a group; charged against the server's budget.
int create_group(nbg_server* srv, int N, int grad, unsigned long long kick, Group** out) {
  Group* G = new Group();
  G->N = N; G->grad = grad; G->kick = kick;
  const int K = srv->cfg.chunk_steps;
  const int C = srv->cfg.slots_per_group;
  G->C = C;
  int npk = 0;
  for (int i = 0; i < N - 1; i++)
    for (int j = i + 1; j < N; j++)
      if (!((kick >> pair_bit(i, j, N)) & 1)) npk++;
  G->npk = npk;
  G->lay = StageLayout(N, grad);
  GroupArgs& g = G->g;
  memset(&g, 0, sizeof(g));
  g.N = N; g.S = C; g.nsys = C; g.grad = grad; g.K = K; g.kick = kick; g.npk = npk;
  g.spw = srv->cfg.orbit_lanes;
  g.team = use_team(srv->cfg.orbit_team, N, kick);
  g.R = step_record_size(N, npk, kick != 0);
  g.task_cap = K * (N - 1) * C;
  g.tgrid = std::min(((g.task_cap + 31) / 32) * 32, std::max(1, srv->sm_count) * 4 * 32);
  // sizes first, so that the budget is checked before anything is allocated
  struct Item { void** p; size_t bytes; };
  std::vector<Item> items;
  auto want = [&](auto** p, size_t count) {
    items.push_back({(void**)p, std::max<size_t>(count * sizeof(**p), 16)});
  };
  const size_t S = C;
  want(&g.x, 3 * N * S); want(&g.v, 3 * N * S); want(&g.xe, 3 * N * S); want(&g.ve, 3 * N * S);
  want(&g.m, N * S); want(&g.dqdt, 7 * N * S); want(&g.gsave, N * S); want(&g.count, N * S);
  want(&g.t0, S); want(&g.h, S); want(&g.hI, S); want(&g.nsteps, S); want(&g.ntt, S); want(&g.ti, S);
  want(&g.sysidx, S); want(&g.status, S);
  // per-chunk buffers: two halves (chunk c uses half c % 2)
  const size_t nf = (size_t)g.task_cap * (12 * N + 2), ni = (size_t)g.task_cap * 3;
  const size_t nrec = (size_t)K * g.R * S, ntrec = (size_t)K * (N - 1) * trec_size(N, 0) * S;
  const size_t nflag = (size_t)K * (N - 1) * S, ncap = (size_t)K * 2 * npk * PCAP * S + 1;
  const size_t nsnap = (size_t)K * snap_count(kick != 0) * 3 * N * S;
  want(&g.task_f, 2 * nf); want(&g.task_i, 2 * ni); want(&g.task_count, 2);
  if (grad) {
    want(&g.steprec, 2 * nrec); want(&g.trec, 2 * ntrec);
    want(&g.tflag, 2 * nflag); want(&g.tscratch, (size_t)g.R * g.tgrid);
    want(&g.pcap, 2 * ncap);
    want(&g.xsnap, 2 * nsnap);
    want(&g.Jint, S * 6 * N * 7 * N); want(&g.Eint, S * 6 * N * 7 * N);
  }
  want(&G->stage, S * G->lay.stride);
  want(&G->d_off, S); want(&G->d_kbase, S); want(&G->d_offtt, S); want(&G->d_offdq, S);
  want(&G->d_mask, S); want(&G->d_mask_r, S); want(&G->d_bad, 1); want(&G->d_admit, S); want(&G->d_list, S); want(&G->d_list_c, S);
  size_t total = 0;
  for (auto& it : items) total += (it.bytes + 255) / 256 * 256;
  if (srv->group_bytes + total > srv->cfg.hbm_budget_bytes / 2) {
    delete G;
    return set_error(NBG_ENOMEM,
                     "server: a group for n = %d, grad = %d needs %zu bytes; groups hold %zu of their %llu-byte half "
                     "of the HBM budget",
                     N, grad, total, srv->group_bytes, (unsigned long long)(srv->cfg.hbm_budget_bytes / 2));
  }
  // one allocation per group, carved into the buffers
  unsigned char* base = nullptr;
  if (cudaMalloc(&base, total) != cudaSuccess) {
    cudaGetLastError();
    delete G;
    return set_error(NBG_ENOMEM, "server: cudaMalloc(%zu bytes) for a group of n = %d failed", total, N);
  }
  G->allocs.push_back(base);
  size_t at = 0;
  for (auto& it : items) {
    *it.p = base + at;
    at += (it.bytes + 255) / 256 * 256;
  }
  G->bytes = total;
  g.kbase = G->d_kbase;
  g.tt = srv->heap;
  g.off_tt = G->d_offtt;
  g.dtdq0 = srv->heap;
  g.off_dq = G->d_offdq;
  G->gh = g;
  G->gh.task_f += nf; G->gh.task_i += ni; G->gh.task_count += 1;
  if (grad) {
    G->gh.steprec += nrec; G->gh.trec += ntrec; G->gh.tflag += nflag; G->gh.pcap += ncap; G->gh.xsnap += nsnap;
  }
  int rc = NBG_OK;
  if (cudaStreamCreateWithFlags(&G->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&G->sw, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&G->stt, cudaStreamNonBlocking) != cudaSuccess)
    rc = NBG_ECUDA;
  for (int e = 0; !rc && e < 2; e++)
    if (cudaEventCreateWithFlags(&G->ev_orb[e], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&G->ev_tr[e], cudaEventDisableTiming) != cudaSuccess)
      rc = NBG_ECUDA;
  G->ring_entry = (sizeof(AdmitRec) + sizeof(int)) * (size_t)C;
  const int D = srv->cfg.max_inflight;
  if (!rc && cudaHostAlloc((void**)&G->ring, G->ring_entry * (D + 1), cudaHostAllocPortable) != cudaSuccess)
    rc = NBG_ECUDA;
  for (int e = 0; !rc && e < D + 1; e++) {
    cudaEvent_t ev;
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) rc = NBG_ECUDA;
    else G->events.push_back(ev);
  }
  if (!rc && (cudaMemsetAsync(g.sysidx, 0xff, sizeof(int) * S, G->st) != cudaSuccess ||
              cudaMemsetAsync(g.nsteps, 0, sizeof(long long) * S, G->st) != cudaSuccess ||
              cudaMemsetAsync(G->d_kbase, 0x3f, sizeof(long long) * S, G->st) != cudaSuccess ||  // KBASE_FREE
              cudaStreamSynchronize(G->st) != cudaSuccess))
    rc = NBG_ECUDA;
  G->slot_req.assign(C, nullptr);
  G->free_at.assign(C, 0);
  if (rc) {
    cudaGetLastError();
    for (auto e : G->events) cudaEventDestroy(e);
    for (int e = 0; e < 2; e++) {
      if (G->ev_orb[e]) cudaEventDestroy(G->ev_orb[e]);
      if (G->ev_tr[e]) cudaEventDestroy(G->ev_tr[e]);
    }
    if (G->ring) cudaFreeHost(G->ring);
    for (cudaStream_t s2 : {G->st, G->sw, G->stt})
      if (s2) cudaStreamDestroy(s2);
    cudaFree(base);
    delete G;
    return set_error(NBG_ECUDA, "server: stream / event / pinned ring creation failed for a group of n = %d", N);
  }
  srv->group_bytes += total;
  *out = G;
  return NBG_OK;
}

void destroy_group(Group* G) {
  for (cudaStream_t s2 : {G->st, G->sw, G->stt})
    if (s2) cudaStreamSynchronize(s2);
  for (auto e : G->events) cudaEventDestroy(e);
  for (int e = 0; e < 2; e++) {
    if (G->ev_orb[e]) cudaEventDestroy(G->ev_orb[e]);
    if (G->ev_tr[e]) cudaEventDestroy(G->ev_tr[e]);
  }
  if (G->ring) cudaFreeHost(G->ring);
  for (cudaStream_t s2 : {G->st, G->sw, G->stt})
    if (s2) cudaStreamDestroy(s2);
  for (void* p : G->allocs) cudaFree(p);
  delete G;
}

// Marks a pending or running request done (rc == 0) or failed; under srv->mu.
void finish(nbg_server* srv, Request* r, int rc, const char* msg = nullptr) {
  if (r->state == REQ_PENDING) srv->stats.pending--;
  else if (r->state == REQ_RUNNING) srv->stats.running--;
  r->state = rc ? REQ_FAILED : REQ_DONE;
  r->rc = rc;
  if (msg) r->msg = msg;
  r->t_done = Clock::now();
  if (rc) srv->stats.failed++;
  else srv->stats.completed++;
  srv->done_ids.push_back(r->id);
}

// One pass over a group: completions, then (room permitting) admission, one
// chunk and retirement.  Returns 1 if it queued GPU work, 0 if not, <0 on error.
int service_group(nbg_server* srv, int gi) {
  Group* G = srv->groups[gi];
  GroupArgs& g = G->g;
  const int N = G->N, K = g.K, C = G->C, D = srv->cfg.max_inflight;
  // ---- completions
  while (!G->inflight.empty()) {
    cudaError_t e = cudaEventQuery(G->inflight.front().ev);
    if (e == cudaErrorNotReady) break;
    if (e != cudaSuccess) return set_error(NBG_ECUDA, "server: chunk failed: %s", cudaGetErrorString(e));
    Inflight f = G->inflight.front();
    G->inflight.pop_front();
    std::lock_guard<std::mutex> lk(srv->mu);
    for (Request* r : f.retired) {
      srv->arena.release(r->heap_off, r->heap_n);
      uint32_t st32;
      memcpy(&st32, r->host + r->stage_n + r->heap_n, sizeof(st32));
      r->status = st32;
      finish(srv, r, NBG_OK);
    }
    for (Request* r : f.cancelled) {
      srv->arena.release(r->heap_off, r->heap_n);
      finish(srv, r, NBG_ECANCELLED, "cancelled while running; its slot was retired at a chunk boundary");
    }
    srv->stats.hbm_outputs_in_use = srv->arena.used * sizeof(double);
    if (!f.retired.empty() || !f.cancelled.empty()) srv->cv_done.notify_all();
  }
  // ---- cancelled requests still waiting for a slot leave the queue
  if (!G->pending.empty()) {
    bool any = false;
    for (Request* r : G->pending) any = any || r->cancel.load(std::memory_order_relaxed);
    if (any) {
      std::lock_guard<std::mutex> lk(srv->mu);
      std::deque<Request*> keep;
      for (Request* r : G->pending) {
        if (r->cancel.load()) finish(srv, r, NBG_ECANCELLED, "cancelled before it was admitted");
        else keep.push_back(r);
      }
      G->pending.swap(keep);
      srv->cv_done.notify_all();
    }
  }
  if ((int)G->inflight.size() >= D) return 0;
  // ---- admission (host decisions; a slot's previous occupant, if any, was
  // retired at chunk c - 2 or earlier, and the producer stream waits for it)
  const long long c = G->chunk;
  const int e = (int)(c % (D + 1));
  AdmitRec* up = (AdmitRec*)(G->ring + (size_t)e * G->ring_entry);
  int* ulist = (int*)(G->ring + (size_t)e * G->ring_entry + sizeof(AdmitRec) * (size_t)C);
  std::vector<Request*> admitted;
  {
    int free_slot = 0;
    while (!G->pending.empty()) {
      while (free_slot < C && (G->slot_req[free_slot] || G->free_at[free_slot] > c)) free_slot++;
      if (free_slot >= C) break;
      Request* r = G->pending.front();
      size_t off;
      if (!srv->arena.alloc(r->heap_n, &off)) break;  // the output arena is full: wait for retirements
      G->pending.pop_front();
      r->heap_off = off;
      r->slot = free_slot;
      r->c_admit = c;
      r->c_end = r->nsteps > 0 ? c + (r->nsteps + K - 1) / K - 1 : c;
      G->slot_req[free_slot] = r;
      G->active++;
      admitted.push_back(r);
    }
  }
  if (!admitted.empty()) {
    std::lock_guard<std::mutex> lk(srv->mu);
    const Clock::time_point now = Clock::now();
    for (Request* r : admitted) {
      r->state = REQ_RUNNING;
      r->t_adm = now;
    }
    srv->stats.admitted += (int64_t)admitted.size();
    srv->stats.pending -= (int64_t)admitted.size();
    srv->stats.running += (int64_t)admitted.size();
    srv->stats.hbm_outputs_in_use = srv->arena.used * sizeof(double);
  }
  if (G->active == 0) return 0;
  cudaStream_t st = G->st, sw = G->sw, stt = G->stt;
  const int par = (int)(c & 1);
  const GroupArgs& gc = par ? G->gh : g;  // this chunk's half of the per-chunk buffers
  const StageLayout& L = G->lay;
  const size_t stride = L.stride;
  long long launches = 0;
  // chunk c reuses chunk c - 2's buffer half and may refill slots retired at
  // chunk c - 2 or earlier: the producer stream waits for that chunk's end
  if (c >= 2) NBG_CUDA(cudaStreamWaitEvent(st, G->events[(c - 2) % (D + 1)], 0));
  if (!admitted.empty()) {
    const int na = (int)admitted.size();
    for (int q = 0; q < na; q++) {
      Request* r = admitted[q];
      AdmitRec& a = up[q];
      memset(&a, 0, sizeof(a));
      const long long sb = (long long)r->slot * (long long)stride;
      a.off.x = a.off.m = a.off.J = a.off.dqdt = a.off.cnt = sb;
      a.off.pair = 0;
      a.off.tt = (long long)r->heap_off;
      a.off.dq = (long long)r->heap_off + (long long)N * r->d.ntt;
      a.off.n = N; a.off.ntt = r->d.ntt; a.off.grad = G->grad; a.off.nr = 1;
      a.kbase = c * K;
      a.nsteps = r->nsteps;
      a.t0 = r->t0; a.h = r->hsig; a.hI = r->d.h;
      a.slot = r->slot; a.ntt = r->d.ntt; a.ti = r->d.ti;
      NBG_CUDA(cudaMemcpyAsync(G->stage + sb, r->host, sizeof(double) * stride, cudaMemcpyHostToDevice, st));
      // a fresh TransitTiming: tt, dtdq0 and dtdelements start at zero
      NBG_CUDA(cudaMemsetAsync(srv->heap + r->heap_off, 0, sizeof(double) * r->heap_n, st));
    }
    NBG_CUDA(cudaMemcpyAsync(G->d_admit, up, sizeof(AdmitRec) * na, cudaMemcpyHostToDevice, st));
    NBG_CUDA(cudaMemsetAsync(G->d_mask, 0xff, sizeof(int) * C, st));
    admit_kernel<<<(na + 127) / 128, 128, 0, st>>>(na, G->d_admit, G->d_off, G->d_kbase, G->d_offtt, G->d_offdq,
                                                    G->d_mask, g);
    const double* sg = G->stage;
    launch_pack_state(N, C, G->d_mask, G->d_off, sg + L.X, sg + L.V, sg + L.XE, sg + L.VE, sg + L.MM, sg + L.DQ,
                      (const long long*)(sg + L.CNT), g, st);
    launches += 2;
    if (G->grad) {
      launch_pack_jac(N, C, G->d_mask, G->d_off, sg + L.JJ, sg + L.EE, g, G->d_bad, st);
      launches++;
    }
    GroupArgs gm = g;
    gm.sysidx = G->d_mask;
    launch_group_seed(N, gm, st);
    launches++;
  }
  // ---- which slots this chunk retires: those whose last step it runs, and
  // those of cancelled requests (cut to the steps already run, below).
  // Decided under the mutex, so that nbg_server_cancel sees either a request
  // whose retirement is queued (too late to cancel) or one that a chunk not
  // yet produced will retire as cancelled.
  Inflight f;
  f.ev = G->events[e];
  int nr = 0, nc = 0;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    for (int s = 0; s < C; s++) {
      Request* r = G->slot_req[s];
      if (!r) continue;
      if (r->cancel.load()) {
        f.cancelled.push_back(r);
      } else if (r->c_end == c) {
        r->retiring = true;
        ulist[nr++] = s;
        f.retired.push_back(r);
      }
    }
  }
  for (Request* r : f.cancelled) ulist[nr + nc++] = r->slot;  // deactivated, not copied out
  if (nc) {
    NBG_CUDA(cudaMemcpyAsync(G->d_list_c, ulist + nr, sizeof(int) * nc, cudaMemcpyHostToDevice, st));
    truncate_kernel<<<(nc + 127) / 128, 128, 0, st>>>(nc, G->d_list_c, g.nsteps, G->d_kbase, c * K);
    launches++;
  }
  // ---- one chunk of every active slot: the producer on st, then the
  // searches on stt beside the operator records on sw, then the consumer
  NBG_CUDA(cudaMemsetAsync(gc.task_count, 0, sizeof(int), st));
  int rc;
  {
    // the wide team form while few slots are running (latency-bound chunks)
    GroupArgs go = gc;
    go.wide = use_wide(srv->cfg.orbit_team, G->active <= std::max(32, srv->sm_count / 2), G->kick) ? 1 : 0;
    if ((rc = launch_group_orbit(N, go, (int)c, st))) return rc;
  }
  NBG_CUDA(cudaEventRecord(G->ev_orb[par], st));
  NBG_CUDA(cudaStreamWaitEvent(stt, G->ev_orb[par], 0));
  NBG_CUDA(cudaStreamWaitEvent(sw, G->ev_orb[par], 0));
  {
    // the team form of the searches while few slots are running (latency-bound searches)
    GroupArgs gs = gc;
    gs.search_team = (G->active <= std::max(32, srv->sm_count / 2)) ? 1 : 0;
    if ((rc = launch_group_transit(N, gs, (int)c, stt))) return rc;
  }
  NBG_CUDA(cudaEventRecord(G->ev_tr[par], stt));
  launches += 2;
  if (G->grad) {
    if ((rc = launch_group_operators(N, gc, (int)c, sw))) return rc;
    launches += 2;
  }
  NBG_CUDA(cudaStreamWaitEvent(sw, G->ev_tr[par], 0));
  if (G->grad) {
    if ((rc = launch_group_jacobian(N, gc, (int)c, sw))) return rc;
    launches += 1;
  }
  // ---- retirement of the slots whose last step ran in this chunk, and of
  // the cancelled ones
  if (nr + nc) {
    // on the consumer stream, after the chunk's consumer and searches
    NBG_CUDA(cudaMemcpyAsync(G->d_list, ulist, sizeof(int) * (nr + nc), cudaMemcpyHostToDevice, sw));
  }
  if (nr) {
    NBG_CUDA(cudaMemsetAsync(G->d_mask_r, 0xff, sizeof(int) * C, sw));
    mark_kernel<<<(nr + 127) / 128, 128, 0, sw>>>(nr, G->d_list, G->d_mask_r);
    double* sg = G->stage;
    launch_unpack_state(N, C, G->grad, G->d_mask_r, G->d_off, sg + L.X, sg + L.V, sg + L.XE, sg + L.VE, sg + L.DQ,
                        (long long*)(sg + L.CNT), g, sw);
    launches += 2;
    if (G->grad) {
      launch_unpack_jac(N, C, G->d_mask_r, G->d_off, sg + L.JJ, sg + L.EE, g, sw);
      launch_dtdelements(nr, G->d_list, G->d_off, srv->heap, sg + L.JI, srv->heap, (const long long*)(sg + L.CNT),
                         true, sw);
      launches += 2;
    }
  }
  if (nr + nc) {
    deactivate_kernel<<<(nr + nc + 127) / 128, 128, 0, sw>>>(nr + nc, G->d_list, g.sysidx, G->d_kbase);
    launches++;
    for (Request* r : f.cancelled) {
      G->slot_req[r->slot] = nullptr;
      G->free_at[r->slot] = c + 2;
      G->active--;
    }
    for (Request* r : f.retired) {
      NBG_CUDA(cudaMemcpyAsync(r->host, G->stage + (size_t)r->slot * stride, sizeof(double) * stride,
                               cudaMemcpyDeviceToHost, sw));
      NBG_CUDA(cudaMemcpyAsync(r->host + r->stage_n, srv->heap + r->heap_off, sizeof(double) * r->heap_n,
                               cudaMemcpyDeviceToHost, sw));
      NBG_CUDA(cudaMemcpyAsync(r->host + r->stage_n + r->heap_n, g.status + r->slot, sizeof(uint32_t),
                               cudaMemcpyDeviceToHost, sw));
      G->slot_req[r->slot] = nullptr;
      G->free_at[r->slot] = c + 2;  // refilled once this chunk's retirement has run
      G->active--;
    }
  }
  NBG_CUDA(cudaGetLastError());
  NBG_CUDA(cudaEventRecord(f.ev, sw));
  G->inflight.push_back(std::move(f));
  G->chunk++;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stats.chunks++;
    srv->stats.kernels += launches;
  }
  return 1;
}

void server_main(nbg_server* srv) {
  if (cudaSetDevice(srv->device) != cudaSuccess) {
    srv->fail(NBG_ECUDA, "server: cudaSetDevice failed");
    return;
  }
  while (true) {
    // new requests -> their group's queue (creating the group on first use)
    std::deque<Request*> in;
    bool stopping;
    {
      std::unique_lock<std::mutex> lk(srv->mu);
      bool busy = false;
      for (Group* G : srv->groups)
        if (G->active || !G->inflight.empty() || !G->pending.empty()) busy = true;
      if (!busy && srv->incoming.empty() && !srv->stop)
        srv->cv_work.wait_for(lk, std::chrono::milliseconds(5));
      in.swap(srv->incoming);
      stopping = srv->stop;
    }
    for (Request* r : in) {
      if (r->cancel.load()) {
        std::lock_guard<std::mutex> lk(srv->mu);
        finish(srv, r, NBG_ECANCELLED, "cancelled before it was admitted");
        srv->cv_done.notify_all();
        continue;
      }
      auto key = std::make_tuple((int)r->d.n, (int)r->d.grad, r->kick);
      auto it = srv->group_of.find(key);
      int gi;
      if (it == srv->group_of.end()) {
        Group* G = nullptr;
        int rc = create_group(srv, r->d.n, r->d.grad, r->kick, &G);
        if (rc) {
          char buf[512];
          nbg_last_error(buf, sizeof(buf));
          std::lock_guard<std::mutex> lk(srv->mu);
          finish(srv, r, rc, buf);
          srv->cv_done.notify_all();
          continue;
        }
        gi = (int)srv->groups.size();
        srv->groups.push_back(G);
        srv->group_of[key] = gi;
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->stats.groups = (int32_t)srv->groups.size();
        srv->stats.hbm_groups = srv->group_bytes;
      } else {
        gi = it->second;
      }
      if (Arena::round(r->heap_n) > srv->arena.size) {
        char buf[256];
        snprintf(buf, sizeof(buf), "server: the request needs %zu output bytes, the output arena holds %zu",
                 r->heap_n * sizeof(double), srv->arena.size * sizeof(double));
        std::lock_guard<std::mutex> lk(srv->mu);
        finish(srv, r, NBG_ENOMEM, buf);
        srv->cv_done.notify_all();
        continue;
      }
      r->group = gi;
      srv->groups[gi]->pending.push_back(r);
    }
    if (stopping) {
      // requests not yet admitted are cancelled; admitted ones run to the end
      std::lock_guard<std::mutex> lk(srv->mu);
      for (Group* G : srv->groups) {
        for (Request* r : G->pending) finish(srv, r, NBG_ECANCELLED, "server stopped before the request ran");
        G->pending.clear();
      }
      srv->cv_done.notify_all();
    }
    int work = 0;
    for (int gi = 0; gi < (int)srv->groups.size(); gi++) {
      int rc = service_group(srv, gi);
      if (rc < 0) {
        char buf[512];
        nbg_last_error(buf, sizeof(buf));
        srv->fail(rc, buf);
        return;
      }
      work += rc;
    }
    if (stopping) {
      bool idle = true;
      for (Group* G : srv->groups)
        if (!G->inflight.empty() || G->active) idle = false;
      if (idle) return;
    }
    if (!work) std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

}  // namespace

// ===================================================================== C ABI

extern "C" {

int nbg_server_start(int device, const nbg_server_config* cfg_in, nbg_server** out) {
  if (!out) return set_error(NBG_EINVAL, "out is NULL");
  *out = nullptr;
  int ndev = 0;
  NBG_CUDA(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) return set_error(NBG_EINVAL, "device %d not in 0..%d", device, ndev - 1);
  NBG_CUDA(cudaSetDevice(device));
  nbg_server_config cfg;
  memset(&cfg, 0, sizeof(cfg));
  if (cfg_in) cfg = *cfg_in;
  if (cfg.slots_per_group < 0 || cfg.chunk_steps < 0 || cfg.max_inflight < 0 || cfg.orbit_lanes < 0 ||
      cfg.orbit_lanes > 32 || cfg.chunk_steps > 4096 || cfg.slots_per_group > (1 << 20) || cfg.max_inflight > 16)
    return set_error(NBG_EINVAL, "server config out of range");
  if (!cfg.slots_per_group) cfg.slots_per_group = 256;
  cfg.slots_per_group = (cfg.slots_per_group + 31) / 32 * 32;
  if (!cfg.chunk_steps) cfg.chunk_steps = 32;
  if (!cfg.max_inflight) cfg.max_inflight = 2;
  if (!cfg.orbit_lanes) cfg.orbit_lanes = 32;
  if (cfg.orbit_team < -2 || cfg.orbit_team > 1) return set_error(NBG_EINVAL, "orbit_team = %d", cfg.orbit_team);
  cfg.orbit_team = cfg.orbit_team == 0 ? -1 : (cfg.orbit_team == -2 ? 0 : cfg.orbit_team);  // use_team's modes
  if (!cfg.hbm_budget_bytes) {
    size_t fr = 0, tot = 0;
    NBG_CUDA(cudaMemGetInfo(&fr, &tot));
    cfg.hbm_budget_bytes = fr / 4;
  }
  nbg_server* srv = new nbg_server();
  srv->device = device;
  srv->cfg = cfg;
  memset(&srv->stats, 0, sizeof(srv->stats));
  srv->stats.hbm_budget = cfg.hbm_budget_bytes;
  {
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, device) == cudaSuccess) srv->sm_count = p.multiProcessorCount;
  }
  const size_t arena_doubles = (size_t)(cfg.hbm_budget_bytes / 2) / sizeof(double) / 32 * 32;
  if (arena_doubles == 0 || cudaMalloc(&srv->heap, arena_doubles * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    delete srv;
    return set_error(NBG_ENOMEM, "server: output arena of %zu bytes could not be allocated",
                     arena_doubles * sizeof(double));
  }
  srv->arena.init(arena_doubles);
  srv->thread = std::thread(server_main, srv);
  *out = srv;
  return NBG_OK;
}

int nbg_server_enqueue(nbg_server* srv, const nbg_system_desc* desc, double t0, const double* x, const double* v,
                       const double* m, const double* xerror, const double* verror, const double* jac_step,
                       const double* jac_error, const double* dqdt, const uint8_t* pair, const double* jac_init,
                       int64_t* id) {
  if (!srv || !desc || !id) return set_error(NBG_EINVAL, "NULL argument");
  const nbg_system_desc d = *desc;
  if (d.n < NBG_MIN_BODIES || d.n > NBG_MAX_BODIES)
    return set_error(NBG_EUNSUPPORTED, "n = %d outside the built range %d..%d", d.n, NBG_MIN_BODIES, NBG_MAX_BODIES);
  if (d.ti < 0 || d.ti >= d.n) return set_error(NBG_EINVAL, "ti = %d not in 0..%d", d.ti, d.n - 1);
  if (d.ntt < 1) return set_error(NBG_EINVAL, "ntt = %d < 1", d.ntt);
  if (!(d.h != 0.0) || !std::isfinite(d.h) || !std::isfinite(d.tmax) || !std::isfinite(t0))
    return set_error(NBG_EINVAL, "h = %g, tmax = %g, t0 = %g", d.h, d.tmax, t0);
  if (!x || !v || !m || !xerror || !verror || !pair) return set_error(NBG_EINVAL, "NULL array argument");
  const int grad = d.grad ? 1 : 0;
  const int N = d.n, M = 7 * N;
  if (grad && (!jac_step || !jac_error || !jac_init || !dqdt))
    return set_error(NBG_EINVAL, "grad requests need jac_step, jac_error, jac_init and dqdt");
  if (grad)
    for (int r = 6; r < M; r += 7)
      for (int c2 = 0; c2 < M; c2++)
        if (jac_step[r + (size_t)M * c2] != ((r == c2) ? 1.0 : 0.0) || jac_error[r + (size_t)M * c2] != 0.0)
          return set_error(NBG_EUNSUPPORTED,
                           "jac_step mass rows must be unit rows with zero jac_error (true for every State the "
                           "reference builds and integrates)");
  Request* r = new Request();
  r->d = d;
  r->d.grad = grad;
  r->t0 = t0;
  r->nsteps = steps_of(d.h, d.tmax);
  r->hsig = d.h * check_step(t0, d.tmax + t0);
  for (int i = 0; i < N - 1; i++)
    for (int j = i + 1; j < N; j++)
      if (pair[i + (size_t)N * j]) r->kick |= 1ull << pair_bit(i, j, N);
  const StageLayout L(N, grad);
  r->stage_n = L.stride;
  r->heap_n = (size_t)N * d.ntt + (grad ? 2 * (size_t)7 * N * N * d.ntt : 0);
  const size_t bytes = sizeof(double) * (r->stage_n + r->heap_n + 1);
  int prev_dev = 0;
  cudaGetDevice(&prev_dev);
  cudaSetDevice(srv->device);
  r->host = (double*)srv->pinned.get(bytes, &r->host_cap);
  cudaSetDevice(prev_dev);
  if (!r->host) {
    delete r;
    return set_error(NBG_ENOMEM, "server: pinned host buffer of %zu bytes", bytes);
  }
  double* h = r->host;
  memcpy(h + L.X, x, sizeof(double) * 3 * N);
  memcpy(h + L.V, v, sizeof(double) * 3 * N);
  memcpy(h + L.XE, xerror, sizeof(double) * 3 * N);
  memcpy(h + L.VE, verror, sizeof(double) * 3 * N);
  memcpy(h + L.MM, m, sizeof(double) * N);
  if (dqdt) memcpy(h + L.DQ, dqdt, sizeof(double) * M);
  else memset(h + L.DQ, 0, sizeof(double) * M);
  memset(h + L.CNT, 0, sizeof(double) * N);  // a fresh TransitTiming: count = 0
  if (grad) {
    memcpy(h + L.JJ, jac_step, sizeof(double) * M * M);
    memcpy(h + L.EE, jac_error, sizeof(double) * M * M);
    memcpy(h + L.JI, jac_init, sizeof(double) * M * M);
  }
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    if (srv->stop) {
      srv->pinned.put(r->host, r->host_cap);
      delete r;
      return set_error(NBG_ECANCELLED, "server is stopping");
    }
    if (srv->fail_rc) {
      srv->pinned.put(r->host, r->host_cap);
      delete r;
      return set_error(srv->fail_rc, "server failed: %s", srv->fail_msg.c_str());
    }
    r->id = srv->next_id++;
    r->t_arr = Clock::now();
    srv->reqs[r->id] = r;
    srv->incoming.push_back(r);
    srv->stats.submitted++;
    srv->stats.pending++;
    *id = r->id;
  }
  srv->cv_work.notify_one();
  return NBG_OK;
}

int nbg_server_wait_any(nbg_server* srv, int32_t timeout_ms, int64_t* id) {
  if (!srv || !id) return set_error(NBG_EINVAL, "NULL argument");
  ClientGuard guard(srv);
  std::unique_lock<std::mutex> lk(srv->mu);
  auto pred = [&] {
    while (!srv->done_ids.empty()) {
      auto it = srv->reqs.find(srv->done_ids.front());
      if (it != srv->reqs.end() && !it->second->released) return true;
      srv->done_ids.pop_front();  // already collected by nbg_server_poll
    }
    return srv->fail_rc != NBG_OK || srv->closing;
  };
  if (timeout_ms < 0) srv->cv_done.wait(lk, pred);
  else if (!srv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred))
    return set_error(NBG_ETIMEOUT, "no request completed within %d ms", timeout_ms);
  if (srv->done_ids.empty()) {
    if (srv->fail_rc != NBG_OK) return set_error(srv->fail_rc, "server failed: %s", srv->fail_msg.c_str());
    return set_error(NBG_ECANCELLED, "server stopped with no completed request left to collect");
  }
  *id = srv->done_ids.front();
  srv->done_ids.pop_front();
  return NBG_OK;
}

int nbg_server_poll(nbg_server* srv, int64_t id, int32_t timeout_ms, double* t, double* x, double* v,
                    double* xerror, double* verror, double* jac_step, double* jac_error, double* dqdt, double* tt,
                    double* dtdq0, double* dtdelements, int64_t* count, nbg_request_info* info) {
  if (!srv) return set_error(NBG_EINVAL, "srv is NULL");
  ClientGuard guard(srv);
  Request* r;
  {
    std::unique_lock<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(id);
    if (it == srv->reqs.end()) return set_error(NBG_EINVAL, "unknown request id %lld", (long long)id);
    r = it->second;
    auto done = [&] { return r->state == REQ_DONE || r->state == REQ_FAILED || srv->fail_rc != NBG_OK; };
    if (timeout_ms < 0) srv->cv_done.wait(lk, done);
    else if (!srv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done))
      return set_error(NBG_ETIMEOUT, "request %lld not complete within %d ms", (long long)id, timeout_ms);
    if (r->state != REQ_DONE && r->state != REQ_FAILED)
      return set_error(srv->fail_rc, "server failed: %s", srv->fail_msg.c_str());
    srv->reqs.erase(it);
    r->released = true;
  }
  const int N = r->d.n, M = 7 * N, grad = r->d.grad;
  const int rc = r->rc;
  if (info) {
    memset(info, 0, sizeof(*info));
    info->id = r->id;
    info->n = N;
    info->grad = grad;
    info->nsteps = r->nsteps;
    auto ms = [](Clock::time_point a, Clock::time_point b) {
      return std::chrono::duration<double, std::milli>(b - a).count();
    };
    const bool ran = r->slot >= 0;
    info->queue_ms = ran ? ms(r->t_arr, r->t_adm) : ms(r->t_arr, r->t_done);
    info->run_ms = ran ? ms(r->t_adm, r->t_done) : 0.0;
    info->latency_ms = ms(r->t_arr, r->t_done);
    info->status = r->status;
    info->rc = rc;
  }
  const std::string msg = r->msg;
  if (rc == NBG_OK) {
    const StageLayout L(N, grad);
    const double* h = r->host;
    if (t) t[0] = r->nsteps > 0 ? r->t0 + (double)r->nsteps * r->hsig : r->t0;
    if (x) memcpy(x, h + L.X, sizeof(double) * 3 * N);
    if (v) memcpy(v, h + L.V, sizeof(double) * 3 * N);
    if (xerror) memcpy(xerror, h + L.XE, sizeof(double) * 3 * N);
    if (verror) memcpy(verror, h + L.VE, sizeof(double) * 3 * N);
    if (count) memcpy(count, h + L.CNT, sizeof(int64_t) * N);
    const double* ho = h + r->stage_n;
    if (tt) memcpy(tt, ho, sizeof(double) * N * r->d.ntt);
    if (grad) {
      const size_t lq = (size_t)7 * N * N * r->d.ntt;
      if (dqdt) memcpy(dqdt, h + L.DQ, sizeof(double) * M);
      if (jac_step) memcpy(jac_step, h + L.JJ, sizeof(double) * M * M);
      if (jac_error) memcpy(jac_error, h + L.EE, sizeof(double) * M * M);
      if (dtdq0) memcpy(dtdq0, ho + (size_t)N * r->d.ntt, sizeof(double) * lq);
      if (dtdelements) memcpy(dtdelements, ho + (size_t)N * r->d.ntt + lq, sizeof(double) * lq);
    }
  }
  srv->pinned.put(r->host, r->host_cap);
  delete r;
  if (rc) return set_error(rc, "request %lld failed: %s", (long long)id, msg.empty() ? "(no message)" : msg.c_str());
  return NBG_OK;
}

int nbg_server_cancel(nbg_server* srv, int64_t id) {
  if (!srv) return set_error(NBG_EINVAL, "srv is NULL");
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(id);
    if (it == srv->reqs.end()) return set_error(NBG_EINVAL, "unknown request id %lld", (long long)id);
    Request* r = it->second;
    if (r->state == REQ_DONE || r->state == REQ_FAILED || r->retiring)
      return set_error(NBG_EINVAL, "request %lld has already finished or is being retired: its result stands",
                       (long long)id);
    r->cancel.store(true);
  }
  srv->cv_work.notify_one();
  return NBG_OK;
}

int nbg_server_stats(nbg_server* srv, nbg_server_stats_t* out) {
  if (!srv || !out) return set_error(NBG_EINVAL, "NULL argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  *out = srv->stats;
  return NBG_OK;
}

int nbg_server_stop(nbg_server* srv) {
  if (!srv) return NBG_OK;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stop = true;
  }
  srv->cv_work.notify_all();
  if (srv->thread.joinable()) srv->thread.join();
  {
    // every request has reached its end (admitted ones ran to completion,
    // the others were cancelled): let the threads collecting them finish
    std::unique_lock<std::mutex> lk(srv->mu);
    srv->closing = true;
    srv->cv_done.notify_all();
    srv->cv_done.wait(lk, [&] { return srv->clients == 0; });
  }
  cudaSetDevice(srv->device);
  for (Group* G : srv->groups) destroy_group(G);
  srv->groups.clear();
  if (srv->heap) cudaFree(srv->heap);
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    for (auto& kv : srv->reqs) {
      srv->pinned.put(kv.second->host, kv.second->host_cap);
      delete kv.second;
    }
    srv->reqs.clear();
    srv->incoming.clear();  // every request not yet polled is in reqs
  }
  srv->pinned.clear();
  const int rc = srv->fail_rc;
  delete srv;
  return rc == NBG_OK ? NBG_OK : rc;
}

}  // extern "C"
