// nbg_kernels_impl.cuh -- the per-body-count kernels of libnbg_cuda and their
// launchers.  Included only by nbg_inst.cu, which instantiates them for one
// body count N per translation unit (the units compile in parallel).
//
// Work decomposition (one launch pair per chunk of K steps):
//   orbit_chunk_kernel<N>     one lane per system: x, v, dq/dt, transit search
//                             (src/transits/timing.jl:3-109); writes the step
//                             operator records, tt and per-transit adjoint rows
//   jacobian_chunk_kernel<N>  one lane per (system, column of jac_step): applies
//                             the records with Kahan summation and turns each
//                             transit's adjoint row into dtdq0 entries
// Systems are grouped by (N, grad, kick pattern) so that every warp runs one
// control-flow path; within a group systems are sorted longest first.
#pragma once
#include <algorithm>

#include "../../include/nbg.h"
#include "nbg_jacobian.cuh"
#include "nbg_orbit_team.cuh"

namespace nbg {

// Orbit producer for one chunk of K steps of one group (one lane per system).
template <int N>
__global__ void __launch_bounds__(PROD_BS * PROD_MAX_WARPS) orbit_chunk_kernel(GroupArgs g, int chunk) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane >= g.spw) return;
  const int s = (blockIdx.x * (g.pwarps > 0 ? g.pwarps : 1) + warp) * g.spw + lane;
  if (s >= g.S || g.sysidx[s] < 0) return;
  const int S = g.S;
  const long long nst = g.nsteps[s];
  const long long k0 = chunk_first_step(g, chunk, s);
  if (k0 >= nst || k0 < 0) return;  // done, or admitted for a later chunk
  Sys<N> st;
  Work<N> w;
  for (int q = 0; q < 3 * N; q++) {
    st.x[q] = g.x[q * S + s];
    st.v[q] = g.v[q * S + s];
    st.xe[q] = g.xe[q * S + s];
    st.ve[q] = g.ve[q * S + s];
  }
  for (int q = 0; q < N; q++) st.m[q] = g.m[q * S + s];
  for (int q = 0; q < 7 * N; q++) st.dqdt[q] = g.dqdt[q * S + s];
  double gsave[N];
  long long count[N];
  for (int q = 0; q < N; q++) {
    gsave[q] = g.gsave[q * S + s];
    count[q] = g.count[q * S + s];
  }
  const double t0 = g.t0[s], h = g.h[s], hI = g.hI[s];
  const int ntt = g.ntt[s], ti = g.ti[s];
  const uint64_t kick = g.kick;
  // status bits raised in this chunk; or-ed into the system's word at the end
  // (the transit searches and the consumer of the previous chunk may be
  // or-ing theirs in meanwhile)
  unsigned int status = 0;
  for (int kk = 0; kk < g.K; kk++) {
    const long long istep = k0 + kk;
    if (istep >= nst) break;
    const double hs = step_length(g, s, istep, nst, h);
    if (g.trajxv) {
      double* rx = g.trajxv + ((size_t)s * g.K + kk) * 6 * N;
      for (int q = 0; q < 3 * N; q++) {
        rx[q] = st.x[q];
        rx[3 * N + q] = st.v[q];
      }
    }
    if (g.grad) {
      // x, v only; the operators are built from the captures by the operator
      // kernels.  The last step also computes dq/dt, the State's output.
      Rec cap{g.pcap + (size_t)kk * 2 * g.npk * PCAP * S + s, S};
      Rec xs{g.xsnap + (size_t)kk * snap_count(kick != 0) * 3 * N * S + s, S};
      if (istep == nst - 1) ahl21_step<N, true, true>(st, w, hs, kick, Rec{nullptr, 0}, cap, xs);
      else ahl21_step<N, false, false>(st, w, hs, kick, Rec{nullptr, 0}, cap, xs);
    } else {
      ahl21_step<N, false, false>(st, w, hs, kick, Rec{nullptr, 0}, Rec{nullptr, 0}, Rec{nullptr, 0});
    }
    if (g.notransit) continue;
    const double t = t0 + (double)(istep + 1) * h;
    // detect_transits! (timing.jl:3-28).  The search itself (findtransit!) is
    // queued: it runs from a copy of this state in transit_kernel, with full
    // warps, instead of stalling the 31 other systems of this warp.
    for (int o = 0; o < N - 1; o++) {
      const int ib = (o < ti) ? o : o + 1;
      const double gi = gsky(st, ib, ti);
      const double xi = st.x[3 * ib], yi = st.x[3 * ib + 1], zi = st.x[3 * ib + 2];
      const double ri = sqrt(xi * xi + yi * yi + zi * zi);
      if (g.grad) g.tflag[(size_t)(kk * (N - 1) + o) * S + s] = -1;
      if (gi > 0.0 && gsave[ib] < 0.0 && -zi > 0.25 * ri && ri < 1e12) {
        count[ib] += 1;
        if (count[ib] <= ntt) {
          const int idx = atomicAdd(g.task_count, 1);
          if (idx < g.task_cap) {  // the capacity is the number of (step, occultor, system) slots
            double* tf = g.task_f + (size_t)idx * (12 * N + 2);
            for (int q = 0; q < 3 * N; q++) {
              tf[q] = st.x[q];
              tf[3 * N + q] = st.v[q];
              tf[6 * N + q] = st.xe[q];
              tf[9 * N + q] = st.ve[q];
            }
            tf[12 * N] = -gi * hI / (gi - gsave[ib]);  // first estimate (timing.jl:20)
            tf[12 * N + 1] = t;
            int* tk = g.task_i + 3 * idx;
            tk[0] = s;
            tk[1] = kk * (N - 1) + o;
            tk[2] = (int)(count[ib] - 1);
          }
        } else {
          status |= NBG_STATUS_NTT_OVERFLOW;
        }
      }
      gsave[ib] = gi;
    }
  }
  for (int q = 0; q < 3 * N; q++) {
    g.x[q * S + s] = st.x[q];
    g.v[q * S + s] = st.v[q];
    g.xe[q * S + s] = st.xe[q];
    g.ve[q * S + s] = st.ve[q];
  }
  if (g.grad && nst <= k0 + g.K)  // the chunk that ran the last step holds the final dq/dt
    for (int q = 0; q < 7 * N; q++) g.dqdt[q * S + s] = st.dqdt[q];
  for (int q = 0; q < N; q++) {
    g.gsave[q * S + s] = gsave[q];
    g.count[q * S + s] = count[q];
  }
  if (!state_finite<N>(st)) status |= NBG_STATUS_NONFINITE;
  if (status) atomicOr(g.status + s, status);
}


// findtransit! (src/transits/timing.jl:31-109) for the searches the orbit
// producer queued in this chunk: Newton iterations on partial AHL21 steps
// from the end-of-step state, then (grad) the partial step at the converged
// dt0 with its operator records and the adjoint row u^T = w^T S(dt0) that the
// Jacobian consumer turns into dtdq0 (dtbvdq! row 1, timing.jl:155-171).
// The iterations take x, v only and the physical time derivative of g
// (gdot_physical) where the reference builds the full gradient step to read
// g's step derivative: both iterations stop at the same root of g to
// rounding; the converged search's step keeps the reference's derivative,
// which dtdq0 divides by.
//
// Everything after the Newton iterations, for one search on one lane: st is
// the search's start state, wk the last iterate's state, dt0 the converged
// step; the operator records of the final partial step go to this lane's
// column `lane_id` of tscratch (lane_ids in 0..lanes-1).
template <int N>
__device__ void search_finish(const GroupArgs& g, int s, int slot, int c, int ib, int ti, const Sys<N>& st,
                              Sys<N>& wk, double dt0, double t, int iter, Work<N>& w, int lane_id, int lanes) {
  const int S = g.S;
  const uint64_t kick = g.kick;
  if (iter >= 20) atomicOr(g.status + s, NBG_STATUS_NEWTON_ITMAX);
  const int nr = g.tbv ? 3 : 1;
  double* ttout = g.tt + g.off_tt[g.sysidx[s]] + (long long)nr * (ib + (long long)N * c);
  if (g.tbv && !g.grad) {
    // TransitParameters without gradient (timing.jl:96-97): v_sky and
    // b_sky^2 of the last Newton iteration's state
    const double dvx = wk.v[3 * ib] - wk.v[3 * ti], dvy = wk.v[3 * ib + 1] - wk.v[3 * ti + 1];
    const double dx = wk.x[3 * ib] - wk.x[3 * ti], dy = wk.x[3 * ib + 1] - wk.x[3 * ti + 1];
    ttout[1] = sqrt(dvx * dvx + dvy * dvy);
    ttout[2] = dx * dx + dy * dy;
  }
  if (g.grad) {
    wk = st;
    Rec rec{g.tscratch + lane_id, lanes};
    ahl21_step<N, true, true>(wk, w, dt0, kick, rec, Rec{nullptr, 0}, Rec{nullptr, 0});
    double u[7 * N];
    for (int q = 0; q < 7 * N; q++) u[q] = 0.0;
    const double dvx = wk.v[3 * ib] - wk.v[3 * ti], dvy = wk.v[3 * ib + 1] - wk.v[3 * ti + 1];
    const double dx = wk.x[3 * ib] - wk.x[3 * ti], dy = wk.x[3 * ib + 1] - wk.x[3 * ti + 1];
    u[7 * ib + 0] = dvx;
    u[7 * ti + 0] = -dvx;
    u[7 * ib + 1] = dvy;
    u[7 * ti + 1] = -dvy;
    u[7 * ib + 3] = dx;
    u[7 * ti + 3] = -dx;
    u[7 * ib + 4] = dy;
    u[7 * ti + 4] = -dy;
    adjoint_step<N>(u, dt0, kick, rec);
    const double gd = gdot(wk, ti, ib);
    double* tr = g.trec + ((size_t)slot * trec_size(N, g.tbv)) * S + s;
    for (int q = 0; q < 7 * N; q++) tr[(size_t)q * S] = u[q];
    if (g.tbv) {
      // dtbvdq! rows 2 and 3 (timing.jl:173-191): v_sky and b_sky^2 of the
      // converged state, dv_sky/dt, and the adjoint rows of their
      // numerators (d v_sky: the sky velocity difference on the velocity
      // rows; d b_sky^2 / 2: the sky position difference on the position rows)
      const double vsky = sqrt(dvx * dvx + dvy * dvy);
      const double bsky2 = dx * dx + dy * dy;
      const double* q = wk.dqdt;
      const double dvdt = (dvx * (q[7 * ib + 3] - q[7 * ti + 3]) + dvy * (q[7 * ib + 4] - q[7 * ti + 4])) / vsky;
      for (int r = 0; r < 2; r++) {
        for (int e = 0; e < 7 * N; e++) u[e] = 0.0;
        if (r == 0) {
          u[7 * ib + 3] = dvx;
          u[7 * ti + 3] = -dvx;
          u[7 * ib + 4] = dvy;
          u[7 * ti + 4] = -dvy;
        } else {
          u[7 * ib + 0] = dx;
          u[7 * ti + 0] = -dx;
          u[7 * ib + 1] = dy;
          u[7 * ti + 1] = -dy;
        }
        adjoint_step<N>(u, dt0, kick, rec);
        for (int e = 0; e < 7 * N; e++) tr[(size_t)(7 * N * (r + 1) + e) * S] = u[e];
      }
      tr[(size_t)(21 * N) * S] = gd;
      tr[(size_t)(21 * N + 1) * S] = vsky;
      tr[(size_t)(21 * N + 2) * S] = dvdt;
      ttout[1] = vsky;
      ttout[2] = bsky2;
    } else {
      tr[(size_t)(7 * N) * S] = gd;
    }
    g.tflag[(size_t)slot * S + s] = c;
  }
  ttout[0] = t + dt0;
}

// One lane per search, grid-stride over the queue.
template <int N>
__global__ void __launch_bounds__(TRANSIT_BS) transit_kernel(GroupArgs g, int chunk) {
  const int ntask = min(*g.task_count, g.task_cap);
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int G = gridDim.x * blockDim.x;
  const int S = g.S;
  Work<N> w;
  for (int idx = tid; idx < ntask; idx += G) {
    const int* tk = g.task_i + 3 * idx;
    const int s = tk[0], slot = tk[1], c = tk[2];
    const int o = slot % (N - 1);
    const int ti = g.ti[s];
    const int ib = (o < ti) ? o : o + 1;
    const double* tf = g.task_f + (size_t)idx * (12 * N + 2);
    Sys<N> st;
    for (int q = 0; q < 3 * N; q++) {
      st.x[q] = tf[q];
      st.v[q] = tf[3 * N + q];
      st.xe[q] = tf[6 * N + q];
      st.ve[q] = tf[9 * N + q];
    }
    for (int q = 0; q < N; q++) st.m[q] = g.m[q * S + s];
    for (int q = 0; q < 7 * N; q++) st.dqdt[q] = 0.0;
    double dt0 = tf[12 * N];
    const double t = tf[12 * N + 1];
    const uint64_t kick = g.kick;
    double stmp = 0.0, tt1 = dt0 + 1.0, tt2 = dt0 + 2.0;
    int iter = 0;
    Sys<N> wk;
    while (true) {
      tt2 = tt1;
      tt1 = dt0;
      wk = st;
      ahl21_step<N, false, false>(wk, w, dt0, kick, Rec{nullptr, 0}, Rec{nullptr, 0}, Rec{nullptr, 0});
      const double gs = gsky(wk, ti, ib);
      const double gd = gdot_physical(wk, ti, ib);
      const double dt = -gs / gd;
      kahan(dt0, stmp, dt);
      iter += 1;
      if (iter >= 20 || dt0 == tt1 || dt0 == tt2) break;
    }
    search_finish<N>(g, s, slot, c, ib, ti, st, wk, dt0, t, iter, w, tid, G);
  }
}

// Shared memory of the team search per warp: per team the search's start
// state, the Newton iterate and the accelerations of phisalpha!.
template <int N>
__host__ __device__ constexpr int search_team_smem_bytes() {
  return (PROD_BS / team_lanes(N)) * (int)(2 * sizeof(Sys<N>) + 3 * N * sizeof(double));
}

// Team form of the searches (groups without kick pairs): a team of
// L = team_lanes(N) lanes per search, T = 32 / L searches per warp, one warp
// per block.  The Newton iterations run the level-parallel step of the team
// producer (team_step, bitwise the one-lane no-gradient step) on the
// team's shared-memory copy of the state, so their critical path is
// 2(2N - 3) pair solves per iteration instead of N(N - 1); every lane of a
// team computes g, its derivative and the update of dt0 from the same
// shared values, so a team stops together.  The final partial step with its
// records and the adjoint rows run on the team's first lane
// (search_finish), as in the one-lane kernel.  Results are bitwise those of
// transit_kernel.
template <int N>
__global__ void __launch_bounds__(TRANSIT_BS) transit_team_kernel(GroupArgs g, int chunk) {
  constexpr int L = team_lanes(N);
  constexpr int T = PROD_BS / L;
  extern __shared__ double search_smem[];
  Sys<N>* st0 = reinterpret_cast<Sys<N>*>(search_smem);
  Sys<N>* wks = st0 + T;
  double(*acc)[3 * N] = reinterpret_cast<double(*)[3 * N]>(wks + T);
  const int ntask = min(*g.task_count, g.task_cap);
  const int lane = threadIdx.x & 31;
  const int team = lane / L, t = lane % L;
  const bool in_team = team < T;
  const int tm = in_team ? team : 0;  // idle lanes alias team 0 but never write
  const int S = g.S;
  const int teams = gridDim.x * T;
  Work<N> w;
  for (int base = blockIdx.x * T; base < ntask; base += teams) {
    const int idx = base + tm;
    const bool has = in_team && idx < ntask;
    int s = 0, slot = 0, c = 0, ti = 0, ib = 0;
    double dt0 = 0.0, t_end = 0.0;
    if (has) {
      const int* tk = g.task_i + 3 * idx;
      s = tk[0];
      slot = tk[1];
      c = tk[2];
      const int o = slot % (N - 1);
      ti = g.ti[s];
      ib = (o < ti) ? o : o + 1;
      const double* tf = g.task_f + (size_t)idx * (12 * N + 2);
      for (int q = t; q < 3 * N; q += L) {
        st0[tm].x[q] = tf[q];
        st0[tm].v[q] = tf[3 * N + q];
        st0[tm].xe[q] = tf[6 * N + q];
        st0[tm].ve[q] = tf[9 * N + q];
      }
      for (int q = t; q < N; q += L) st0[tm].m[q] = g.m[q * S + s];
      for (int q = t; q < 7 * N; q += L) st0[tm].dqdt[q] = 0.0;
      dt0 = tf[12 * N];
      t_end = tf[12 * N + 1];
    }
    __syncwarp();
    double stmp = 0.0, tt1 = dt0 + 1.0, tt2 = dt0 + 2.0;
    int iter = 0;
    bool active = has;
    while (__any_sync(0xffffffffu, active)) {
      if (active) {
        tt2 = tt1;
        tt1 = dt0;
        for (int q = t; q < 3 * N; q += L) {
          wks[tm].x[q] = st0[tm].x[q];
          wks[tm].v[q] = st0[tm].v[q];
          wks[tm].xe[q] = st0[tm].xe[q];
          wks[tm].ve[q] = st0[tm].ve[q];
        }
        for (int q = t; q < N; q += L) wks[tm].m[q] = st0[tm].m[q];
      }
      __syncwarp();
      team_step<N>(wks[tm], acc[tm], w, t, active, dt0, Rec{nullptr, 0}, Rec{nullptr, 0});
      __syncwarp();
      if (active) {
        const double gs = gsky(wks[tm], ti, ib);
        const double gd = gdot_physical(wks[tm], ti, ib);
        const double dt = -gs / gd;
        kahan(dt0, stmp, dt);
        iter += 1;
        if (iter >= 20 || dt0 == tt1 || dt0 == tt2) active = false;
      }
      __syncwarp();
    }
    if (has && t == 0) {
      Sys<N> st = st0[tm];
      Sys<N> wk = wks[tm];
      search_finish<N>(g, s, slot, c, ib, ti, st, wk, dt0, t_end, iter, w,
                       blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
    }
    __syncwarp();
  }
}

// Kepler-pair records of one chunk: one lane per (step, pair slot, system),
// consecutive lanes = consecutive systems, so a warp shares its pair.
template <int N>
__global__ void __launch_bounds__(OPS_BS) operator_pair_kernel(GroupArgs g, int chunk) {
  const int S = g.S, np2 = 2 * g.npk;
  const long long L = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= (long long)g.K * np2 * S) return;
  const int s = (int)(L % S);
  const long long rest = L / S;
  const int slot = (int)(rest % np2), kk = (int)(rest / np2);
  if (g.sysidx[s] < 0) return;
  const long long istep = chunk_first_step(g, chunk, s) + kk;
  if (istep >= g.nsteps[s] || istep < 0) return;
  const uint64_t kick = g.kick;
  Rec cap{g.pcap + (size_t)kk * np2 * PCAP * S + s, S};
  Rec rec{g.steprec + (size_t)kk * g.R * S + s, S};
  const int roff = (kick ? op_size(N) : 0) + slot * PREC + (slot >= g.npk ? op_size(N) : 0);
  // A pair with G (m_i + m_j) == 0 keeps the jac_ij of the last pair of the
  // step that had mass (ahl21.jl:713 returns before refilling it); zero at the
  // start of the step (zero_out!, ahl21.jl:8).
  int q = slot;
  while (q >= 0 && cap.get(q * PCAP + 6 + 15) == 0.0) q--;
  if (q < 0) {
    for (int e = 0; e < PREC; e++) rec.put(roff + e, 0.0);
    return;
  }
  int i, j;
  pair_of_slot<N>(q, g.npk, kick, &i, &j);
  const double mi = g.m[i * S + s], mj = g.m[j * S + s];
  if (q < g.npk) pair_record_from_capture<true>(cap, q * PCAP, mi, mj, rec, roff);
  else pair_record_from_capture<false>(cap, q * PCAP, mi, mj, rec, roff);
}

// Corrector (and kick) records of one chunk: one lane per (step, system).
template <int N>
__global__ void __launch_bounds__(OPS_BS) operator_phi_kernel(GroupArgs g, int chunk) {
  const int S = g.S;
  const long long L = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= (long long)g.K * S) return;
  const int s = (int)(L % S), kk = (int)(L / S);
  if (g.sysidx[s] < 0) return;
  const long long istep = chunk_first_step(g, chunk, s) + kk;
  if (istep >= g.nsteps[s] || istep < 0) return;
  const uint64_t kick = g.kick;
  const double h = step_length(g, s, istep, g.nsteps[s], g.h[s]);
  Rec xs{g.xsnap + (size_t)kk * snap_count(kick != 0) * 3 * N * S + s, S};
  Rec rec{g.steprec + (size_t)kk * g.R * S + s, S};
  Sys<N> st;
  Work<N> w;
  for (int q = 0; q < N; q++) st.m[q] = g.m[q * S + s];
  for (int q = 0; q < 3 * N; q++) st.x[q] = xs.get(q), st.v[q] = st.xe[q] = st.ve[q] = 0.0;
  phic<N, true>(st, w, h, kick);
  phisalpha<N, true>(st, w, h, 2.0, kick);
  const int off_phi = (kick ? op_size(N) : 0) + g.npk * PREC;
  put_op(rec, off_phi, w.op, op_size(N));
  if (kick) {
    const double h6 = h / 6.0;
    for (int q = 0; q < 3 * N; q++) st.x[q] = xs.get(3 * N + q);
    kickfast<N, true>(st, w, h6, kick);
    put_op(rec, 0, w.op, op_size(N));
    for (int q = 0; q < 3 * N; q++) st.x[q] = xs.get(6 * N + q);
    kickfast<N, true>(st, w, h6, kick);
    put_op(rec, off_phi + op_size(N) + g.npk * PREC, w.op, op_size(N));
  }
}

// Jacobian consumer for one chunk of K steps (one lane per column).
template <int N>
__global__ void __launch_bounds__(CONS_BS) jacobian_chunk_kernel(GroupArgs g, int chunk) {
  extern __shared__ double smem[];
  constexpr int M = 7 * N, R6 = 6 * N;
  const int f = blockIdx.x * CONS_BS + threadIdx.x;
  const int s = f / M, c = f % M;
  if (s >= g.S || g.sysidx[s] < 0) return;
  const int S = g.S;
  const long long nst = g.nsteps[s];
  const long long k0 = chunk_first_step(g, chunk, s);
  if (k0 >= nst || k0 < 0) return;  // done, or admitted for a later chunk
  double* J = smem + threadIdx.x;
  double* E = smem + R6 * CONS_BS + threadIdx.x;
  const double* Jg = g.Jint + (size_t)s * R6 * M + c;
  const double* Eg = g.Eint + (size_t)s * R6 * M + c;
  for (int r = 0; r < R6; r++) {
    J[r * CONS_BS] = Jg[(size_t)r * M];
    E[r * CONS_BS] = Eg[(size_t)r * M];
  }
  const double h = g.h[s];
  const int ntt = g.ntt[s], ti = g.ti[s];
  const int gsys = g.sysidx[s];
  const uint64_t kick = g.kick;
  const int cb = c / 7, ck = c % 7;  // column c is d/d q0[ck] of body cb
  for (int kk = 0; kk < g.K; kk++) {
    const long long istep = k0 + kk;
    if (istep >= nst) break;
    Rec rec{g.steprec + (size_t)kk * g.R * S + s, S};
    if (g.trajJ) {  // column c of jac_step at the start of the step; mass rows are unit rows
      double* rj = g.trajJ + (((size_t)s * g.K + kk) * M + c) * M;
      for (int r = 0; r < M; r++) rj[r] = (r % 7 == 6) ? ((r == c) ? 1.0 : 0.0) : J[(6 * (r / 7) + r % 7) * CONS_BS];
    }
    apply_step<N, CONS_BS>(J, E, c, step_length(g, s, istep, nst, h), kick, rec);
    if (g.notransit) continue;
    for (int o = 0; o < N - 1; o++) {
      const int flag = g.tflag[(size_t)(kk * (N - 1) + o) * S + s];
      if (flag < 0) continue;
      const double* tr = g.trec + ((size_t)(kk * (N - 1) + o) * trec_size(N, g.tbv)) * S + s;
      const int ib = (o < ti) ? o : o + 1;
      if (!g.tbv) {
        double acc = 0.0;
        for (int b = 0; b < N; b++)
          for (int r = 0; r < 6; r++) {
            const double ur = tr[(size_t)(7 * b + r) * S];
            acc = fma(ur, J[(6 * b + r) * CONS_BS], acc);
            acc = fma(ur, E[(6 * b + r) * CONS_BS], acc);
          }
        if (ck == 6) acc = acc + tr[(size_t)c * S];  // unit mass row of this column
        const double gd = tr[(size_t)(7 * N) * S];
        g.dtdq0[g.off_dq[gsys] + ib + (long long)N * (flag + (long long)ntt * (ck + 7LL * cb))] = -acc / gd;
      } else {
        double acc[3] = {0.0, 0.0, 0.0};
        for (int b = 0; b < N; b++)
          for (int r = 0; r < 6; r++) {
            const double jv = J[(6 * b + r) * CONS_BS], ev = E[(6 * b + r) * CONS_BS];
            for (int w = 0; w < 3; w++) {
              const double ur = tr[(size_t)(7 * N * w + 7 * b + r) * S];
              acc[w] = fma(ur, jv, acc[w]);
              acc[w] = fma(ur, ev, acc[w]);
            }
          }
        if (ck == 6)
          for (int w = 0; w < 3; w++) acc[w] = acc[w] + tr[(size_t)(7 * N * w + c) * S];
        const double gd = tr[(size_t)(21 * N) * S], vsky = tr[(size_t)(21 * N + 1) * S];
        const double dvdt = tr[(size_t)(21 * N + 2) * S];
        const double d1 = -acc[0] / gd;
        double* out = g.dtdq0 + g.off_dq[gsys] + 3 * (ib + (long long)N * (flag + (long long)ntt * (ck + 7LL * cb)));
        out[0] = d1;
        out[1] = acc[1] / vsky + dvdt * d1;
        out[2] = 2.0 * acc[2];
      }
    }
  }
  double* Jw = g.Jint + (size_t)s * R6 * M + c;
  double* Ew = g.Eint + (size_t)s * R6 * M + c;
  bool finite = true;
  for (int r = 0; r < R6; r++) {
    Jw[(size_t)r * M] = J[r * CONS_BS];
    Ew[(size_t)r * M] = E[r * CONS_BS];
    finite = finite && isfinite(J[r * CONS_BS]);
  }
  if (!finite) atomicOr(g.status + s, NBG_STATUS_NONFINITE);
}

// gsave[i] = g!(i, ti, x, v) for every occultor (Transits.jl:146-149).
template <int N>
__global__ void seed_gsave_kernel(GroupArgs g) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= g.S || g.sysidx[s] < 0) return;
  const int S = g.S, ti = g.ti[s];
  for (int i = 0; i < N; i++) {
    if (i == ti) continue;
    const double dx = g.x[(3 * ti) * S + s] - g.x[(3 * i) * S + s];
    const double dy = g.x[(3 * ti + 1) * S + s] - g.x[(3 * i + 1) * S + s];
    const double dvx = g.v[(3 * ti) * S + s] - g.v[(3 * i) * S + s];
    const double dvy = g.v[(3 * ti + 1) * S + s] - g.v[(3 * i + 1) * S + s];
    g.gsave[i * S + s] = dx * dvx + dy * dvy;
  }
}

// Dynamic shared memory above the default 48 KB must be allowed per kernel.
template <class K>
inline void allow_smem(K kernel, int bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

template <int N>
int launch_orbit(const GroupArgs& g, int chunk, cudaStream_t st) {
  const int W = g.pwarps > 0 ? g.pwarps : 1;
  if (g.wide && !g.kick) {
    constexpr int T = PROD_BS / (2 * team_lanes(N));
    const int smem = std::max(team_smem_bytes<N, 2>(W), g.prod_smem);
    allow_smem(orbit_team_kernel<N, 2>, smem);
    orbit_team_kernel<N, 2><<<(g.S + W * T - 1) / (W * T), PROD_BS * W, smem, st>>>(g, chunk);
    return 0;
  }
  if (g.team && !g.kick) {
    constexpr int T = PROD_BS / team_lanes(N);
    const int smem = std::max(team_smem_bytes<N>(W), g.prod_smem);
    allow_smem(orbit_team_kernel<N>, smem);
    orbit_team_kernel<N><<<(g.S + W * T - 1) / (W * T), PROD_BS * W, smem, st>>>(g, chunk);
    return 0;
  }
  const int blocks = (g.S + W * g.spw - 1) / (W * g.spw);
  allow_smem(orbit_chunk_kernel<N>, g.prod_smem);
  orbit_chunk_kernel<N><<<blocks, PROD_BS * W, g.prod_smem, st>>>(g, chunk);
  return 0;
}

template <int N>
int launch_jac(const GroupArgs& g, int chunk, cudaStream_t st) {
  long long threads = (long long)g.S * 7 * N;
  int blocks = (int)((threads + CONS_BS - 1) / CONS_BS);
  const int smem = 2 * 6 * N * CONS_BS * (int)sizeof(double);
  allow_smem(jacobian_chunk_kernel<N>, smem);  // per call: the attribute belongs to the current device
  jacobian_chunk_kernel<N><<<blocks, CONS_BS, smem, st>>>(g, chunk);
  return 0;
}

template <int N>
int launch_transit(const GroupArgs& g, int chunk, cudaStream_t st) {
  if (team_lanes(N) > 1 && g.team && g.search_team && !g.kick) {
    const int smem = std::max(search_team_smem_bytes<N>(), g.guard_smem);
    allow_smem(transit_team_kernel<N>, smem);
    transit_team_kernel<N><<<g.tgrid / TRANSIT_BS, TRANSIT_BS, smem, st>>>(g, chunk);
    return 0;
  }
  allow_smem(transit_kernel<N>, g.guard_smem);
  transit_kernel<N><<<g.tgrid / TRANSIT_BS, TRANSIT_BS, g.guard_smem, st>>>(g, chunk);
  return 0;
}

template <int N>
int launch_operators(const GroupArgs& g, int chunk, cudaStream_t st) {
  long long lanes = (long long)g.K * 2 * g.npk * g.S;
  allow_smem(operator_pair_kernel<N>, g.guard_smem);
  allow_smem(operator_phi_kernel<N>, g.guard_smem);
  if (lanes > 0)
    operator_pair_kernel<N><<<(unsigned)((lanes + OPS_BS - 1) / OPS_BS), OPS_BS, g.guard_smem, st>>>(g, chunk);
  lanes = (long long)g.K * g.S;
  operator_phi_kernel<N><<<(unsigned)((lanes + OPS_BS - 1) / OPS_BS), OPS_BS, g.guard_smem, st>>>(g, chunk);
  return 0;
}

template <int N>
int launch_seed(const GroupArgs& g, cudaStream_t st) {
  int b = (g.S + 127) / 128;
  seed_gsave_kernel<N><<<b, 128, 0, st>>>(g);
  return 0;
}

}  // namespace nbg
