// nbg_orbit_team.cuh -- the orbit producer with a team of lanes per system.
//
// The Kepler sweeps of an AHL21 step (ahl21.jl:25-27 forward, :56-58
// backward) update bodies i and j of each pair in a fixed order.  A pair's
// update reads and writes only x, v (and their Kahan errors) of its two
// bodies, so two pairs with no body in common commute exactly.  In the
// forward order (i = 0..N-2, j = i+1..N-1), the pairs that touch body b come
// in order of increasing i + j: (0,b), (1,b), ..., (b-1,b), (b,b+1), ...,
// (b,N-1).  The pairs with one value of i + j share no body.  Running the
// sweep "level by level" in increasing i + j, with the pairs of one level
// in parallel, therefore applies to every body the same updates in the same
// order as the sequential sweep: the result is bitwise identical.  The
// backward sweep is the exact reverse sequence, so it runs the levels in
// decreasing i + j.  phisalpha!'s two pair loops (the acceleration sums and
// the velocity kicks, ahl21.jl:558-700 without the gradient) follow the same
// pair order and run level by level too.
//
// A level holds at most floor(N/2) pairs, so a team of L = max(1, N/2) lanes
// runs one system, 32 / L systems per warp, the system's x, v, errors and
// masses in shared memory.  The critical path of a sweep drops from
// N(N-1)/2 to 2N-3 pair solves (N = 10: 45 -> 17; N = 8: 28 -> 13).
//
// Groups with kick pairs (pair[i,j] == true) keep the one-lane producer.
// The last step of a grad system (which also forms dq/dt, the State's
// output) runs the one-lane step on the team's first lane.
#pragma once
#include "nbg_orbit.cuh"

namespace nbg {

__host__ __device__ constexpr int team_lanes(int N) { return N / 2 > 1 ? N / 2 : 1; }

// phisalpha!, first pair loop (accelerations), for one pair; the same
// operations in the same order as phisalpha<N, false>.
template <int N>
__device__ __forceinline__ void phis_accel_pair(const Sys<N>& s, double* a, int i, int j) {
  double rij[3];
  for (int k = 0; k < 3; k++) rij[k] = s.x[3 * i + k] - s.x[3 * j + k];
  double r2 = rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2];
  double r3 = r2 * sqrt(r2);
  double fac2 = GNEWT / r3;
  for (int k = 0; k < 3; k++) {
    double fac = fac2 * rij[k];
    a[3 * i + k] = a[3 * i + k] - s.m[j] * fac;
    a[3 * j + k] = a[3 * j + k] + s.m[i] * fac;
  }
}

// phisalpha!, second pair loop (velocity corrections), for one pair.
template <int N>
__device__ __forceinline__ void phis_kick_pair(Sys<N>& s, const double* a, int i, int j, double coeff) {
  double rij[3], aij[3];
  for (int k = 0; k < 3; k++) {
    aij[k] = a[3 * i + k] - a[3 * j + k];
    rij[k] = s.x[3 * i + k] - s.x[3 * j + k];
  }
  double r2 = rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2];
  double r1 = sqrt(r2);
  double ardot = aij[0] * rij[0] + aij[1] * rij[1] + aij[2] * rij[2];
  double fac1 = coeff / (r2 * r2 * r1);
  double mij = s.m[i] + s.m[j];
  double fac2 = 2.0 * GNEWT * mij / r1 + 3.0 * ardot;
  for (int k = 0; k < 3; k++) {
    double fac = fac1 * (rij[k] * fac2 - r2 * aij[k]);
    kahan(s.v[3 * i + k], s.ve[3 * i + k], s.m[j] * fac);
    kahan(s.v[3 * j + k], s.ve[3 * j + k], (-s.m[i]) * fac);
  }
}

// The pair of level `lev` (i + j == lev) that lane t of a team takes, if any.
template <int N>
__device__ __forceinline__ bool level_pair(int lev, int t, int* i, int* j) {
  const int imin = lev - (N - 1) > 0 ? lev - (N - 1) : 0;
  const int ii = imin + t;
  if (2 * ii >= lev) return false;  // i < j = lev - i
  *i = ii;
  *j = lev - ii;
  return true;
}

// kepler_pair<N, DRIFT_FIRST, false, false> on the two lanes of a pair slot
// (kep_delxv2): both lanes read the pair's coordinates and solve it; role 0
// then updates body i and writes the first half of the capture, role 1 body
// j and the rest.  x_i and x_j are separate variables, so splitting their
// updates between the lanes changes no value.
template <int N, bool DRIFT_FIRST>
__device__ __forceinline__ void kepler_pair_w2(Sys<N>& s, int i, int j, double h2, const Rec& cap, int coff,
                                               int role, unsigned mask, int base) {
  double x0[3], v0[3];
  for (int k = 0; k < 3; k++) {
    x0[k] = s.x[3 * i + k] - s.x[3 * j + k];
    v0[k] = s.v[3 * i + k] - s.v[3 * j + k];
  }
  const double gm = GNEWT * (s.m[i] + s.m[j]);
  __syncwarp(mask);  // both lanes have read the pair before either writes
  if (cap.p && gm == 0.0 && role == 0) cap.put(coff + 6 + 15, 0.0);
  if (gm != 0.0) {
    KepParams P;
    double delxv[6];
    kep_delxv2<DRIFT_FIRST>(x0, v0, gm, h2, delxv, P, role, mask, base);
    if (cap.p) {
      const double pv[22] = {P.gamma, P.g0, P.g1, P.g2, P.g3, P.h1, P.h2, P.dfdt, P.fm1, P.gmh, P.dgdtm1,
                             P.r0, P.r, P.r0inv, P.rinv, P.k, P.h, P.beta, P.betainv, P.eta, P.sqb, P.zeta};
      if (role == 0) {
        for (int q = 0; q < 3; q++) {
          cap.put(coff + q, x0[q]);
          cap.put(coff + 3 + q, v0[q]);
        }
        for (int q = 0; q < 8; q++) cap.put(coff + 6 + q, pv[q]);
      } else {
        for (int q = 8; q < 22; q++) cap.put(coff + 6 + q, pv[q]);
      }
    }
    const double mijinv = 1.0 / (s.m[i] + s.m[j]);
    const double mi = s.m[i] * mijinv, mj = s.m[j] * mijinv;
    const int b = role ? j : i;
    const double f = role ? (-mi) : mj;
    for (int k = 0; k < 3; k++) kahan(s.x[3 * b + k], s.xe[3 * b + k], f * delxv[k]);
    for (int k = 0; k < 3; k++) kahan(s.v[3 * b + k], s.ve[3 * b + k], f * delxv[3 + k]);
  }
}

// One AHL21 step without gradient operators for a group with no kick pairs
// (ahl21_no_grad.jl:6-18 order), run by the R * L lanes of a team (R = 2:
// each pair slot p on two lanes, roles 0 and 1, kepler_pair_w2); `run` is
// false for lanes whose system does not step (they still meet every
// __syncwarp).  cap / xs as in ahl21_step.  a: the team's 3N acceleration
// scratch.
template <int N, int R = 1>
__device__ __forceinline__ void team_step(Sys<N>& s, double* a, Work<N>& w, int t, bool run, double h,
                                          const Rec& cap, const Rec& xs) {
  constexpr int L = R * team_lanes(N);
  constexpr int P = N * (N - 1) / 2;
  const int p = t / R, role = t % R;
  const int lane = threadIdx.x & 31;
  const int base = lane - role;
  const unsigned mask = (R == 2) ? (3u << base) : 0u;
  const double h2 = 0.5 * h;
  if (run)
    for (int q = t; q < 3 * N; q += L) kahan(s.x[q], s.xe[q], h2 * s.v[q]);
  __syncwarp();
  for (int lev = 1; lev <= 2 * N - 3; lev++) {
    int i, j;
    if (run && level_pair<N>(lev, p, &i, &j)) {
      if (R == 1) kepler_pair<N, true, false, false>(s, w, i, j, h2, Rec{nullptr, 0}, 0, cap, pair_bit(i, j, N) * PCAP);
      else kepler_pair_w2<N, true>(s, i, j, h2, cap, pair_bit(i, j, N) * PCAP, role, mask, base);
    }
    __syncwarp();
  }
  if (run) {
    if (xs.p)
      for (int q = t; q < 3 * N; q += L) xs.put(q, s.x[q]);
    for (int q = t; q < 3 * N; q += L) a[q] = 0.0;
  }
  __syncwarp();
  const double coeff = 2.0 * (h * h * h) / 96.0 * 2.0 * GNEWT;  // alpha = 2 (ahl21.jl:47)
  for (int lev = 1; lev <= 2 * N - 3; lev++) {
    int i, j;
    if (run && role == 0 && level_pair<N>(lev, p, &i, &j)) phis_accel_pair<N>(s, a, i, j);
    __syncwarp();
  }
  for (int lev = 1; lev <= 2 * N - 3; lev++) {
    int i, j;
    if (run && role == 0 && level_pair<N>(lev, p, &i, &j)) phis_kick_pair<N>(s, a, i, j, coeff);
    __syncwarp();
  }
  for (int lev = 2 * N - 3; lev >= 1; lev--) {
    int i, j;
    if (run && level_pair<N>(lev, p, &i, &j)) {
      const int coff = (P + (P - 1 - pair_bit(i, j, N))) * PCAP;
      if (R == 1) kepler_pair<N, false, false, false>(s, w, i, j, h2, Rec{nullptr, 0}, 0, cap, coff);
      else kepler_pair_w2<N, false>(s, i, j, h2, cap, coff, role, mask, base);
    }
    __syncwarp();
  }
  if (run)
    for (int q = t; q < 3 * N; q += L) kahan(s.x[q], s.xe[q], h2 * s.v[q]);
  __syncwarp();
}

// Dynamic shared memory the team producer needs for W warps per block:
// per team a Sys<N>, 3N accelerations, N g values and N transit counts.
template <int N, int R = 1>
__host__ __device__ constexpr int team_smem_bytes(int W) {
  return W * (PROD_BS / (R * team_lanes(N))) *
         (int)(sizeof(Sys<N>) + (3 * N + N) * sizeof(double) + N * sizeof(long long));
}

// Orbit producer, team form: L = R * team_lanes(N) lanes per system
// (R = 2: the wide form, two lanes per pair solve), T = 32 / L systems per
// warp (lanes beyond T * L idle), pwarps independent warps per block.  Same
// inputs, outputs and arithmetic as orbit_chunk_kernel<N> for groups
// without kick pairs.
template <int N, int R = 1>
__global__ void __launch_bounds__(PROD_BS * PROD_MAX_WARPS) orbit_team_kernel(GroupArgs g, int chunk) {
  constexpr int L = R * team_lanes(N);
  constexpr int T = PROD_BS / L;
  const int W = g.pwarps > 0 ? g.pwarps : 1;
  extern __shared__ double team_smem[];
  Sys<N>* sys = reinterpret_cast<Sys<N>*>(team_smem);
  double(*acc)[3 * N] = reinterpret_cast<double(*)[3 * N]>(sys + W * T);
  double(*gsv)[N] = reinterpret_cast<double(*)[N]>(acc + W * T);
  long long(*cnt)[N] = reinterpret_cast<long long(*)[N]>(gsv + W * T);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int team = lane / L, t = lane % L;
  const bool in_team = team < T;
  const int tm = warp * T + (in_team ? team : 0);  // idle lanes alias their warp's team 0 but never write
  const int s = blockIdx.x * W * T + tm;
  const int S = g.S;
  bool valid = in_team && s < S && g.sysidx[s] >= 0;
  const long long nst = valid ? g.nsteps[s] : 0;
  const long long k0 = valid ? chunk_first_step(g, chunk, s) : 0;
  if (k0 >= nst || k0 < 0) valid = false;  // done, or admitted for a later chunk
  Sys<N>& st = sys[tm];
  if (valid) {
    for (int q = t; q < 3 * N; q += L) {
      st.x[q] = g.x[q * S + s];
      st.v[q] = g.v[q * S + s];
      st.xe[q] = g.xe[q * S + s];
      st.ve[q] = g.ve[q * S + s];
    }
    for (int q = t; q < N; q += L) {
      st.m[q] = g.m[q * S + s];
      gsv[tm][q] = g.gsave[q * S + s];
      cnt[tm][q] = g.count[q * S + s];
    }
    for (int q = t; q < 7 * N; q += L) st.dqdt[q] = g.dqdt[q * S + s];
  }
  __syncwarp();
  Work<N> w;
  const double t0 = valid ? g.t0[s] : 0.0, h = valid ? g.h[s] : 0.0, hI = valid ? g.hI[s] : 0.0;
  const int ntt = valid ? g.ntt[s] : 0, ti = valid ? g.ti[s] : 0;
  for (int kk = 0; kk < g.K; kk++) {
    const long long istep = k0 + kk;
    const bool run = valid && istep < nst;
    if (!__any_sync(0xffffffffu, run)) break;
    const bool last = run && g.grad && istep == nst - 1;
    Rec cap{nullptr, 0}, xs{nullptr, 0};
    if (g.grad) {
      cap = Rec{g.pcap + (size_t)kk * 2 * g.npk * PCAP * S + s, S};
      xs = Rec{g.xsnap + (size_t)kk * snap_count(false) * 3 * N * S + s, S};
    }
    const double hs = run ? step_length(g, s, istep, nst, h) : h;
    if (run && g.trajxv) {
      double* rx = g.trajxv + ((size_t)s * g.K + kk) * 6 * N;
      for (int q = t; q < 3 * N; q += L) {
        rx[q] = st.x[q];
        rx[3 * N + q] = st.v[q];
      }
    }
    team_step<N, R>(st, acc[tm], w, t, run && !last, hs, cap, xs);
    // the last step also forms dq/dt: the one-lane step, on the team's first lane
    if (last && t == 0) ahl21_step<N, true, true>(st, w, hs, 0, Rec{nullptr, 0}, cap, xs);
    __syncwarp();
    // detect_transits! (timing.jl:3-28); occultor o on lane o % L
    if (run && !g.notransit) {
      const double tnow = t0 + (double)(istep + 1) * h;
      for (int o = t; o < N - 1; o += L) {
        const int ib = (o < ti) ? o : o + 1;
        const double gi = gsky(st, ib, ti);
        const double xi = st.x[3 * ib], yi = st.x[3 * ib + 1], zi = st.x[3 * ib + 2];
        const double ri = sqrt(xi * xi + yi * yi + zi * zi);
        if (g.grad) g.tflag[(size_t)(kk * (N - 1) + o) * S + s] = -1;
        if (gi > 0.0 && gsv[tm][ib] < 0.0 && -zi > 0.25 * ri && ri < 1e12) {
          cnt[tm][ib] += 1;
          if (cnt[tm][ib] <= ntt) {
            const int idx = atomicAdd(g.task_count, 1);
            if (idx < g.task_cap) {
              double* tf = g.task_f + (size_t)idx * (12 * N + 2);
              for (int q = 0; q < 3 * N; q++) {
                tf[q] = st.x[q];
                tf[3 * N + q] = st.v[q];
                tf[6 * N + q] = st.xe[q];
                tf[9 * N + q] = st.ve[q];
              }
              tf[12 * N] = -gi * hI / (gi - gsv[tm][ib]);  // first estimate (timing.jl:20)
              tf[12 * N + 1] = tnow;
              int* tk = g.task_i + 3 * idx;
              tk[0] = s;
              tk[1] = kk * (N - 1) + o;
              tk[2] = (int)(cnt[tm][ib] - 1);
            }
          } else {
            atomicOr(g.status + s, NBG_STATUS_NTT_OVERFLOW);
          }
        }
        gsv[tm][ib] = gi;
      }
    }
    __syncwarp();
  }
  if (valid) {
    for (int q = t; q < 3 * N; q += L) {
      g.x[q * S + s] = st.x[q];
      g.v[q * S + s] = st.v[q];
      g.xe[q * S + s] = st.xe[q];
      g.ve[q * S + s] = st.ve[q];
    }
    if (g.grad && nst <= k0 + g.K)
      for (int q = t; q < 7 * N; q += L) g.dqdt[q * S + s] = st.dqdt[q];
    for (int q = t; q < N; q += L) {
      g.gsave[q * S + s] = gsv[tm][q];
      g.count[q * S + s] = cnt[tm][q];
    }
    if (t == 0 && !state_finite<N>(st)) atomicOr(g.status + s, NBG_STATUS_NONFINITE);
  }
}

}  // namespace nbg
