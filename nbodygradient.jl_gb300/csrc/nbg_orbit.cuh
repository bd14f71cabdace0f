// nbg_orbit.cuh -- the orbit producer: one GPU lane advances one system.
//
// Per AHL21 step (src/integrator/ahl21/ahl21.jl:5-95) the producer updates x,
// v (with their Kahan errors) and, when asked, dq/dt, exactly as the
// reference does, and emits the step's linear operators for the Jacobian
// consumer instead of applying them to jac_step itself:
//   * each Kepler pair (i, j): the 6x6 block K of jac_kepler, m_i/(m_i+m_j),
//     m_j/(m_i+m_j) and the two mass columns of jac_ij (62 doubles) -- the
//     14x14 jac_ij of ahl21.jl:734-750 is exactly these numbers;
//   * phic!/phisalpha! (ahl21.jl:392-700): jac_phi restricted to its only
//     non-zero block, velocity rows x (position, mass) columns (3N x 4N);
//   * kickfast! (ahl21.jl:337-386) for pair[i,j] == true: jac_kick on the
//     same block.
// The operators depend on x, v only, never on jac_step, so orbit and Jacobian
// are decoupled (the producer/consumer split of this package).
//
// Compact operator layout: row 3b + k is body b's velocity component k,
// column 4d + p is body d's position component p (p < 3) or mass (p == 3).
#pragma once
#include "nbg_layout.cuh"
#include "nbg_kepler.cuh"

namespace nbg {

// Record writer: element e of this lane's record at p[e * stride].
struct Rec {
  double* p;
  int stride;
  __device__ __forceinline__ void put(int e, double v) const {
    if (p) p[(size_t)e * stride] = v;
  }
  __device__ __forceinline__ double get(int e) const { return p[(size_t)e * stride]; }
};

template <int N>
struct Sys {
  double x[3 * N], v[3 * N], xe[3 * N], ve[3 * N], m[N];
  double dqdt[7 * N];
};

// x and v all finite (the State check of Integrator.jl:137-143, which the
// reference only prints; here it raises NBG_STATUS_NONFINITE).
template <int N>
__device__ __forceinline__ bool state_finite(const Sys<N>& st) {
  bool ok = true;
#pragma unroll
  for (int q = 0; q < 3 * N; q++) ok = ok && isfinite(st.x[q]) && isfinite(st.v[q]);
  return ok;
}

// Scratch of one step (the Derivatives fields the producer needs,
// src/PreAllocArrays.jl:65-113), compact layouts.
template <int N>
struct Work {
  double op[12 * N * N];    // jac_kick or jac_phi block
  double dadq[12 * N * N];  // d a / d (x, m), rows 3i+k, cols 4d+p
  double dot[4 * N];
  double a[3 * N];
  double dqop[3 * N];       // dqdt_kick or dqdt_phi velocity entries
  // last pair's jac_ij (factored) and dqdt_ij: stale values are reused when
  // G (m_i + m_j) == 0, as ahl21.jl:713 returns before refilling them.
  double lk[36], lmi, lmj, lmc6[12], lmc13[12], ldq[14];
};

#define OPX(r, c) w.op[(r) * (4 * N) + (c)]
#define DAX(r, c) w.dadq[(r) * (4 * N) + (c)]

template <int N>
__device__ __forceinline__ void reset_last(Work<N>& w) {
  for (int q = 0; q < 36; q++) w.lk[q] = 0.0;
  w.lmi = w.lmj = 0.0;
  for (int q = 0; q < 12; q++) w.lmc6[q] = w.lmc13[q] = 0.0;
  for (int q = 0; q < 14; q++) w.ldq[q] = 0.0;
}

// drift (ahl21.jl:318-331 for x; the jac_step part is the consumer's)
template <int N>
__device__ __forceinline__ void drift(Sys<N>& s, double h) {
#pragma unroll
  for (int q = 0; q < 3 * N; q++) kahan(s.x[q], s.xe[q], h * s.v[q]);
}

// kickfast! (ahl21.jl:337-386 / ahl21_no_grad.jl:35-56)
template <int N, bool GRADOPS>
__device__ void kickfast(Sys<N>& s, Work<N>& w, double h, uint64_t kick) {
  if (GRADOPS) {
    for (int q = 0; q < 12 * N * N; q++) w.op[q] = 0.0;
    for (int q = 0; q < 3 * N; q++) w.dqop[q] = 0.0;
  }
  for (int i = 0; i < N - 1; i++)
    for (int j = i + 1; j < N; j++) {
      if (!((kick >> pair_bit(i, j, N)) & 1)) continue;
      double rij[3];
      for (int k = 0; k < 3; k++) rij[k] = s.x[3 * i + k] - s.x[3 * j + k];
      double r2inv = 1.0 / (rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2]);
      double r3inv = r2inv * sqrt(r2inv);
      double fac2 = h * GNEWT * r3inv;
      for (int k = 0; k < 3; k++) {
        double fac = fac2 * rij[k];
        kahan(s.v[3 * i + k], s.ve[3 * i + k], (-s.m[j]) * fac);
        kahan(s.v[3 * j + k], s.ve[3 * j + k], s.m[i] * fac);
        if (GRADOPS) {
          w.dqop[3 * i + k] = w.dqop[3 * i + k] - s.m[j] * fac / h;
          w.dqop[3 * j + k] = w.dqop[3 * j + k] + s.m[i] * fac / h;
          OPX(3 * i + k, 4 * j + 3) -= fac;
          OPX(3 * j + k, 4 * i + 3) += fac;
          fac = fac * (3.0 * r2inv);
          for (int p = 0; p < 3; p++) {
            OPX(3 * i + k, 4 * i + p) += fac * s.m[j] * rij[p];
            OPX(3 * i + k, 4 * j + p) -= fac * s.m[j] * rij[p];
            OPX(3 * j + k, 4 * j + p) += fac * s.m[i] * rij[p];
            OPX(3 * j + k, 4 * i + p) -= fac * s.m[i] * rij[p];
          }
          OPX(3 * i + k, 4 * i + k) -= fac2 * s.m[j];
          OPX(3 * i + k, 4 * j + k) += fac2 * s.m[j];
          OPX(3 * j + k, 4 * j + k) -= fac2 * s.m[i];
          OPX(3 * j + k, 4 * i + k) += fac2 * s.m[i];
        }
      }
    }
}

// dqdt += dqop/div + op * dqdt (ahl21.jl:11-14, :51-52, :86-89); the gemv
// is one FMA chain per row in the reference's column order; columns with a
// zero operator entry or a zero dq/dt entry (velocity and mass columns) are
// exact no-ops of that chain and are skipped.
template <int N>
__device__ __forceinline__ void dqdt_op(Sys<N>& s, Work<N>& w, double div) {
  for (int b = 0; b < N; b++)
    for (int k = 0; k < 3; k++) {
      int vr = 3 * b + k;
      double acc = 0.0;
      for (int d = 0; d < N; d++)
        for (int p = 0; p < 3; p++) acc = fma(OPX(vr, 4 * d + p), s.dqdt[7 * d + p], acc);
      double dq = (div != 1.0) ? w.dqop[vr] / div : w.dqop[vr];
      s.dqdt[7 * b + 3 + k] = s.dqdt[7 * b + 3 + k] + (dq + acc);
    }
}

__device__ __forceinline__ void put_op(const Rec& rec, int off, const double* op, int n) {
  for (int q = 0; q < n; q++) rec.put(off + q, op[q]);
}

// phic! (ahl21.jl:392-552 / ahl21_no_grad.jl:62-104): corrector for kick pairs
template <int N, bool GRADOPS>
__device__ void phic(Sys<N>& s, Work<N>& w, double h, uint64_t kick) {
  for (int q = 0; q < 3 * N; q++) w.a[q] = 0.0;
  if (GRADOPS) {
    for (int q = 0; q < 12 * N * N; q++) { w.dadq[q] = 0.0; w.op[q] = 0.0; }
    for (int q = 0; q < 3 * N; q++) w.dqop[q] = 0.0;
  }
  if (!kick) return;
  double coeff = h * h * h / 36.0 * GNEWT;
  for (int i = 0; i < N - 1; i++)
    for (int j = i + 1; j < N; j++) {
      if (!((kick >> pair_bit(i, j, N)) & 1)) continue;
      double rij[3];
      for (int k = 0; k < 3; k++) rij[k] = s.x[3 * i + k] - s.x[3 * j + k];
      double r2inv = 1.0 / (rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2]);
      double r3inv = r2inv * sqrt(r2inv);
      for (int k = 0; k < 3; k++) {
        double fac = GNEWT * rij[k] * r3inv;
        double facv = fac * 2.0 * h / 3.0;
        kahan(s.v[3 * i + k], s.ve[3 * i + k], (-s.m[j]) * facv);
        kahan(s.v[3 * j + k], s.ve[3 * j + k], s.m[i] * facv);
        w.a[3 * i + k] = w.a[3 * i + k] - s.m[j] * fac;
        w.a[3 * j + k] = w.a[3 * j + k] + s.m[i] * fac;
        if (GRADOPS) {
          w.dqop[3 * i + k] = w.dqop[3 * i + k] - 1.0 / h * s.m[j] * facv;
          w.dqop[3 * j + k] = w.dqop[3 * j + k] + 1.0 / h * s.m[i] * facv;
          OPX(3 * i + k, 4 * j + 3) -= facv;
          OPX(3 * j + k, 4 * i + 3) += facv;
          facv = facv * (3.0 * r2inv);
          for (int p = 0; p < 3; p++) {
            OPX(3 * i + k, 4 * i + p) += facv * s.m[j] * rij[p];
            OPX(3 * i + k, 4 * j + p) -= facv * s.m[j] * rij[p];
            OPX(3 * j + k, 4 * j + p) += facv * s.m[i] * rij[p];
            OPX(3 * j + k, 4 * i + p) -= facv * s.m[i] * rij[p];
          }
          facv = 2.0 * h / 3.0 * GNEWT * r3inv;
          OPX(3 * i + k, 4 * i + k) -= facv * s.m[j];
          OPX(3 * i + k, 4 * j + k) += facv * s.m[j];
          OPX(3 * j + k, 4 * j + k) -= facv * s.m[i];
          OPX(3 * j + k, 4 * i + k) += facv * s.m[i];
          DAX(3 * i + k, 4 * j + 3) -= fac;
          DAX(3 * j + k, 4 * i + 3) += fac;
          fac = fac * (3.0 * r2inv);
          for (int p = 0; p < 3; p++) {
            DAX(3 * i + k, 4 * i + p) += fac * s.m[j] * rij[p];
            DAX(3 * i + k, 4 * j + p) -= fac * s.m[j] * rij[p];
            DAX(3 * j + k, 4 * j + p) += fac * s.m[i] * rij[p];
            DAX(3 * j + k, 4 * i + p) -= fac * s.m[i] * rij[p];
          }
          fac = GNEWT * r3inv;
          DAX(3 * i + k, 4 * i + k) -= fac * s.m[j];
          DAX(3 * i + k, 4 * j + k) += fac * s.m[j];
          DAX(3 * j + k, 4 * j + k) -= fac * s.m[i];
          DAX(3 * j + k, 4 * i + k) += fac * s.m[i];
        }
      }
    }
  for (int i = 0; i < N - 1; i++)
    for (int j = i + 1; j < N; j++) {
      if (!((kick >> pair_bit(i, j, N)) & 1)) continue;
      double rij[3], aij[3];
      for (int k = 0; k < 3; k++) {
        aij[k] = w.a[3 * i + k] - w.a[3 * j + k];
        rij[k] = s.x[3 * i + k] - s.x[3 * j + k];
      }
      if (GRADOPS) {
        for (int q = 0; q < 4 * N; q++) w.dot[q] = 0.0;
        for (int di = 0; di < N; di++)
          for (int p = 0; p < 4; p++)
            for (int k = 0; k < 3; k++)
              w.dot[4 * di + p] += rij[k] * (DAX(3 * i + k, 4 * di + p) - DAX(3 * j + k, 4 * di + p));
      }
      double r2 = rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2];
      double r1 = sqrt(r2);
      double ardot = aij[0] * rij[0] + aij[1] * rij[1] + aij[2] * rij[2];
      double fac1 = coeff / (r2 * r2 * r1);
      double fac2 = 3.0 * ardot;
      for (int k = 0; k < 3; k++) {
        double fac = fac1 * (rij[k] * fac2 - r2 * aij[k]);
        kahan(s.v[3 * i + k], s.ve[3 * i + k], s.m[j] * fac);
        kahan(s.v[3 * j + k], s.ve[3 * j + k], (-s.m[i]) * fac);
        if (GRADOPS) {
          w.dqop[3 * i + k] = w.dqop[3 * i + k] + 3.0 / h * s.m[j] * fac;
          w.dqop[3 * j + k] = w.dqop[3 * j + k] - 3.0 / h * s.m[i] * fac;
          OPX(3 * i + k, 4 * j + 3) += fac;
          OPX(3 * j + k, 4 * i + 3) -= fac;
          fac = fac * (5.0 / r2);
          for (int p = 0; p < 3; p++) {
            OPX(3 * i + k, 4 * i + p) -= fac * s.m[j] * rij[p];
            OPX(3 * i + k, 4 * j + p) += fac * s.m[j] * rij[p];
            OPX(3 * j + k, 4 * j + p) -= fac * s.m[i] * rij[p];
            OPX(3 * j + k, 4 * i + p) += fac * s.m[i] * rij[p];
          }
          fac = fac1 * fac2;
          OPX(3 * i + k, 4 * i + k) += fac * s.m[j];
          OPX(3 * i + k, 4 * j + k) -= fac * s.m[j];
          OPX(3 * j + k, 4 * j + k) += fac * s.m[i];
          OPX(3 * j + k, 4 * i + k) -= fac * s.m[i];
          fac = -2.0 * fac1 * aij[k];
          for (int p = 0; p < 3; p++) {
            double fac3 = fac * rij[p] + fac1 * 3.0 * rij[k] * aij[p];
            OPX(3 * i + k, 4 * i + p) += s.m[j] * fac3;
            OPX(3 * i + k, 4 * j + p) -= s.m[j] * fac3;
            OPX(3 * j + k, 4 * j + p) += s.m[i] * fac3;
            OPX(3 * j + k, 4 * i + p) -= s.m[i] * fac3;
          }
          fac = (-fac1) * r2;
          for (int di = 0; di < N; di++) {
            for (int p = 0; p < 3; p++) {
              OPX(3 * i + k, 4 * di + p) += fac * s.m[j] * (DAX(3 * i + k, 4 * di + p) - DAX(3 * j + k, 4 * di + p));
              OPX(3 * j + k, 4 * di + p) -= fac * s.m[i] * (DAX(3 * i + k, 4 * di + p) - DAX(3 * j + k, 4 * di + p));
            }
            OPX(3 * i + k, 4 * di + 3) += fac * s.m[j] * (DAX(3 * i + k, 4 * di + 3) - DAX(3 * j + k, 4 * di + 3));
            OPX(3 * j + k, 4 * di + 3) -= fac * s.m[i] * (DAX(3 * i + k, 4 * di + 3) - DAX(3 * j + k, 4 * di + 3));
          }
          fac = 3.0 * fac1 * rij[k];
          for (int di = 0; di < N; di++) {
            for (int p = 0; p < 3; p++) {
              OPX(3 * i + k, 4 * di + p) += fac * s.m[j] * w.dot[4 * di + p];
              OPX(3 * j + k, 4 * di + p) -= fac * s.m[i] * w.dot[4 * di + p];
            }
            OPX(3 * i + k, 4 * di + 3) += fac * s.m[j] * w.dot[4 * di + 3];
            OPX(3 * j + k, 4 * di + 3) -= fac * s.m[i] * w.dot[4 * di + 3];
          }
        }
      }
    }
}

// phisalpha! (ahl21.jl:558-700 / ahl21_no_grad.jl:110-158) for Kepler pairs.
// Accumulates onto the phic! operator (jac_phi is not cleared in between).
template <int N, bool GRADOPS>
__device__ void phisalpha(Sys<N>& s, Work<N>& w, double h, double alpha, uint64_t kick) {
  for (int q = 0; q < 3 * N; q++) w.a[q] = 0.0;
  if (GRADOPS)
    for (int q = 0; q < 12 * N * N; q++) w.dadq[q] = 0.0;
  double coeff = alpha * (h * h * h) / 96.0 * 2.0 * GNEWT;
  for (int i = 0; i < N - 1; i++)
    for (int j = i + 1; j < N; j++) {
      if ((kick >> pair_bit(i, j, N)) & 1) continue;
      double rij[3];
      for (int k = 0; k < 3; k++) rij[k] = s.x[3 * i + k] - s.x[3 * j + k];
      double r2 = rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2];
      double r3 = r2 * sqrt(r2);
      double fac2 = GNEWT / r3;
      for (int k = 0; k < 3; k++) {
        double fac = fac2 * rij[k];
        w.a[3 * i + k] = w.a[3 * i + k] - s.m[j] * fac;
        w.a[3 * j + k] = w.a[3 * j + k] + s.m[i] * fac;
        if (GRADOPS) {
          DAX(3 * i + k, 4 * j + 3) -= fac;
          DAX(3 * j + k, 4 * i + 3) += fac;
          fac = fac * (3.0 / r2);
          for (int p = 0; p < 3; p++) {
            DAX(3 * i + k, 4 * i + p) += fac * s.m[j] * rij[p];
            DAX(3 * i + k, 4 * j + p) -= fac * s.m[j] * rij[p];
            DAX(3 * j + k, 4 * j + p) += fac * s.m[i] * rij[p];
            DAX(3 * j + k, 4 * i + p) -= fac * s.m[i] * rij[p];
          }
          DAX(3 * i + k, 4 * i + k) -= fac2 * s.m[j];
          DAX(3 * i + k, 4 * j + k) += fac2 * s.m[j];
          DAX(3 * j + k, 4 * j + k) -= fac2 * s.m[i];
          DAX(3 * j + k, 4 * i + k) += fac2 * s.m[i];
        }
      }
    }
  for (int i = 0; i < N - 1; i++)
    for (int j = i + 1; j < N; j++) {
      if ((kick >> pair_bit(i, j, N)) & 1) continue;
      double rij[3], aij[3];
      for (int k = 0; k < 3; k++) {
        aij[k] = w.a[3 * i + k] - w.a[3 * j + k];
        rij[k] = s.x[3 * i + k] - s.x[3 * j + k];
      }
      if (GRADOPS) {
        for (int q = 0; q < 4 * N; q++) w.dot[q] = 0.0;
        for (int di = 0; di < N; di++)
          for (int p = 0; p < 4; p++)
            for (int k = 0; k < 3; k++)
              w.dot[4 * di + p] += rij[k] * (DAX(3 * i + k, 4 * di + p) - DAX(3 * j + k, 4 * di + p));
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
        if (GRADOPS) {
          w.dqop[3 * i + k] = w.dqop[3 * i + k] + 3.0 / h * s.m[j] * fac;
          w.dqop[3 * j + k] = w.dqop[3 * j + k] - 3.0 / h * s.m[i] * fac;
          OPX(3 * i + k, 4 * j + 3) += fac;
          OPX(3 * j + k, 4 * i + 3) -= fac;
          fac = fac * (5.0 / r2);
          for (int p = 0; p < 3; p++) {
            OPX(3 * i + k, 4 * i + p) -= fac * s.m[j] * rij[p];
            OPX(3 * i + k, 4 * j + p) += fac * s.m[j] * rij[p];
            OPX(3 * j + k, 4 * j + p) -= fac * s.m[i] * rij[p];
            OPX(3 * j + k, 4 * i + p) += fac * s.m[i] * rij[p];
          }
          fac = 2.0 * GNEWT * fac1 * rij[k] / r1;
          OPX(3 * i + k, 4 * i + 3) += fac * s.m[j];
          OPX(3 * i + k, 4 * j + 3) += fac * s.m[j];
          OPX(3 * j + k, 4 * j + 3) -= fac * s.m[i];
          OPX(3 * j + k, 4 * i + 3) -= fac * s.m[i];
          fac = fac1 * fac2;
          OPX(3 * i + k, 4 * i + k) += fac * s.m[j];
          OPX(3 * i + k, 4 * j + k) -= fac * s.m[j];
          OPX(3 * j + k, 4 * j + k) += fac * s.m[i];
          OPX(3 * j + k, 4 * i + k) -= fac * s.m[i];
          fac = -2.0 * fac1 * (rij[k] * GNEWT * mij / (r2 * r1) + aij[k]);
          for (int p = 0; p < 3; p++) {
            double fac3 = fac * rij[p] + fac1 * 3.0 * rij[k] * aij[p];
            OPX(3 * i + k, 4 * i + p) += s.m[j] * fac3;
            OPX(3 * i + k, 4 * j + p) -= s.m[j] * fac3;
            OPX(3 * j + k, 4 * j + p) += s.m[i] * fac3;
            OPX(3 * j + k, 4 * i + p) -= s.m[i] * fac3;
          }
          fac = (-fac1) * r2;
          for (int di = 0; di < N; di++) {
            for (int p = 0; p < 3; p++)
              OPX(3 * i + k, 4 * di + p) += fac * s.m[j] * (DAX(3 * i + k, 4 * di + p) - DAX(3 * j + k, 4 * di + p));
            for (int p = 0; p < 3; p++)
              OPX(3 * j + k, 4 * di + p) -= fac * s.m[i] * (DAX(3 * i + k, 4 * di + p) - DAX(3 * j + k, 4 * di + p));
            OPX(3 * i + k, 4 * di + 3) += fac * s.m[j] * (DAX(3 * i + k, 4 * di + 3) - DAX(3 * j + k, 4 * di + 3));
            OPX(3 * j + k, 4 * di + 3) -= fac * s.m[i] * (DAX(3 * i + k, 4 * di + 3) - DAX(3 * j + k, 4 * di + 3));
          }
          fac = 3.0 * fac1 * rij[k];
          for (int di = 0; di < N; di++) {
            for (int p = 0; p < 3; p++) OPX(3 * i + k, 4 * di + p) += fac * s.m[j] * w.dot[4 * di + p];
            for (int p = 0; p < 3; p++) OPX(3 * j + k, 4 * di + p) -= fac * s.m[i] * w.dot[4 * di + p];
            OPX(3 * i + k, 4 * di + 3) += fac * s.m[j] * w.dot[4 * di + 3];
            OPX(3 * j + k, 4 * di + 3) -= fac * s.m[i] * w.dot[4 * di + 3];
          }
        }
      }
    }
}

// kepler_driftij_gamma! (ahl21.jl:706-760 with the block update of :31-42 on
// dq/dt; ahl21_no_grad.jl:192-212 without Jacobian).
template <int N, bool DRIFT_FIRST, bool GRADOPS, bool DQDT>
__device__ void kepler_pair(Sys<N>& s, Work<N>& w, int i, int j, double h2, const Rec& rec, int roff,
                            const Rec& cap, int coff) {
  double x0[3], v0[3];
  for (int k = 0; k < 3; k++) {
    x0[k] = s.x[3 * i + k] - s.x[3 * j + k];
    v0[k] = s.v[3 * i + k] - s.v[3 * j + k];
  }
  double gm = GNEWT * (s.m[i] + s.m[j]);
  if (cap.p && gm == 0.0) cap.put(coff + 6 + 15, 0.0);  // k = 0 marks a pair that keeps the stale jac_ij
  if (gm != 0.0) {
    KepParams P;
    double delxv[6];
    kep_delxv<DRIFT_FIRST, GRADOPS>(x0, v0, gm, h2, delxv, P);
    if (cap.p) {
      for (int q = 0; q < 3; q++) {
        cap.put(coff + q, x0[q]);
        cap.put(coff + 3 + q, v0[q]);
      }
      const double pv[22] = {P.gamma, P.g0, P.g1, P.g2, P.g3, P.h1, P.h2, P.dfdt, P.fm1, P.gmh, P.dgdtm1,
                             P.r0, P.r, P.r0inv, P.rinv, P.k, P.h, P.beta, P.betainv, P.eta, P.sqb, P.zeta};
      for (int q = 0; q < 22; q++) cap.put(coff + 6 + q, pv[q]);
    }
    double mijinv = 1.0 / (s.m[i] + s.m[j]);
    double mi = s.m[i] * mijinv, mj = s.m[j] * mijinv;
    if (GRADOPS) {
      double jk[48], jm[6];
      kep_jacobian<DRIFT_FIRST>(P, x0, v0, jk, jm);
      for (int r = 0; r < 6; r++)
        for (int l = 0; l < 6; l++) w.lk[r * 6 + l] = jk[r + 6 * l];
      w.lmi = mi;
      w.lmj = mj;
      for (int r = 0; r < 6; r++) {
        w.lmc6[r] = jm[r] * s.m[j];
        w.lmc13[r] = mi * delxv[r] * mijinv + GNEWT * mj * jk[r + 6 * 6];
        w.lmc6[6 + r] = (-mj) * delxv[r] * mijinv - GNEWT * mi * jk[r + 6 * 6];
        w.lmc13[6 + r] = (-jm[r]) * s.m[i];
      }
      for (int r = 0; r < 6; r++) {
        w.ldq[r] = mj * jk[r + 6 * 7];
        w.ldq[7 + r] = (-mi) * jk[r + 6 * 7];
      }
      w.ldq[6] = w.ldq[13] = 0.0;
    }
    for (int k = 0; k < 3; k++) {
      kahan(s.x[3 * i + k], s.xe[3 * i + k], mj * delxv[k]);
      kahan(s.x[3 * j + k], s.xe[3 * j + k], (-mi) * delxv[k]);
    }
    for (int k = 0; k < 3; k++) {
      kahan(s.v[3 * i + k], s.ve[3 * i + k], mj * delxv[3 + k]);
      kahan(s.v[3 * j + k], s.ve[3 * j + k], (-mi) * delxv[3 + k]);
    }
  }
  if (GRADOPS && rec.p) {
    for (int q = 0; q < 36; q++) rec.put(roff + q, w.lk[q]);
    rec.put(roff + PREC_MI, w.lmi);
    rec.put(roff + PREC_MJ, w.lmj);
    for (int q = 0; q < 12; q++) {
      rec.put(roff + PREC_MC6 + q, w.lmc6[q]);
      rec.put(roff + PREC_MC13 + q, w.lmc13[q]);
    }
  }
  if (DQDT) {
    // d.dqdt_ij .*= 1/2; d.dqdt_ij .+= dqdt_tmp1 .+ jac_ij * dqdt_tmp1 (ahl21.jl:38-40)
    double t1[14];
    for (int q = 0; q < 7; q++) {
      t1[q] = s.dqdt[7 * i + q];
      t1[7 + q] = s.dqdt[7 * j + q];
    }
    for (int q = 0; q < 14; q++) w.ldq[q] = w.ldq[q] * 0.5;
    for (int r = 0; r < 6; r++) {
      double ai = 0.0, aj = 0.0;
      for (int l = 0; l < 6; l++) {
        double kij = w.lmj * w.lk[r * 6 + l];
        double kji = w.lmi * w.lk[r * 6 + l];
        ai = fma(kij, t1[l], ai);
        aj = fma(-kji, t1[l], aj);
      }
      for (int l = 0; l < 6; l++) {
        double kij = w.lmj * w.lk[r * 6 + l];
        double kji = w.lmi * w.lk[r * 6 + l];
        ai = fma(-kij, t1[7 + l], ai);
        aj = fma(kji, t1[7 + l], aj);
      }
      w.ldq[r] = w.ldq[r] + (t1[r] + ai);
      w.ldq[7 + r] = w.ldq[7 + r] + (t1[7 + r] + aj);
    }
    w.ldq[6] = w.ldq[6] + (t1[6] + 0.0);
    w.ldq[13] = w.ldq[13] + (t1[13] + 0.0);
    for (int q = 0; q < 7; q++) {
      s.dqdt[7 * i + q] = w.ldq[q];
      s.dqdt[7 * j + q] = w.ldq[7 + q];
    }
  }
}

// One AHL21 step (ahl21.jl:5-95 / ahl21_no_grad.jl:6-18).
//   GRADOPS: build the operators (needed for records and for dq/dt);
//   DQDT:    compute dq/dt as the reference does;
//   rec:     where the operator record goes (rec.p == nullptr: nowhere).
//   cap, xs: where the Kepler-pair parameters and the position snapshots go
//            for the operator kernel (p == nullptr: nowhere).
template <int N, bool GRADOPS, bool DQDT>
__device__ __noinline__ void ahl21_step(Sys<N>& s, Work<N>& w, double h, uint64_t kick, const Rec& rec,
                                        const Rec& cap, const Rec& xs) {
  const double h2 = 0.5 * h, h6 = h / 6.0;
  if (GRADOPS) reset_last(w);
  if (DQDT)
    for (int q = 0; q < 7 * N; q++) s.dqdt[q] = 0.0;
  int roff = 0, slot = 0;
  if (kick && xs.p)
    for (int q = 0; q < 3 * N; q++) xs.put(3 * N + q, s.x[q]);
  if (kick) {
    kickfast<N, GRADOPS>(s, w, h6, kick);
    if (DQDT) dqdt_op(s, w, 6.0);
    if (GRADOPS) { put_op(rec, roff, w.op, op_size(N)); }
    roff += op_size(N);
  }
  drift(s, h2);
  if (DQDT)
    for (int b = 0; b < N; b++)
      for (int k = 0; k < 3; k++) s.dqdt[7 * b + k] = 0.5 * s.v[3 * b + k] + h2 * s.dqdt[7 * b + 3 + k];
  for (int i = 0; i < N - 1; i++)
    for (int j = i + 1; j < N; j++) {
      if ((kick >> pair_bit(i, j, N)) & 1) continue;
      kepler_pair<N, true, GRADOPS, DQDT>(s, w, i, j, h2, rec, roff, cap, slot * PCAP);
      roff += PREC;
      slot++;
    }
  if (xs.p)
    for (int q = 0; q < 3 * N; q++) xs.put(q, s.x[q]);
  phic<N, GRADOPS>(s, w, h, kick);
  phisalpha<N, GRADOPS>(s, w, h, 2.0, kick);
  if (DQDT) dqdt_op(s, w, 1.0);
  if (GRADOPS) put_op(rec, roff, w.op, op_size(N));
  roff += op_size(N);
  for (int i = N - 2; i >= 0; i--)
    for (int j = N - 1; j > i; j--) {
      if ((kick >> pair_bit(i, j, N)) & 1) continue;
      kepler_pair<N, false, GRADOPS, DQDT>(s, w, i, j, h2, rec, roff, cap, slot * PCAP);
      roff += PREC;
      slot++;
    }
  drift(s, h2);
  if (DQDT)
    for (int b = 0; b < N; b++)
      for (int k = 0; k < 3; k++)
        s.dqdt[7 * b + k] = s.dqdt[7 * b + k] + (0.5 * s.v[3 * b + k] + h2 * s.dqdt[7 * b + 3 + k]);
  if (kick) {
    if (xs.p)
      for (int q = 0; q < 3 * N; q++) xs.put(6 * N + q, s.x[q]);
    kickfast<N, GRADOPS>(s, w, h6, kick);
    if (DQDT) dqdt_op(s, w, 6.0);
    if (GRADOPS) put_op(rec, roff, w.op, op_size(N));
    roff += op_size(N);
  }
}

// g! and gd! (src/transits/timing.jl:141-150) for transited body i and
// occultor j.
template <int N>
__device__ __forceinline__ double gsky(const Sys<N>& s, int i, int j) {
  return (s.x[3 * j] - s.x[3 * i]) * (s.v[3 * j] - s.v[3 * i]) +
         (s.x[3 * j + 1] - s.x[3 * i + 1]) * (s.v[3 * j + 1] - s.v[3 * i + 1]);
}
template <int N>
__device__ __forceinline__ double gdot(const Sys<N>& s, int i, int j) {
  const double* q = s.dqdt;
  return ((s.x[3 * j] - s.x[3 * i]) * (q[7 * j + 3] - q[7 * i + 3]) +
          (s.x[3 * j + 1] - s.x[3 * i + 1]) * (q[7 * j + 4] - q[7 * i + 4]) +
          (s.v[3 * j] - s.v[3 * i]) * (q[7 * j + 0] - q[7 * i + 0]) +
          (s.v[3 * j + 1] - s.v[3 * i + 1]) * (q[7 * j + 1] - q[7 * i + 1]));
}

// u <- u + A^T u for the compact operator block A (velocity rows x position
// and mass columns); reads the record at roff.
template <int N>
__device__ void adj_op(double* u, const Rec& rec, int roff) {
  double add[4 * N];
  for (int d = 0; d < N; d++)
    for (int p = 0; p < 4; p++) {
      double acc = 0.0;
      for (int b = 0; b < N; b++)
        for (int k = 0; k < 3; k++) acc = fma(rec.get(roff + (3 * b + k) * (4 * N) + 4 * d + p), u[7 * b + 3 + k], acc);
      add[4 * d + p] = acc;
    }
  for (int d = 0; d < N; d++) {
    for (int p = 0; p < 3; p++) u[7 * d + p] = u[7 * d + p] + add[4 * d + p];
    u[7 * d + 6] = u[7 * d + 6] + add[4 * d + 3];
  }
}

// u <- u + A^T u for one Kepler pair record (the transpose of the factored
// jac_ij update the consumer applies).
__device__ __forceinline__ void adj_pair(double* u, int i, int j, const Rec& rec, int roff) {
  double mi = rec.get(roff + PREC_MI), mj = rec.get(roff + PREC_MJ);
  double z[6], ymi = 0.0, ymj = 0.0;
  for (int r = 0; r < 6; r++) {
    z[r] = mj * u[7 * i + r] - mi * u[7 * j + r];
    ymi = fma(rec.get(roff + PREC_MC6 + r), u[7 * i + r], ymi);
    ymi = fma(rec.get(roff + PREC_MC6 + 6 + r), u[7 * j + r], ymi);
    ymj = fma(rec.get(roff + PREC_MC13 + r), u[7 * i + r], ymj);
    ymj = fma(rec.get(roff + PREC_MC13 + 6 + r), u[7 * j + r], ymj);
  }
  double y[6];
  for (int l = 0; l < 6; l++) {
    double acc = 0.0;
    for (int r = 0; r < 6; r++) acc = fma(rec.get(roff + r * 6 + l), z[r], acc);
    y[l] = acc;
  }
  for (int l = 0; l < 6; l++) {
    u[7 * i + l] = u[7 * i + l] + y[l];
    u[7 * j + l] = u[7 * j + l] - y[l];
  }
  u[7 * i + 6] = u[7 * i + 6] + ymi;
  u[7 * j + 6] = u[7 * j + 6] + ymj;
}

// Adjoint of one recorded step: u^T <- u^T S where S is the step's map on
// jac_step (ahl21.jl:5-95): (I+K2)(I+D)prod_bwd(I+A)(I+Phi)prod_fwd(I+A)(I+D+K1).
// The first kick's product is formed before the first drift and added after
// it (ahl21.jl:16-23), hence the I + D + K1 factor.
template <int N>
__device__ void adjoint_step(double* u, double h, uint64_t kick, const Rec& rec) {
  const double h2 = 0.5 * h;
  int npk = 0;
  for (int i = 0; i < N - 1; i++)
    for (int j = i + 1; j < N; j++)
      if (!((kick >> pair_bit(i, j, N)) & 1)) npk++;
  int off_k1 = 0;
  int off_fwd = kick ? op_size(N) : 0;
  int off_phi = off_fwd + npk * PREC;
  int off_bwd = off_phi + op_size(N);
  int off_k2 = off_bwd + npk * PREC;
  if (kick) adj_op<N>(u, rec, off_k2);
  for (int b = 0; b < N; b++)
    for (int k = 0; k < 3; k++) u[7 * b + 3 + k] = u[7 * b + 3 + k] + h2 * u[7 * b + k];
  // backward sweep was applied in order (N-2..0, N-1..i+1); undo in reverse
  {
    int q = npk - 1;
    for (int i = 0; i < N - 1; i++)
      for (int j = i + 1; j < N; j++) {
        if ((kick >> pair_bit(i, j, N)) & 1) continue;
        adj_pair(u, i, j, rec, off_bwd + q * PREC);
        q--;
      }
  }
  adj_op<N>(u, rec, off_phi);
  {
    int q = npk - 1;
    for (int i = N - 2; i >= 0; i--)
      for (int j = N - 1; j > i; j--) {
        if ((kick >> pair_bit(i, j, N)) & 1) continue;
        adj_pair(u, i, j, rec, off_fwd + q * PREC);
        q--;
      }
  }
  if (kick) {
    // both terms of I + D + K1 act on the same u: D^T reads the position
    // entries, K1^T reads the velocity entries and writes positions/masses.
    double ux[3 * N];
    for (int b = 0; b < N; b++)
      for (int k = 0; k < 3; k++) ux[3 * b + k] = u[7 * b + k];
    adj_op<N>(u, rec, off_k1);
    for (int b = 0; b < N; b++)
      for (int k = 0; k < 3; k++) u[7 * b + 3 + k] = u[7 * b + 3 + k] + h2 * ux[3 * b + k];
  } else {
    for (int b = 0; b < N; b++)
      for (int k = 0; k < 3; k++) u[7 * b + 3 + k] = u[7 * b + 3 + k] + h2 * u[7 * b + k];
  }
}

#undef OPX
#undef DAX

}  // namespace nbg
