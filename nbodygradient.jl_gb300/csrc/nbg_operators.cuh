// nbg_operators.cuh -- builds the step operator records from the parameters
// the orbit producer captured, in parallel over (step, pair, system).
//
// The producer advances x, v only (the arithmetic of ahl21_no_grad.jl, bitwise
// the x, v of the gradient step) and captures, per Kepler pair, x0, v0 and the
// 22 values jac_delxv_gamma! returns (ahl21.jl:888-889), plus the positions at
// the correctors and kicks.  Everything else kepler_driftij_gamma!,
// phic!/phisalpha! and kickfast! compute for the Jacobian depends only on
// those values, so it runs here, off the producer's sequential chain:
//   * compute_jacobian_gamma! (ahl21.jl:896-1139) and the jac_ij assembly
//     (ahl21.jl:727-750) per pair;
//   * jac_phi (ahl21.jl:392-700) and jac_kick (ahl21.jl:337-386) per step.
#pragma once
#include "nbg_orbit.cuh"

namespace nbg {

// Bodies (i, j) of Kepler-pair slot q of a step: slots 0..npk-1 follow the
// forward sweep (i ascending, j ascending), npk..2npk-1 the backward sweep.
template <int N>
__device__ __forceinline__ void pair_of_slot(int q, int npk, uint64_t kick, int* pi, int* pj) {
  int c = 0;
  if (q < npk) {
    for (int i = 0; i < N - 1; i++)
      for (int j = i + 1; j < N; j++) {
        if ((kick >> pair_bit(i, j, N)) & 1) continue;
        if (c++ == q) { *pi = i; *pj = j; return; }
      }
  } else {
    q -= npk;
    for (int i = N - 2; i >= 0; i--)
      for (int j = N - 1; j > i; j--) {
        if ((kick >> pair_bit(i, j, N)) & 1) continue;
        if (c++ == q) { *pi = i; *pj = j; return; }
      }
  }
  *pi = 0;
  *pj = 1;
}

// kepler_driftij_gamma!'s Jacobian part for one pair from its capture.
template <bool DRIFT_FIRST>
__device__ void pair_record_from_capture(const Rec& cap, int coff, double m_i, double m_j, const Rec& rec,
                                         int roff) {
  double x0[3], v0[3];
  for (int q = 0; q < 3; q++) {
    x0[q] = cap.get(coff + q);
    v0[q] = cap.get(coff + 3 + q);
  }
  KepParams P;
  double* pv[22] = {&P.gamma, &P.g0, &P.g1, &P.g2, &P.g3, &P.h1, &P.h2, &P.dfdt, &P.fm1, &P.gmh, &P.dgdtm1,
                    &P.r0, &P.r, &P.r0inv, &P.rinv, &P.k, &P.h, &P.beta, &P.betainv, &P.eta, &P.sqb, &P.zeta};
  for (int q = 0; q < 22; q++) *pv[q] = cap.get(coff + 6 + q);
  GH gh = gh_functions<GH_H1 | GH_H2 | GH_H3 | GH_H5 | GH_H6>(P.gamma, P.beta, P.sqb);
  P.H1v = gh.h1; P.H2v = gh.h2; P.H3v = gh.h3; P.H5v = gh.h5; P.H6v = gh.h6;
  double jk[48], jm[6];
  kep_jacobian<DRIFT_FIRST>(P, x0, v0, jk, jm);
  double delxv[6];
  for (int j = 0; j < 3; j++) delxv[j] = P.fm1 * x0[j] + P.gmh * v0[j];
  for (int j = 0; j < 3; j++) delxv[3 + j] = P.dfdt * x0[j] + P.dgdtm1 * v0[j];
  const double mijinv = 1.0 / (m_i + m_j);
  const double mi = m_i * mijinv, mj = m_j * mijinv;
  for (int r = 0; r < 6; r++)
    for (int l = 0; l < 6; l++) rec.put(roff + r * 6 + l, jk[r + 6 * l]);
  rec.put(roff + PREC_MI, mi);
  rec.put(roff + PREC_MJ, mj);
  for (int r = 0; r < 6; r++) {
    rec.put(roff + PREC_MC6 + r, jm[r] * m_j);
    rec.put(roff + PREC_MC13 + r, mi * delxv[r] * mijinv + GNEWT * mj * jk[r + 6 * 6]);
    rec.put(roff + PREC_MC6 + 6 + r, (-mj) * delxv[r] * mijinv - GNEWT * mi * jk[r + 6 * 6]);
    rec.put(roff + PREC_MC13 + 6 + r, (-jm[r]) * m_i);
  }
}

// Physical time derivative of the sky-plane projection g (timing.jl:141-144)
// for transited body i and occultor j: |dv|^2 in the sky plane plus the
// relative acceleration term.  Drives the transit Newton iterations; the
// converged search's dtdq0 uses the reference's step derivative (gd!).
template <int N>
__device__ __forceinline__ double gdot_physical(const Sys<N>& s, int i, int j) {
  double ai[2] = {0.0, 0.0}, aj[2] = {0.0, 0.0};
  for (int b = 0; b < N; b++) {
    if (b != i) {
      double d0 = s.x[3 * b] - s.x[3 * i], d1 = s.x[3 * b + 1] - s.x[3 * i + 1], d2 = s.x[3 * b + 2] - s.x[3 * i + 2];
      double r2 = d0 * d0 + d1 * d1 + d2 * d2;
      double f = GNEWT * s.m[b] / (r2 * sqrt(r2));
      ai[0] += f * d0;
      ai[1] += f * d1;
    }
    if (b != j) {
      double d0 = s.x[3 * b] - s.x[3 * j], d1 = s.x[3 * b + 1] - s.x[3 * j + 1], d2 = s.x[3 * b + 2] - s.x[3 * j + 2];
      double r2 = d0 * d0 + d1 * d1 + d2 * d2;
      double f = GNEWT * s.m[b] / (r2 * sqrt(r2));
      aj[0] += f * d0;
      aj[1] += f * d1;
    }
  }
  const double dvx = s.v[3 * j] - s.v[3 * i], dvy = s.v[3 * j + 1] - s.v[3 * i + 1];
  const double dx = s.x[3 * j] - s.x[3 * i], dy = s.x[3 * j + 1] - s.x[3 * i + 1];
  return dvx * dvx + dvy * dvy + dx * (aj[0] - ai[0]) + dy * (aj[1] - ai[1]);
}

}  // namespace nbg
