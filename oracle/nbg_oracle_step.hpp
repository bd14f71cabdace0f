// nbg_oracle_step.hpp -- TEST INFRASTRUCTURE ONLY (parity oracle; see
// nbg_oracle.hpp).  Restates src/integrator/ahl21/ahl21.jl (the step with
// Jacobian) and src/integrator/ahl21/ahl21_no_grad.jl (the step without).
// Row/column indices are 0-based: body i owns rows 7i..7i+6 ordered
// (x, y, z, vx, vy, vz, m).
#pragma once

namespace nbgo {

// drift_grad! (ahl21.jl:318-331)
template <class T> void drift_grad(State<T>& s, T h) {
  int M = 7 * s.n;
  for (int i = 0; i < s.n; i++) {
    int indi = 7 * i;
    for (int j = 0; j < 3; j++) comp_sum(s.X(j, i), s.XE(j, i), h * s.V(j, i));
    for (int k = 0; k < M; k++)
      for (int j = 0; j < 3; j++)
        comp_sum(s.J(indi + j, k), s.JE(indi + j, k), h * s.J(indi + 3 + j, k));
  }
}

// kickfast! with Jacobian (ahl21.jl:337-386)
template <class T> void kickfast(State<T>& s, Derivs<T>& d, T h) {
  const T G = T(GNEWT_D);
  int n = s.n;
  for (int k = 0; k < 3; k++) s.rij[k] = T(0);
  std::fill(d.jac_kick.begin(), d.jac_kick.end(), T(0));
  for (int i = 0; i < n - 1; i++) {
    int indi = 7 * i;
    for (int j = i + 1; j < n; j++) {
      int indj = 7 * j;
      if (!s.P(i, j)) continue;
      for (int k = 0; k < 3; k++) s.rij[k] = s.X(k, i) - s.X(k, j);
      T r2inv = T(1) / dot3(s.rij, s.rij);
      T r3inv = r2inv * Mth<T>::sqrt(r2inv);
      T fac2 = h * G * r3inv;
      for (int k = 0; k < 3; k++) {
        T fac = fac2 * s.rij[k];
        comp_sum(s.V(k, i), s.VE(k, i), (-s.m[j]) * fac);
        comp_sum(s.V(k, j), s.VE(k, j), s.m[i] * fac);
        d.dqdt_kick[indi + 3 + k] = d.dqdt_kick[indi + 3 + k] - s.m[j] * fac / h;
        d.dqdt_kick[indj + 3 + k] = d.dqdt_kick[indj + 3 + k] + s.m[i] * fac / h;
        d.kick(indi + 3 + k, indj + 6) -= fac;
        d.kick(indj + 3 + k, indi + 6) += fac;
        fac = fac * (T(3) * r2inv);
        for (int p = 0; p < 3; p++) {
          d.kick(indi + 3 + k, indi + p) += fac * s.m[j] * s.rij[p];
          d.kick(indi + 3 + k, indj + p) -= fac * s.m[j] * s.rij[p];
          d.kick(indj + 3 + k, indj + p) += fac * s.m[i] * s.rij[p];
          d.kick(indj + 3 + k, indi + p) -= fac * s.m[i] * s.rij[p];
        }
        d.kick(indi + 3 + k, indi + k) -= fac2 * s.m[j];
        d.kick(indi + 3 + k, indj + k) += fac2 * s.m[j];
        d.kick(indj + 3 + k, indj + k) -= fac2 * s.m[i];
        d.kick(indj + 3 + k, indi + k) += fac2 * s.m[i];
      }
    }
  }
}

// phic! with Jacobian (ahl21.jl:392-552)
template <class T> void phic(State<T>& s, Derivs<T>& d, T h) {
  const T G = T(GNEWT_D);
  int n = s.n;
  std::fill(s.a.begin(), s.a.end(), T(0));
  for (int k = 0; k < 3; k++) s.rij[k] = s.aij[k] = T(0);
  std::fill(d.dadq.begin(), d.dadq.end(), T(0));
  std::fill(d.dotdadq.begin(), d.dotdadq.end(), T(0));
  std::fill(d.jac_phi.begin(), d.jac_phi.end(), T(0));
  T coeff = h * h * h / T(36) * G;
  for (int i = 0; i < n - 1; i++) {
    int indi = 7 * i;
    for (int j = i + 1; j < n; j++) {
      if (!s.P(i, j)) continue;
      int indj = 7 * j;
      for (int k = 0; k < 3; k++) s.rij[k] = s.X(k, i) - s.X(k, j);
      T r2inv = T(1) / dot3(s.rij, s.rij);
      T r3inv = r2inv * Mth<T>::sqrt(r2inv);
      for (int k = 0; k < 3; k++) {
        T fac = G * s.rij[k] * r3inv;
        T facv = fac * T(2) * h / T(3);
        comp_sum(s.V(k, i), s.VE(k, i), (-s.m[j]) * facv);
        comp_sum(s.V(k, j), s.VE(k, j), s.m[i] * facv);
        d.dqdt_phi[indi + 3 + k] = d.dqdt_phi[indi + 3 + k] - T(1) / h * s.m[j] * facv;
        d.dqdt_phi[indj + 3 + k] = d.dqdt_phi[indj + 3 + k] + T(1) / h * s.m[i] * facv;
        s.A(k, i) = s.A(k, i) - s.m[j] * fac;
        s.A(k, j) = s.A(k, j) + s.m[i] * fac;
        d.phi(indi + 3 + k, indj + 6) -= facv;
        d.phi(indj + 3 + k, indi + 6) += facv;
        facv = facv * (T(3) * r2inv);
        for (int p = 0; p < 3; p++) {
          d.phi(indi + 3 + k, indi + p) += facv * s.m[j] * s.rij[p];
          d.phi(indi + 3 + k, indj + p) -= facv * s.m[j] * s.rij[p];
          d.phi(indj + 3 + k, indj + p) += facv * s.m[i] * s.rij[p];
          d.phi(indj + 3 + k, indi + p) -= facv * s.m[i] * s.rij[p];
        }
        facv = T(2) * h / T(3) * G * r3inv;
        d.phi(indi + 3 + k, indi + k) -= facv * s.m[j];
        d.phi(indi + 3 + k, indj + k) += facv * s.m[j];
        d.phi(indj + 3 + k, indj + k) -= facv * s.m[i];
        d.phi(indj + 3 + k, indi + k) += facv * s.m[i];
        d.DA(k, i, 3, j) -= fac;
        d.DA(k, j, 3, i) += fac;
        fac = fac * (T(3) * r2inv);
        for (int p = 0; p < 3; p++) {
          d.DA(k, i, p, i) += fac * s.m[j] * s.rij[p];
          d.DA(k, i, p, j) -= fac * s.m[j] * s.rij[p];
          d.DA(k, j, p, j) += fac * s.m[i] * s.rij[p];
          d.DA(k, j, p, i) -= fac * s.m[i] * s.rij[p];
        }
        fac = G * r3inv;
        d.DA(k, i, k, i) -= fac * s.m[j];
        d.DA(k, i, k, j) += fac * s.m[j];
        d.DA(k, j, k, j) -= fac * s.m[i];
        d.DA(k, j, k, i) += fac * s.m[i];
      }
    }
  }
  for (int i = 0; i < n - 1; i++) {
    int indi = 7 * i;
    for (int j = i + 1; j < n; j++) {
      if (!s.P(i, j)) continue;
      int indj = 7 * j;
      for (int k = 0; k < 3; k++) {
        s.aij[k] = s.A(k, i) - s.A(k, j);
        s.rij[k] = s.X(k, i) - s.X(k, j);
      }
      std::fill(d.dotdadq.begin(), d.dotdadq.end(), T(0));
      for (int di = 0; di < n; di++)
        for (int p = 0; p < 4; p++)
          for (int k = 0; k < 3; k++)
            d.DOT(p, di) += s.rij[k] * (d.DA(k, i, p, di) - d.DA(k, j, p, di));
      T r2 = dot3(s.rij, s.rij);
      T r1 = Mth<T>::sqrt(r2);
      T ardot = dot3(s.aij, s.rij);
      T fac1 = coeff / (r2 * r2 * r1);
      T fac2 = T(3) * ardot;
      for (int k = 0; k < 3; k++) {
        T fac = fac1 * (s.rij[k] * fac2 - r2 * s.aij[k]);
        comp_sum(s.V(k, i), s.VE(k, i), s.m[j] * fac);
        comp_sum(s.V(k, j), s.VE(k, j), (-s.m[i]) * fac);
        d.dqdt_phi[indi + 3 + k] = d.dqdt_phi[indi + 3 + k] + T(3) / h * s.m[j] * fac;
        d.dqdt_phi[indj + 3 + k] = d.dqdt_phi[indj + 3 + k] - T(3) / h * s.m[i] * fac;
        d.phi(indi + 3 + k, indj + 6) += fac;
        d.phi(indj + 3 + k, indi + 6) -= fac;
        fac = fac * (T(5) / r2);
        for (int p = 0; p < 3; p++) {
          d.phi(indi + 3 + k, indi + p) -= fac * s.m[j] * s.rij[p];
          d.phi(indi + 3 + k, indj + p) += fac * s.m[j] * s.rij[p];
          d.phi(indj + 3 + k, indj + p) -= fac * s.m[i] * s.rij[p];
          d.phi(indj + 3 + k, indi + p) += fac * s.m[i] * s.rij[p];
        }
        fac = fac1 * fac2;
        d.phi(indi + 3 + k, indi + k) += fac * s.m[j];
        d.phi(indi + 3 + k, indj + k) -= fac * s.m[j];
        d.phi(indj + 3 + k, indj + k) += fac * s.m[i];
        d.phi(indj + 3 + k, indi + k) -= fac * s.m[i];
        fac = T(-2) * fac1 * s.aij[k];
        for (int p = 0; p < 3; p++) {
          T fac3 = fac * s.rij[p] + fac1 * T(3) * s.rij[k] * s.aij[p];
          d.phi(indi + 3 + k, indi + p) += s.m[j] * fac3;
          d.phi(indi + 3 + k, indj + p) -= s.m[j] * fac3;
          d.phi(indj + 3 + k, indj + p) += s.m[i] * fac3;
          d.phi(indj + 3 + k, indi + p) -= s.m[i] * fac3;
        }
        fac = (-fac1) * r2;
        for (int di = 0; di < n; di++) {
          int indd = 7 * di;
          for (int p = 0; p < 3; p++) {
            d.phi(indi + 3 + k, indd + p) += fac * s.m[j] * (d.DA(k, i, p, di) - d.DA(k, j, p, di));
            d.phi(indj + 3 + k, indd + p) -= fac * s.m[i] * (d.DA(k, i, p, di) - d.DA(k, j, p, di));
          }
          d.phi(indi + 3 + k, indd + 6) += fac * s.m[j] * (d.DA(k, i, 3, di) - d.DA(k, j, 3, di));
          d.phi(indj + 3 + k, indd + 6) -= fac * s.m[i] * (d.DA(k, i, 3, di) - d.DA(k, j, 3, di));
        }
        fac = T(3) * fac1 * s.rij[k];
        for (int di = 0; di < n; di++) {
          int indd = 7 * di;
          for (int p = 0; p < 3; p++) {
            d.phi(indi + 3 + k, indd + p) += fac * s.m[j] * d.DOT(p, di);
            d.phi(indj + 3 + k, indd + p) -= fac * s.m[i] * d.DOT(p, di);
          }
          d.phi(indi + 3 + k, indd + 6) += fac * s.m[j] * d.DOT(3, di);
          d.phi(indj + 3 + k, indd + 6) -= fac * s.m[i] * d.DOT(3, di);
        }
      }
    }
  }
}

// phisalpha! with Jacobian (ahl21.jl:558-700)
template <class T> void phisalpha(State<T>& s, Derivs<T>& d, T h, T alpha) {
  const T G = T(GNEWT_D);
  int n = s.n;
  std::fill(s.a.begin(), s.a.end(), T(0));
  std::fill(d.dadq.begin(), d.dadq.end(), T(0));
  std::fill(d.dotdadq.begin(), d.dotdadq.end(), T(0));
  for (int k = 0; k < 3; k++) s.rij[k] = s.aij[k] = T(0);
  T coeff = alpha * (h * h * h) / T(96) * T(2) * G;
  for (int i = 0; i < n - 1; i++)
    for (int j = i + 1; j < n; j++) {
      if (s.P(i, j)) continue;
      for (int k = 0; k < 3; k++) s.rij[k] = s.X(k, i) - s.X(k, j);
      T r2 = dot3(s.rij, s.rij);
      T r3 = r2 * Mth<T>::sqrt(r2);
      T fac2 = G / r3;
      for (int k = 0; k < 3; k++) {
        T fac = fac2 * s.rij[k];
        s.A(k, i) = s.A(k, i) - s.m[j] * fac;
        s.A(k, j) = s.A(k, j) + s.m[i] * fac;
        d.DA(k, i, 3, j) -= fac;
        d.DA(k, j, 3, i) += fac;
        fac = fac * (T(3) / r2);
        for (int p = 0; p < 3; p++) {
          d.DA(k, i, p, i) += fac * s.m[j] * s.rij[p];
          d.DA(k, i, p, j) -= fac * s.m[j] * s.rij[p];
          d.DA(k, j, p, j) += fac * s.m[i] * s.rij[p];
          d.DA(k, j, p, i) -= fac * s.m[i] * s.rij[p];
        }
        d.DA(k, i, k, i) -= fac2 * s.m[j];
        d.DA(k, i, k, j) += fac2 * s.m[j];
        d.DA(k, j, k, j) -= fac2 * s.m[i];
        d.DA(k, j, k, i) += fac2 * s.m[i];
      }
    }
  for (int i = 0; i < n - 1; i++) {
    int indi = 7 * i;
    for (int j = i + 1; j < n; j++) {
      if (s.P(i, j)) continue;
      int indj = 7 * j;
      for (int k = 0; k < 3; k++) {
        s.aij[k] = s.A(k, i) - s.A(k, j);
        s.rij[k] = s.X(k, i) - s.X(k, j);
      }
      std::fill(d.dotdadq.begin(), d.dotdadq.end(), T(0));
      for (int di = 0; di < n; di++)
        for (int p = 0; p < 4; p++)
          for (int k = 0; k < 3; k++)
            d.DOT(p, di) += s.rij[k] * (d.DA(k, i, p, di) - d.DA(k, j, p, di));
      T r2 = dot3(s.rij, s.rij);
      T r1 = Mth<T>::sqrt(r2);
      T ardot = dot3(s.aij, s.rij);
      T fac1 = coeff / (r2 * r2 * r1);
      T mij = s.m[i] + s.m[j];
      T fac2 = T(2) * G * mij / r1 + T(3) * ardot;
      for (int k = 0; k < 3; k++) {
        T fac = fac1 * (s.rij[k] * fac2 - r2 * s.aij[k]);
        comp_sum(s.V(k, i), s.VE(k, i), s.m[j] * fac);
        comp_sum(s.V(k, j), s.VE(k, j), (-s.m[i]) * fac);
        d.dqdt_phi[indi + 3 + k] = d.dqdt_phi[indi + 3 + k] + T(3) / h * s.m[j] * fac;
        d.dqdt_phi[indj + 3 + k] = d.dqdt_phi[indj + 3 + k] - T(3) / h * s.m[i] * fac;
        d.phi(indi + 3 + k, indj + 6) += fac;
        d.phi(indj + 3 + k, indi + 6) -= fac;
        fac = fac * (T(5) / r2);
        for (int p = 0; p < 3; p++) {
          d.phi(indi + 3 + k, indi + p) -= fac * s.m[j] * s.rij[p];
          d.phi(indi + 3 + k, indj + p) += fac * s.m[j] * s.rij[p];
          d.phi(indj + 3 + k, indj + p) -= fac * s.m[i] * s.rij[p];
          d.phi(indj + 3 + k, indi + p) += fac * s.m[i] * s.rij[p];
        }
        fac = T(2) * G * fac1 * s.rij[k] / r1;
        d.phi(indi + 3 + k, indi + 6) += fac * s.m[j];
        d.phi(indi + 3 + k, indj + 6) += fac * s.m[j];
        d.phi(indj + 3 + k, indj + 6) -= fac * s.m[i];
        d.phi(indj + 3 + k, indi + 6) -= fac * s.m[i];
        fac = fac1 * fac2;
        d.phi(indi + 3 + k, indi + k) += fac * s.m[j];
        d.phi(indi + 3 + k, indj + k) -= fac * s.m[j];
        d.phi(indj + 3 + k, indj + k) += fac * s.m[i];
        d.phi(indj + 3 + k, indi + k) -= fac * s.m[i];
        fac = T(-2) * fac1 * (s.rij[k] * G * mij / (r2 * r1) + s.aij[k]);
        for (int p = 0; p < 3; p++) {
          T fac3 = fac * s.rij[p] + fac1 * T(3) * s.rij[k] * s.aij[p];
          d.phi(indi + 3 + k, indi + p) += s.m[j] * fac3;
          d.phi(indi + 3 + k, indj + p) -= s.m[j] * fac3;
          d.phi(indj + 3 + k, indj + p) += s.m[i] * fac3;
          d.phi(indj + 3 + k, indi + p) -= s.m[i] * fac3;
        }
        fac = (-fac1) * r2;
        for (int di = 0; di < n; di++) {
          int indd = 7 * di;
          for (int p = 0; p < 3; p++)
            d.phi(indi + 3 + k, indd + p) += fac * s.m[j] * (d.DA(k, i, p, di) - d.DA(k, j, p, di));
          for (int p = 0; p < 3; p++)
            d.phi(indj + 3 + k, indd + p) -= fac * s.m[i] * (d.DA(k, i, p, di) - d.DA(k, j, p, di));
          d.phi(indi + 3 + k, indd + 6) += fac * s.m[j] * (d.DA(k, i, 3, di) - d.DA(k, j, 3, di));
          d.phi(indj + 3 + k, indd + 6) -= fac * s.m[i] * (d.DA(k, i, 3, di) - d.DA(k, j, 3, di));
        }
        fac = T(3) * fac1 * s.rij[k];
        for (int di = 0; di < n; di++) {
          int indd = 7 * di;
          for (int p = 0; p < 3; p++) d.phi(indi + 3 + k, indd + p) += fac * s.m[j] * d.DOT(p, di);
          for (int p = 0; p < 3; p++) d.phi(indj + 3 + k, indd + p) -= fac * s.m[i] * d.DOT(p, di);
          d.phi(indi + 3 + k, indd + 6) += fac * s.m[j] * d.DOT(3, di);
          d.phi(indj + 3 + k, indd + 6) -= fac * s.m[i] * d.DOT(3, di);
        }
      }
    }
  }
}

// The 22 values returned by jac_delxv_gamma! (ahl21.jl:888-889).
template <class T> struct KepParams {
  T gamma, g0, g1, g2, g3, h1, h2, dfdt, fm1, gmh, dgdtm1, r0, r, r0inv, rinv, k, h, beta, betainv, eta, sqb, zeta;
};

// jac_delxv_gamma! (ahl21.jl:766-890).  Reads s.x0, s.v0; writes s.delxv.
template <class T> KepParams<T> jac_delxv_gamma(State<T>& s, T k, T h, bool drift_first) {
  s.rtmp[0] = s.x0[0] - h * s.v0[0];
  s.rtmp[1] = s.x0[1] - h * s.v0[1];
  s.rtmp[2] = s.x0[2] - h * s.v0[2];
  T r0 = drift_first ? Mth<T>::sqrt(dot3(s.rtmp, s.rtmp)) : Mth<T>::sqrt(dot3(s.x0, s.x0));
  T r0inv = T(1) / r0;
  T beta0 = T(2) * k * r0inv - dot3(s.v0, s.v0);
  T beta0inv = T(1) / beta0;
  T signb = jsign(beta0);
  T sqb = Mth<T>::sqrt(signb * beta0);
  T zeta = k - r0 * beta0;
  T gamma_guess;
  T eta = drift_first ? dot3(s.rtmp, s.v0) : dot3(s.x0, s.v0);
  if (zeta != T(0)) {
    T zinv = T(6) / zeta;
    gamma_guess = cubic1(T(0.5) * eta * sqb * zinv, r0 * signb * beta0 * zinv,
                         (-h) * signb * beta0 * sqb * zinv);
  } else {
    if (eta != T(0)) {
      T reta = r0 / eta;
      T disc = reta * reta + T(2) * h / eta;
      gamma_guess = (disc > T(0)) ? sqb * ((-reta) + Mth<T>::sqrt(disc)) : h * r0inv * sqb;
    } else {
      gamma_guess = h * r0inv * sqb;
    }
  }
  T gamma = gamma_guess;
  T gamma1 = T(2) * gamma, gamma2 = T(3) * gamma;
  int iter = 0;
  const int ITMAX = 20;
  T c2 = T(-2) * zeta, c3 = T(2) * eta * signb * sqb, c4 = (-sqb) * h * beta0, c5 = T(2) * eta * signb * sqb;
  T sx, cx;
  while (iter < ITMAX) {
    gamma2 = gamma1;
    gamma1 = gamma;
    T xx = T(0.5) * gamma;
    if (beta0 > T(0)) {
      sx = Mth<T>::sin(xx); cx = Mth<T>::cos(xx);
    } else {
      sx = Mth<T>::sinh(xx); cx = Mth<T>::exp(-xx) + sx;
    }
    gamma = gamma - (k * gamma + c2 * sx * cx + c3 * (sx * sx) + c4) /
                        (T(2) * signb * zeta * (sx * sx) + c5 * sx * cx + r0 * beta0);
    iter += 1;
    if (gamma == gamma2 || gamma == gamma1) break;
  }
  for (int q = 0; q < 6; q++) s.delxv[q] = T(0);
  T xx = T(0.5) * gamma;
  if (beta0 > T(0)) {
    sx = Mth<T>::sin(xx); cx = Mth<T>::cos(xx);
  } else {
    sx = Mth<T>::sinh(xx); cx = Mth<T>::exp(-xx) + sx;
  }
  T g1bs = T(2) * sx * cx / sqb;
  T g2bs = T(2) * signb * (sx * sx) * beta0inv;
  T g0bs = T(1) - beta0 * g2bs;
  T g3bs = G3(gamma, beta0, sqb);
  T h1 = T(0), h2 = T(0);
  T r = r0 * g0bs + eta * g1bs + k * g2bs;
  T rinv = T(1) / r;
  T dfdt = (-k) * g1bs * rinv * r0inv;
  T fm1, gmh, dgdtm1;
  if (drift_first) {
    fm1 = (-k) * r0inv * g2bs;
    gmh = k * r0inv * (h * g2bs - r0 * g3bs);
  } else {
    h1 = H1(gamma, beta0);
    h2 = H2(gamma, beta0, sqb);
    fm1 = k * rinv * (g2bs - k * r0inv * h1);
    gmh = k * rinv * (r0 * h2 + eta * h1);
  }
  if (drift_first) dgdtm1 = k * r0inv * rinv * (h * g1bs - r0 * g2bs);
  else dgdtm1 = (-k) * rinv * g2bs;
  for (int j = 0; j < 3; j++) s.delxv[j] = fm1 * s.x0[j] + gmh * s.v0[j];
  for (int j = 0; j < 3; j++) s.delxv[3 + j] = dfdt * s.x0[j] + dgdtm1 * s.v0[j];
  KepParams<T> P;
  P.gamma = gamma; P.g0 = g0bs; P.g1 = g1bs; P.g2 = g2bs; P.g3 = g3bs; P.h1 = h1; P.h2 = h2;
  P.dfdt = dfdt; P.fm1 = fm1; P.gmh = gmh; P.dgdtm1 = dgdtm1; P.r0 = r0; P.r = r; P.r0inv = r0inv;
  P.rinv = rinv; P.k = k; P.h = h; P.beta = beta0; P.betainv = beta0inv; P.eta = eta; P.sqb = sqb;
  P.zeta = zeta;
  return P;
}

// compute_jacobian_gamma! (ahl21.jl:896-1139) with debug = false.
// jk is the 6x8 jac_kepler (col-major), jm the 6-vector jac_mass.
template <class T>
void compute_jacobian_gamma(const KepParams<T>& P, const T* x0, const T* v0, T* jk, T* jm,
                            bool drift_first) {
  const T G = T(GNEWT_D);
  const T gamma = P.gamma, g0 = P.g0, g1 = P.g1, g2 = P.g2, g3 = P.g3, h1 = P.h1;
  T h2 = P.h2;
  const T dfdt = P.dfdt, fm1 = P.fm1, gmh = P.gmh, dgdtm1 = P.dgdtm1, r0 = P.r0, r = P.r;
  const T r0inv = P.r0inv, rinv = P.rinv, k = P.k, h = P.h, beta = P.beta, betainv = P.betainv;
  const T eta = P.eta, sqb = P.sqb, zeta = P.zeta;
  auto JK = [&](int a, int b) -> T& { return jk[a + 6 * b]; };
  T r0inv2 = r0inv * r0inv;
  T r0inv3 = r0inv2 * r0inv;
  T rinv2 = rinv * rinv;
  T rinv3 = rinv2 * rinv;
  T hsq = h * h;
  T ksq = k * k;
  if (drift_first) {
    T d = (h + eta * g2 + T(2) * k * g3) * betainv;
    T c1 = d - r0 * g3;
    T c2 = eta * g0 + g1 * zeta;
    T c3 = d * k + g1 * (r0 * r0);
    T c13 = g1 * h - g2 * r0;
    T c9 = T(2) * g2 * h - T(3) * g3 * r0;
    T c10 = k * (r0inv2 * r0inv2) * ((-g2) * r0 * h + k * c9 * betainv - c3 * c13 * rinv);
    T c24 = r0inv3 * (r0 * (T(2) * k * r0inv - beta) * betainv - g1 * c3 * rinv / g2);
    T h6 = H6(gamma, beta);
    T dfm1dxx = fm1 * c24;
    T dfm1dxv = (-fm1) * (g1 * rinv + h * c24);
    T dfm1dvx = dfm1dxv;
    T dfm1dvv = fm1 * rinv * ((-r0) * g2 + k * h6 * betainv / g2 + h * (T(2) * g1 + h * r * c24));
    T dfm1dh = fm1 * (g1 * rinv * (T(1) / g2 + T(2) * k * r0inv - beta) - eta * c24);
    T dfm1dk = fm1 * (T(1) / k + g1 * c1 * rinv * r0inv / g2 - T(2) * betainv * r0inv);
    T h4 = (-H1(gamma, beta)) * beta;
    T h5 = H5(gamma, beta, sqb);
    T dfm1dk2 = (r0 * h4 + k * h6);
    T dgmhdxx = c10;
    T dgmhdxv = (-g2) * k * c13 * rinv * r0inv - h * c10;
    T dgmhdvx = dgmhdxv;
    T h3 = H3(gamma, beta, sqb);
    T h8 = (-(T(2) * h3)) + T(3) * h5;
    T dgmhdvv = T(2) * g2 * h * k * c13 * rinv * r0inv + hsq * c10 +
                k * betainv * rinv * r0inv *
                    ((r0 * r0) * h8 - beta * h * r0 * (g2 * g2) + (h * k + eta * r0) * h6);
    T dgmhdh = g2 * k * r0inv + k * c13 * rinv * r0inv +
               g2 * k * (T(2) * k * r0inv - beta) * c13 * rinv * r0inv - eta * c10;
    T dgmhdk = r0inv * (k * c1 * c13 * rinv * r0inv + g2 * h - g3 * r0 - k * c9 * betainv * r0inv);
    T dgmhdk2 = (h6 * g3 * ksq + eta * r0 * (h6 + g2 * h4) + (r0 * r0) * g0 * h5 + k * eta * g2 * h6 +
                 (g1 * h6 + g3 * h4) * k * r0);
    for (int j = 0; j < 3; j++) {
      JK(j, j) = fm1;
      JK(j, 3 + j) = gmh;
      for (int i = 0; i < 3; i++) {
        JK(j, i) = JK(j, i) + ((dfm1dxx * x0[i] + dfm1dxv * v0[i]) * x0[j] +
                               (dgmhdxx * x0[i] + dgmhdxv * v0[i]) * v0[j]);
        JK(j, 3 + i) = JK(j, 3 + i) + ((dfm1dvx * x0[i] + dfm1dvv * v0[i]) * x0[j] +
                                       (dgmhdvx * x0[i] + dgmhdvv * v0[i]) * v0[j]);
      }
      JK(j, 6) = dfm1dk * x0[j] + dgmhdk * v0[j];
      JK(j, 7) = dfm1dh * x0[j] + dgmhdh * v0[j];
      jm[j] = (G * r0inv) * (G * r0inv) * betainv * rinv * (dfm1dk2 * x0[j] - dgmhdk2 * v0[j]);
    }
    T c12 = g0 * h - g1 * r0;
    T c17 = r0 - r - g2 * k;
    T c21 = (g2 * k - r0) * (beta * c3 - k * g1 * r) * betainv * rinv2 * r0inv3 / g1 +
            eta * g1 * rinv * r0inv2 - T(2) * r0inv2;
    T c22 = rinv * ((-g1) - g0 * g2 / g1 + g2 * c2 * rinv);
    T c25 = k * rinv * r0inv2 *
            ((-g2) + k * (c13 - g2 * r0) * betainv * r0inv2 - c13 * r0inv - c12 * c3 * rinv * r0inv2 +
             c13 * c2 * c3 * rinv2 * r0inv2 -
             c13 * (k * (g2 * k + r) - g0 * r0 * zeta) * betainv * rinv * r0inv2);
    T c26 = k * rinv2 * r0inv * ((-g2) * c12 - g1 * c13 + g2 * c13 * c2 * rinv);
    T ddfdtdxx = dfdt * c21;
    T ddfdtdxv = dfdt * (c22 - h * c21);
    T ddfdtdvx = ddfdtdxv;
    T c34 = ((-beta) * (eta * eta) * (g2 * g2) - eta * k * h8 - h6 * ksq - T(2) * beta * eta * r0 * g1 * g2 +
             ((g2 * g2) - T(3) * g1 * g3) * beta * k * r0 - beta * (g1 * g1) * (r0 * r0)) *
                betainv * rinv2 +
            (eta * (g2 * g2)) * rinv / g1 + (k * h8) * betainv * rinv / g1;
    T ddfdtdvv = dfdt * (c34 - T(2) * h * c22 + hsq * c21);
    T ddfdtdk = dfdt * (T(1) / k - betainv * r0inv - c17 * betainv * rinv * r0inv -
                        c1 * (g1 * c2 - g0 * r) * rinv2 * r0inv / g1);
    T ddfdtdk2 = (-(g2 * k - r0)) * (beta * r0 * (g3 - g1 * g2) - beta * eta * (g2 * g2) + k * h3) * betainv *
                 rinv2 * r0inv;
    T ddfdtdh = dfdt * (g0 * rinv / g1 - c2 * rinv2 - (T(2) * k * r0inv - beta) * c22 - eta * c21);
    T dgdtmhdfdtm1dxx = c25;
    T dgdtmhdfdtm1dxv = c26 - h * c25;
    T dgdtmhdfdtm1dvx = c26 - h * c25;
    h2 = H2(gamma, beta, sqb);
    T c33 = d * k * rinv3 * r0inv * k * (h * g2 - r0 * g3) +
            k *
                ((-eta) * k * g1 * (g2 * g2) - g1 * g2 * g3 * ksq - r0 * eta * beta * g1 * (g2 * g2) -
                 r0 * k * g1 * h2 - beta * (g2 * g2) * g0 * (r0 * r0)) *
                betainv * rinv2 * r0inv;
    T dgdtmhdfdtm1dvv = c33 - T(2) * h * c26 + hsq * c25;
    T dgdtmhdfdtm1dk = rinv * r0inv *
                       ((-k) * (c13 - g2 * r0) * betainv * r0inv + c13 - k * c13 * c17 * betainv * rinv * r0inv +
                        k * c1 * c12 * rinv * r0inv - k * c1 * c2 * c13 * rinv2 * r0inv);
    T dgdtmhdfdtm1dk2 =
        k * betainv * rinv2 * r0inv *
        ((-beta) * (eta * eta) * pow4(g2) + eta * g2 * (g1 * (g2 * g2) + (g1 * g1) * g3 - T(5) * g2 * g3) * k +
         g2 * g3 * h3 * ksq + T(2) * eta * r0 * beta * (g2 * g2) * (g3 - g1 * g2) +
         (T(4) * g3 - g0 * g3 - g1 * g2) * (g3 - g1 * g2) * r0 * k +
         beta * (T(2) * g1 * g3 * g2 - (g1 * g1) * (g2 * g2) - (g3 * g3)) * (r0 * r0));
    T dgdtmhdfdtm1dh = g1 * k * rinv * r0inv + k * c12 * rinv2 * r0inv - k * c2 * c13 * rinv3 * r0inv -
                       (T(2) * k * r0inv - beta) * c26 - eta * c25;
    for (int j = 0; j < 3; j++) {
      JK(3 + j, j) = dfdt;
      JK(3 + j, 3 + j) = dgdtm1;
      for (int i = 0; i < 3; i++) {
        JK(3 + j, i) = JK(3 + j, i) + ((ddfdtdxx * x0[i] + ddfdtdxv * v0[i]) * x0[j] +
                                       (dgdtmhdfdtm1dxx * x0[i] + dgdtmhdfdtm1dxv * v0[i]) * v0[j]);
        JK(3 + j, 3 + i) = JK(3 + j, 3 + i) + ((ddfdtdvx * x0[i] + ddfdtdvv * v0[i]) * x0[j] +
                                               (dgdtmhdfdtm1dvx * x0[i] + dgdtmhdfdtm1dvv * v0[i]) * v0[j]);
      }
      JK(3 + j, 6) = ddfdtdk * x0[j] + dgdtmhdfdtm1dk * v0[j];
      JK(3 + j, 7) = ddfdtdh * x0[j] + dgdtmhdfdtm1dh * v0[j];
      jm[3 + j] = G * G * r0inv * rinv * (ddfdtdk2 * x0[j] + dgdtmhdfdtm1dk2 * v0[j]);
    }
  } else {
    T d = (h + eta * g2 + T(2) * k * g3) * betainv;
    T c1 = d - r0 * g3;
    T c2 = eta * g0 + g1 * zeta;
    T c3 = d * k + g1 * (r0 * r0);
    T c14 = r0 * g2 - k * h1;
    T c15 = eta * h1 + h2 * r0;
    T c16 = eta * h2 + g1 * gamma * r0 / sqb;
    T c17 = r0 - r - g2 * k;
    T c19 = T(4) * eta * h1 + T(3) * h2 * r0;
    T c23 = h2 * k - r0 * g1;
    T h6 = H6(gamma, beta);
    T h3 = H3(gamma, beta, sqb);
    T h5 = H5(gamma, beta, sqb);
    T h8 = (-(T(2) * h3)) + T(3) * h5;
    T dfm1dxx = k * rinv3 * betainv * pow4(r0inv) *
                (k * h1 * (r * r) * r0 * (beta - T(2) * k * r0inv) + beta * c3 * (r * c23 + c14 * c2) +
                 c14 * r * (k * (r - g2 * k) + g0 * r0 * zeta));
    T dfm1dxv = k * rinv2 * r0inv * (k * (g2 * h2 + g1 * h1) - T(2) * g1 * g2 * r0 + g2 * c14 * c2 * rinv);
    T dfm1dvx = dfm1dxv;
    T dfm1dvv =
        k * r0inv * rinv2 * betainv *
        (T(2) * eta * k * (g2 * g3 - g1 * h1) + (T(3) * g3 * h2 - T(4) * h1 * g2) * ksq +
         beta * g2 * r0 * (T(3) * h1 * k - g2 * r0) +
         c14 * rinv *
             ((-beta) * (g2 * g2) * (eta * eta) + eta * k * (T(2) * g0 * g3 - h2) - h6 * ksq +
              ((-(T(2) * eta)) * g1 * g2 + k * (h1 - T(2) * g1 * g3)) * beta * r0 - beta * (g1 * g1) * (r0 * r0)));
    T dfm1dh = (g1 * k - h2 * ksq * r0inv - k * c14 * c2 * rinv * r0inv) * rinv2;
    T dfm1dk = rinv * r0inv *
               (T(4) * h1 * ksq * betainv * r0inv - k * h1 - T(2) * g2 * k * betainv + c14 -
                k * c14 * c17 * betainv * rinv * r0inv + k * (g1 * r0 - k * h2) * c1 * rinv * r0inv -
                k * c14 * c1 * c2 * rinv2 * r0inv);
    T dfm1dk2 =
        betainv * r0inv * rinv2 *
        (r * (T(2) * eta * k * (g1 * h1 - g3 * g2) + (T(4) * g2 * h1 - T(3) * g3 * h2) * ksq -
              eta * r0 * beta * g1 * h1 + (g3 * h2 - T(4) * g2 * h1) * beta * k * r0 +
              g2 * h1 * (beta * beta) * (r0 * r0)) -
         c14 * ((-(eta * eta)) * beta * (g2 * g2) - k * eta * h8 - ksq * h6 - eta * r0 * beta * (g1 * g2 + g0 * g3) +
                T(2) * (h1 - g1 * g3) * beta * k * r0 - (g2 - beta * g1 * g3) * beta * (r0 * r0)));
    T dgmhdxx = k * rinv * r0inv *
                (h2 + k * c19 * betainv * r0inv2 - c16 * c3 * rinv * r0inv2 +
                 c2 * c3 * c15 * ((rinv * r0inv) * (rinv * r0inv)) -
                 c15 * (k * (g2 * k + r) - g0 * r0 * zeta) * betainv * rinv * r0inv2);
    T dgmhdxv = k * rinv2 * (h1 * r - g2 * c16 - g1 * c15 + g2 * c2 * c15 * rinv);
    T dgmhdvx = dgmhdxv;
    T dgmhdvv =
        k * betainv * rinv2 *
        (T(2) * (eta * eta) * (g1 * h1 - g2 * g3) + eta * k * (T(4) * g2 * h1 - T(3) * h2 * g3) +
         r0 * eta * (T(4) * g0 * h1 - T(2) * g1 * g3) + T(3) * r0 * k * ((g1 + beta * g3) * h1 - g3 * g2) +
         (g0 * h8 - beta * g1 * ((g2 * g2) + g1 * g3)) * (r0 * r0) -
         c15 * rinv *
             (beta * (g2 * g2) * (eta * eta) + eta * k * h8 + h6 * ksq +
              (T(2) * eta * g1 * g2 - k * ((g2 * g2) - T(3) * g1 * g3)) * beta * r0 + beta * (g1 * g1) * (r0 * r0)));
    T dgmhdk = rinv * (k * c1 * c16 * rinv * r0inv + c15 - k * c15 * c17 * betainv * rinv * r0inv -
                       k * c19 * betainv * r0inv - k * c1 * c2 * c15 * rinv2 * r0inv);
    T h7 = beta * g1 * (g2 * g2) - g0 * h8;
    T dgmhdk2 =
        betainv * rinv2 *
        (r * (T(2) * (eta * eta) * (g3 * g2 - g1 * h1) + eta * k * (T(3) * g3 * h2 - T(4) * g2 * h1) +
              r0 * eta * (beta * g3 * (g1 * g2 + g0 * g3) - T(2) * g0 * h6) +
              ((-h6) * (g1 + beta * g3) + g2 * (T(2) * g3 - h2)) * r0 * k +
              (h7 - (beta * beta) * g1 * (g3 * g3)) * (r0 * r0)) -
         c15 * ((-beta) * (eta * eta) * (g2 * g2) + eta * k * ((-h2) + T(2) * g0 * g3) - h6 * ksq -
                r0 * eta * beta * (h2 + T(2) * g0 * g3) + T(2) * beta * (T(2) * h1 - (g2 * g2)) * r0 * k +
                beta * (beta * g1 * g3 - g2) * (r0 * r0)));
    T dgmhdh = k * rinv3 * (r * c16 - c2 * c15);
    for (int j = 0; j < 3; j++) {
      JK(j, j) = fm1;
      JK(j, 3 + j) = gmh;
      for (int i = 0; i < 3; i++) {
        JK(j, i) = JK(j, i) + ((dfm1dxx * x0[i] + dfm1dxv * v0[i]) * x0[j] +
                               (dgmhdxx * x0[i] + dgmhdxv * v0[i]) * v0[j]);
        JK(j, 3 + i) = JK(j, 3 + i) + ((dfm1dvx * x0[i] + dfm1dvv * v0[i]) * x0[j] +
                                       (dgmhdvx * x0[i] + dgmhdvv * v0[i]) * v0[j]);
      }
      JK(j, 6) = dfm1dk * x0[j] + dgmhdk * v0[j];
      JK(j, 7) = dfm1dh * x0[j] + dgmhdh * v0[j];
      jm[j] = G * G * rinv * r0inv * (dfm1dk2 * x0[j] + dgmhdk2 * v0[j]);
    }
    T ddfdtdxx = dfdt *
                 (eta * g1 * rinv - T(2) - g0 * c3 * rinv * r0inv / g1 + c2 * c3 * r0inv * rinv2 -
                  k * (k * g2 - r0) * betainv * rinv * r0inv) *
                 r0inv2;
    T ddfdtdxv = (-dfdt) * (g0 * g2 / g1 + (r0 * g1 + eta * g2) * rinv) * rinv;
    T ddfdtdvx = ddfdtdxv;
    T ddfdtdvv = (-k) * rinv3 * r0inv * betainv *
                 ((beta * eta * (g2 * g2) + k * h8) * (r0 * g0 + k * g2) +
                  g1 * ((-h6) * ksq + ((-(T(2) * eta)) * g1 * g2 + (h1 - T(2) * g1 * g3) * k) * beta * r0 -
                        beta * (g1 * g1) * (r0 * r0)));
    T ddfdtdk = dfdt * (T(1) / k + c1 * (r0 - g2 * k) * r0inv * rinv2 / g1 - betainv * r0inv * (T(1) + c17 * rinv));
    T ddfdtdk2 = (r0 - g2 * k) * betainv * r0inv * rinv2 *
                 ((-eta) * beta * (g2 * g2) + h3 * k + (g3 - g1 * g2) * beta * r0);
    T ddfdtdh = dfdt * (r0 - g2 * k) * rinv2 / g1;
    T dgdotm1dxx = rinv2 * r0inv3 *
                   ((eta * g2 + g1 * r0) * k * c3 * rinv + g2 * k * (k * (g2 * k - r) - g0 * r0 * zeta) * betainv);
    T dgdotm1dxv = k * g2 * rinv3 * (r * g1 + r0 * g1 + eta * g2);
    T dgdotm1dvx = dgdotm1dxv;
    T dgdotm1dvv = k * betainv * rinv3 *
                   ((eta * eta) * beta * (g2 * g2 * g2) - eta * k * g2 * h3 + T(3) * r0 * eta * beta * g1 * (g2 * g2) +
                    r0 * k * ((-g0) * h6 + T(3) * beta * g1 * g2 * g3) + beta * g2 * (g0 * g2 + (g1 * g1)) * (r0 * r0));
    T dgdotm1dk = rinv * r0inv *
                  ((-r0) * g2 + g2 * k * (r + r0 - g2 * k) * betainv * rinv - k * g1 * c1 * rinv +
                   k * g2 * c1 * c2 * rinv2);
    T dgdotm1dk2 = betainv * rinv2 *
                   ((-beta) * (eta * eta) * (g2 * g2 * g2) + eta * k * g2 * h3 +
                    eta * r0 * beta * g2 * (g3 - T(2) * g1 * g2) + (h6 - beta * (g2 * g2 * g2)) * r0 * k +
                    beta * g1 * (g3 - g1 * g2) * (r0 * r0));
    T dgdotm1dh = k * rinv3 * (g2 * c2 - r * g1);
    for (int j = 0; j < 3; j++) {
      JK(3 + j, j) = dfdt;
      JK(3 + j, 3 + j) = dgdtm1;
      for (int i = 0; i < 3; i++) {
        JK(3 + j, i) = JK(3 + j, i) + ((ddfdtdxx * x0[i] + ddfdtdxv * v0[i]) * x0[j] +
                                       (dgdotm1dxx * x0[i] + dgdotm1dxv * v0[i]) * v0[j]);
        JK(3 + j, 3 + i) = JK(3 + j, 3 + i) + ((ddfdtdvx * x0[i] + ddfdtdvv * v0[i]) * x0[j] +
                                               (dgdotm1dvx * x0[i] + dgdotm1dvv * v0[i]) * v0[j]);
      }
      JK(3 + j, 6) = ddfdtdk * x0[j] + dgdotm1dk * v0[j];
      JK(3 + j, 7) = ddfdtdh * x0[j] + dgdotm1dh * v0[j];
      jm[3 + j] = G * G * rinv * r0inv * (ddfdtdk2 * x0[j] + dgdotm1dk2 * v0[j]);
    }
  }
}

// kepler_driftij_gamma! with Jacobian (ahl21.jl:706-760)
template <class T> void kepler_driftij_gamma(State<T>& s, Derivs<T>& d, int i, int j, T h, bool drift_first) {
  const T G = T(GNEWT_D);
  for (int k = 0; k < 3; k++) {
    s.x0[k] = s.X(k, i) - s.X(k, j);
    s.v0[k] = s.V(k, i) - s.V(k, j);
  }
  T gm = G * (s.m[i] + s.m[j]);
  if (gm == T(0)) return;
  std::fill(d.jac_ij.begin(), d.jac_ij.end(), T(0));
  for (int q = 0; q < 6; q++) s.delxv[q] = T(0);
  std::fill(d.jac_kepler.begin(), d.jac_kepler.end(), T(0));
  std::fill(d.jac_mass.begin(), d.jac_mass.end(), T(0));
  KepParams<T> P = jac_delxv_gamma(s, gm, h, drift_first);
  compute_jacobian_gamma(P, s.x0, s.v0, d.jac_kepler.data(), d.jac_mass.data(), drift_first);
  T mijinv = T(1) / (s.m[i] + s.m[j]);
  T mi = s.m[i] * mijinv, mj = s.m[j] * mijinv;
  for (int k = 0; k < 3; k++) {
    comp_sum(s.X(k, i), s.XE(k, i), mj * s.delxv[k]);
    comp_sum(s.X(k, j), s.XE(k, j), (-mi) * s.delxv[k]);
  }
  for (int k = 0; k < 3; k++) {
    comp_sum(s.V(k, i), s.VE(k, i), mj * s.delxv[3 + k]);
    comp_sum(s.V(k, j), s.VE(k, j), (-mi) * s.delxv[3 + k]);
  }
  for (int l = 0; l < 6; l++)
    for (int k = 0; k < 6; k++) {
      d.ij(k, l) += mj * d.kep(k, l);
      d.ij(k, 7 + l) -= mj * d.kep(k, l);
      d.ij(7 + k, l) -= mi * d.kep(k, l);
      d.ij(7 + k, 7 + l) += mi * d.kep(k, l);
    }
  for (int k = 0; k < 6; k++) {
    d.ij(k, 6) = d.jac_mass[k] * s.m[j];
    d.ij(k, 13) = mi * s.delxv[k] * mijinv + G * mj * d.kep(k, 6);
    d.ij(7 + k, 6) = (-mj) * s.delxv[k] * mijinv - G * mi * d.kep(k, 6);
    d.ij(7 + k, 13) = (-d.jac_mass[k]) * s.m[i];
  }
  for (int k = 0; k < 6; k++) {
    d.dqdt_ij[k] = mj * d.kep(k, 7);
    d.dqdt_ij[7 + k] = (-mi) * d.kep(k, 7);
  }
}

// One forward/backward pair update of ahl21! (ahl21.jl:29-44 and :60-77).
template <class T> void pair_update(State<T>& s, Derivs<T>& d, int i, int j, T h2, bool drift_first) {
  int M = 7 * s.n, indi = 7 * i, indj = 7 * j;
  kepler_driftij_gamma(s, d, i, j, h2, drift_first);
  copy_submatrix(s, d, indi, indj);
  mul(d.jac_tmp2.data(), d.jac_ij.data(), d.jac_tmp1.data(), 14, 14, M);
  comp_sum_matrix(d.jac_tmp1.data(), d.jac_err1.data(), d.jac_tmp2.data(), (size_t)14 * M);
  for (int q = 0; q < 14; q++) d.dqdt_ij[q] = d.dqdt_ij[q] * T(0.5);
  mul(d.tmp14.data(), d.jac_ij.data(), d.dqdt_tmp1.data(), 14, 14, 1);
  for (int q = 0; q < 14; q++) d.dqdt_ij[q] = d.dqdt_ij[q] + (d.dqdt_tmp1[q] + d.tmp14[q]);
  ypoc_submatrix(s, d, indi, indj);
}

// ahl21!(s, d::Derivatives, h) (ahl21.jl:5-95)
template <class T> void ahl21(State<T>& s, Derivs<T>& d, T h) {
  int n = s.n, M = 7 * n;
  size_t MM = (size_t)M * M;
  T half = T(0.5), two = T(2);
  T h2 = half * h, h6 = h / T(6);
  d.zero();
  std::fill(s.dqdt.begin(), s.dqdt.end(), T(0));
  kickfast(s, d, h6);
  for (int q = 0; q < M; q++) d.dqdt_kick[q] = d.dqdt_kick[q] / T(6);
  mul(d.tmp7n.data(), d.jac_kick.data(), s.dqdt.data(), M, M, 1);
  for (int q = 0; q < M; q++) s.dqdt[q] = s.dqdt[q] + (d.dqdt_kick[q] + d.tmp7n[q]);
  mul(d.jac_copy.data(), d.jac_kick.data(), s.jac_step.data(), M, M, M);
  drift_grad(s, h2);
  for (int i = 0; i < n; i++)
    for (int k = 0; k < 3; k++) s.dqdt[7 * i + k] = half * s.V(k, i) + h2 * s.dqdt[7 * i + 3 + k];
  comp_sum_matrix(s.jac_step.data(), s.jac_error.data(), d.jac_copy.data(), MM);
  for (int i = 0; i < n - 1; i++)
    for (int j = i + 1; j < n; j++)
      if (!s.P(i, j)) pair_update(s, d, i, j, h2, true);
  phic(s, d, h);
  phisalpha(s, d, h, two);
  mul(d.jac_copy.data(), d.jac_phi.data(), s.jac_step.data(), M, M, M);
  mul(d.tmp7n.data(), d.jac_phi.data(), s.dqdt.data(), M, M, 1);
  for (int q = 0; q < M; q++) s.dqdt[q] = s.dqdt[q] + (d.dqdt_phi[q] + d.tmp7n[q]);
  comp_sum_matrix(s.jac_step.data(), s.jac_error.data(), d.jac_copy.data(), MM);
  for (int i = n - 2; i >= 0; i--)
    for (int j = n - 1; j > i; j--)
      if (!s.P(i, j)) pair_update(s, d, i, j, h2, false);
  drift_grad(s, h2);
  for (int i = 0; i < n; i++)
    for (int k = 0; k < 3; k++)
      s.dqdt[7 * i + k] = s.dqdt[7 * i + k] + (half * s.V(k, i) + h2 * s.dqdt[7 * i + 3 + k]);
  std::fill(d.dqdt_kick.begin(), d.dqdt_kick.end(), T(0));
  kickfast(s, d, h6);
  for (int q = 0; q < M; q++) d.dqdt_kick[q] = d.dqdt_kick[q] / T(6);
  mul(d.tmp7n.data(), d.jac_kick.data(), s.dqdt.data(), M, M, 1);
  for (int q = 0; q < M; q++) s.dqdt[q] = s.dqdt[q] + (d.dqdt_kick[q] + d.tmp7n[q]);
  mul(d.jac_copy.data(), d.jac_kick.data(), s.jac_step.data(), M, M, M);
  comp_sum_matrix(s.jac_step.data(), s.jac_error.data(), d.jac_copy.data(), MM);
}

// ---------------------------------------------------------- no-grad variant
// drift! (ahl21_no_grad.jl:24-29)
template <class T> void drift_ng(State<T>& s, T h) {
  for (int i = 0; i < s.n; i++)
    for (int j = 0; j < 3; j++) comp_sum(s.X(j, i), s.XE(j, i), h * s.V(j, i));
}
// kickfast! (ahl21_no_grad.jl:35-56)
template <class T> void kickfast_ng(State<T>& s, T h) {
  const T G = T(GNEWT_D);
  for (int k = 0; k < 3; k++) s.rij[k] = T(0);
  for (int i = 0; i < s.n - 1; i++)
    for (int j = i + 1; j < s.n; j++) {
      if (!s.P(i, j)) continue;
      for (int k = 0; k < 3; k++) s.rij[k] = s.X(k, i) - s.X(k, j);
      T r2inv = T(1) / dot3(s.rij, s.rij);
      T r3inv = r2inv * Mth<T>::sqrt(r2inv);
      T fac2 = h * G * r3inv;
      for (int k = 0; k < 3; k++) {
        T fac = fac2 * s.rij[k];
        comp_sum(s.V(k, i), s.VE(k, i), (-s.m[j]) * fac);
        comp_sum(s.V(k, j), s.VE(k, j), s.m[i] * fac);
      }
    }
}
// phic! (ahl21_no_grad.jl:62-104)
template <class T> void phic_ng(State<T>& s, T h) {
  const T G = T(GNEWT_D);
  std::fill(s.a.begin(), s.a.end(), T(0));
  for (int k = 0; k < 3; k++) s.rij[k] = s.aij[k] = T(0);
  for (int i = 0; i < s.n - 1; i++)
    for (int j = i + 1; j < s.n; j++) {
      if (!s.P(i, j)) continue;
      for (int k = 0; k < 3; k++) s.rij[k] = s.X(k, i) - s.X(k, j);
      T r2inv = T(1) / dot3(s.rij, s.rij);
      T r3inv = r2inv * Mth<T>::sqrt(r2inv);
      for (int k = 0; k < 3; k++) {
        T fac = G * s.rij[k] * r3inv;
        T facv = fac * T(2) * h / T(3);
        comp_sum(s.V(k, i), s.VE(k, i), (-s.m[j]) * facv);
        comp_sum(s.V(k, j), s.VE(k, j), s.m[i] * facv);
        s.A(k, i) = s.A(k, i) - s.m[j] * fac;
        s.A(k, j) = s.A(k, j) + s.m[i] * fac;
      }
    }
  T coeff = h * h * h / T(36) * G;
  for (int i = 0; i < s.n - 1; i++)
    for (int j = i + 1; j < s.n; j++) {
      if (!s.P(i, j)) continue;
      for (int k = 0; k < 3; k++) {
        s.aij[k] = s.A(k, i) - s.A(k, j);
        s.rij[k] = s.X(k, i) - s.X(k, j);
      }
      T r2 = dot3(s.rij, s.rij);
      T r1 = Mth<T>::sqrt(r2);
      T ardot = dot3(s.aij, s.rij);
      T fac1 = coeff / (r2 * r2 * r1);
      T fac2 = T(3) * ardot;
      for (int k = 0; k < 3; k++) {
        T fac = fac1 * (s.rij[k] * fac2 - r2 * s.aij[k]);
        comp_sum(s.V(k, i), s.VE(k, i), s.m[j] * fac);
        comp_sum(s.V(k, j), s.VE(k, j), (-s.m[i]) * fac);
      }
    }
}
// phisalpha! (ahl21_no_grad.jl:110-158)
template <class T> void phisalpha_ng(State<T>& s, T h, T alpha) {
  const T G = T(GNEWT_D);
  std::fill(s.a.begin(), s.a.end(), T(0));
  for (int k = 0; k < 3; k++) s.rij[k] = s.aij[k] = T(0);
  T coeff = alpha * (h * h * h) / T(96) * T(2) * G;
  for (int i = 0; i < s.n - 1; i++)
    for (int j = i + 1; j < s.n; j++) {
      if (s.P(i, j)) continue;
      for (int k = 0; k < 3; k++) s.rij[k] = s.X(k, i) - s.X(k, j);
      T r2 = dot3(s.rij, s.rij);
      T r3 = r2 * Mth<T>::sqrt(r2);
      T fac2 = G / r3;
      for (int k = 0; k < 3; k++) {
        T fac = fac2 * s.rij[k];
        s.A(k, i) = s.A(k, i) - s.m[j] * fac;
        s.A(k, j) = s.A(k, j) + s.m[i] * fac;
      }
    }
  for (int i = 0; i < s.n - 1; i++)
    for (int j = i + 1; j < s.n; j++) {
      if (s.P(i, j)) continue;
      for (int k = 0; k < 3; k++) {
        s.aij[k] = s.A(k, i) - s.A(k, j);
        s.rij[k] = s.X(k, i) - s.X(k, j);
      }
      T r2 = dot3(s.rij, s.rij);
      T r1 = Mth<T>::sqrt(r2);
      T ardot = dot3(s.aij, s.rij);
      T fac1 = coeff / (r2 * r2 * r1);
      T fac2 = T(2) * G * (s.m[i] + s.m[j]) / r1 + T(3) * ardot;
      for (int k = 0; k < 3; k++) {
        T fac = fac1 * (s.rij[k] * fac2 - r2 * s.aij[k]);
        comp_sum(s.V(k, i), s.VE(k, i), s.m[j] * fac);
        comp_sum(s.V(k, j), s.VE(k, j), (-s.m[i]) * fac);
      }
    }
}
// kepler_driftij_gamma! without Jacobian (ahl21_no_grad.jl:192-212)
template <class T> void kepler_driftij_ng(State<T>& s, int i, int j, T h, bool drift_first) {
  const T G = T(GNEWT_D);
  for (int k = 0; k < 3; k++) {
    s.x0[k] = s.X(k, i) - s.X(k, j);
    s.v0[k] = s.V(k, i) - s.V(k, j);
  }
  T gm = G * (s.m[i] + s.m[j]);
  if (gm == T(0)) return;
  jac_delxv_gamma(s, gm, h, drift_first);
  T mijinv = T(1) / (s.m[i] + s.m[j]);
  T mi = s.m[i] * mijinv, mj = s.m[j] * mijinv;
  for (int k = 0; k < 3; k++) {
    comp_sum(s.X(k, i), s.XE(k, i), mj * s.delxv[k]);
    comp_sum(s.X(k, j), s.XE(k, j), (-mi) * s.delxv[k]);
    comp_sum(s.V(k, i), s.VE(k, i), mj * s.delxv[3 + k]);
    comp_sum(s.V(k, j), s.VE(k, j), (-mi) * s.delxv[3 + k]);
  }
}
// ahl21!(s, h) without Jacobian (ahl21_no_grad.jl:6-18).  kick_den and alpha
// are the method's constants (the outer kicks take h/6, phisalpha! alpha = 2);
// only the order-of-accuracy pin passes other values, to show that the
// convergence test detects a wrong coefficient.
template <class T> void ahl21_ng(State<T>& s, T h, T kick_den = T(6), T alpha = T(2)) {
  T h2 = T(0.5) * h, h6 = h / kick_den;
  kickfast_ng(s, h6);
  drift_ng(s, h2);
  for (int i = 0; i < s.n - 1; i++)  // drift_kepler! (:164-172)
    for (int j = i + 1; j < s.n; j++)
      if (!s.P(i, j)) kepler_driftij_ng(s, i, j, h2, true);
  phic_ng(s, h);
  phisalpha_ng(s, h, alpha);
  for (int i = s.n - 2; i >= 0; i--)  // kepler_drift! (:178-186)
    for (int j = s.n - 1; j > i; j--)
      if (!s.P(i, j)) kepler_driftij_ng(s, i, j, h2, false);
  drift_ng(s, h2);
  kickfast_ng(s, h6);
}

}  // namespace nbgo
