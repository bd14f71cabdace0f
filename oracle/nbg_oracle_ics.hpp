// nbg_oracle_ics.hpp -- TEST INFRASTRUCTURE ONLY (parity oracle; see
// nbg_oracle.hpp).  Restates the initial-condition path ElementsIC ->
// init_nbody: src/ics/InitialConditions.jl:142-161, src/ics/init_nbody.jl:13-229,
// src/ics/kepler_init.jl:66-210, src/ics/kepler.jl:1-41 and the fully nested
// hierarchy that src/ics/setup_hierarchy.jl:9-145 builds for H = N.
#pragma once

namespace nbgo {

template <class T> struct M3 {
  T a[9];  // col-major 3x3
  T& operator()(int i, int j) { return a[i + 3 * j]; }
  T operator()(int i, int j) const { return a[i + 3 * j]; }
};
template <class T> M3<T> mm3(const M3<T>& A, const M3<T>& B) {
  M3<T> C;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) C(i, j) = A(i, 0) * B(0, j) + A(i, 1) * B(1, j) + A(i, 2) * B(2, j);
  return C;
}
template <class T> void mv3(const M3<T>& A, const T* x, T* y) {
  for (int i = 0; i < 3; i++) y[i] = A(i, 0) * x[0] + A(i, 1) * x[1] + A(i, 2) * x[2];
}
template <class T> M3<T> ms3(const M3<T>& A, T s) {
  M3<T> C;
  for (int q = 0; q < 9; q++) C.a[q] = A.a[q] * s;
  return C;
}
template <class T> M3<T> md3(const M3<T>& A, T s) {
  M3<T> C;
  for (int q = 0; q < 9; q++) C.a[q] = A.a[q] / s;
  return C;
}
template <class T> M3<T> mk3(T a11, T a12, T a13, T a21, T a22, T a23, T a31, T a32, T a33) {
  M3<T> C;
  C(0, 0) = a11; C(0, 1) = a12; C(0, 2) = a13;
  C(1, 0) = a21; C(1, 1) = a22; C(1, 2) = a23;
  C(2, 0) = a31; C(2, 1) = a32; C(2, 2) = a33;
  return C;
}

// Julia mod(x, y) for floats: rem, then shift into the sign of y.
template <class T> T jmod(T x, T y) {
  T r = Mth<T>::fmod(x, y);
  if (r == T(0)) return (y < T(0)) ? -T(0) : T(0);
  if ((r > T(0)) != (y > T(0))) return r + y;
  return r;
}

// ekepler (kepler.jl:1-41): eccentric anomaly from mean anomaly m.
template <class T> T ekepler(T m, T ecc) {
  if (m == T(0)) return T(0);
  T pi2 = T(2) * Mth<T>::pi();
  T ms = jmod(m, pi2);
  T de0 = ecc * T(0.85) * jsign(ms);
  T de1 = T(2) * de0, de2 = T(3) * de0;
  int iter = 0;
  const int ITMAX = 20;
  while (true) {
    de2 = de1;
    de1 = de0;
    T f3 = ecc * Mth<T>::cos(de0 + ms);
    T f2 = ecc * Mth<T>::sin(de0 + ms);
    de0 = (f2 - de1 * f3) / (T(1) - f3);
    iter += 1;
    if (iter >= ITMAX || de0 == de1 || de0 == de2) break;
  }
  return de0 + m;
}

// kepler_init with Jacobian (kepler_init.jl:66-210).  el = (P, t0, ecosw,
// esinw, I, Omega); jac is 7x7 col-major d(x,v,m)/d(el,m).
template <class T> void kepler_init(T time, T mass, const T* el, T* x, T* v, T* jac) {
  const T G = T(GNEWT_D), third = T(THIRD_D), pi = Mth<T>::pi();
  T period = el[0];
  T n = T(2) * pi / period;
  T t0 = el[1];
  T semi = Mth<T>::cbrt(G * mass * (period * period) / T(4) / (pi * pi));
  T dsemidp = T(2) * third * semi / period;
  T dsemidm = third * semi / mass;
  T ecosomega = el[2], esinomega = el[3];
  T ecc = Mth<T>::sqrt(esinomega * esinomega + ecosomega * ecosomega);
  T deccdecos = (ecc != T(0)) ? ecosomega / ecc : T(0);
  T deccdesin = (ecc != T(0)) ? esinomega / ecc : T(0);
  T sqrt1mecc2 = Mth<T>::sqrt(T(1) - ecc * ecc);
  T den1 = esinomega - ecosomega - ecc;
  T tp;
  if (ecc == T(0)) tp = t0 - T(3) * period / T(4);
  else
    tp = (t0 - sqrt1mecc2 / n * ecosomega / (T(1) - esinomega) -
          T(2) / n *
              Mth<T>::atan2(Mth<T>::sqrt(T(1) - ecc) * (esinomega + ecosomega + ecc), Mth<T>::sqrt(T(1) + ecc) * den1));
  T dtpdp = (tp - t0) / period;
  T fac = Mth<T>::sqrt((T(1) - ecc) / (T(1) + ecc));
  T den2 = T(1) / (den1 * den1);
  T theta = fac * (esinomega + ecosomega + ecc) / den1;
  T dthetadecc = ((ecc + ecosomega) * (ecc + ecosomega) + T(2) * (T(1) - ecc * ecc) * esinomega -
                  esinomega * esinomega) /
                 (sqrt1mecc2 * (T(1) + ecc)) * den2;
  T dthetadecos = T(2) * fac * esinomega * den2;
  T dthetadesin = (-(T(2) * fac)) * (ecosomega + ecc) * den2;
  T dtpdecc = ecc / sqrt1mecc2 / n * ecosomega / (T(1) - esinomega) - T(2) / n / (T(1) + theta * theta) * dthetadecc;
  T dtpdecos = dtpdecc * deccdecos - sqrt1mecc2 / n / (T(1) - esinomega) - T(2) / n / (T(1) + theta * theta) * dthetadecos;
  T dtpdesin = dtpdecc * deccdesin - sqrt1mecc2 / n * ecosomega / ((T(1) - esinomega) * (T(1) - esinomega)) -
               T(2) / n / (T(1) + theta * theta) * dthetadesin;
  T dtpdt0 = T(1);
  T m = n * (time - tp);
  T dmdp = -m / period;
  T dmdtp = -n;
  T ekep = ekepler(m, ecc);
  T cosekep = Mth<T>::cos(ekep), sinekep = Mth<T>::sin(ekep);
  T r = semi * (T(1) - ecc * cosekep);
  T denom = semi / r;
  T dekepdecos = sinekep * denom * deccdecos;
  T dekepdesin = sinekep * denom * deccdesin;
  T dekepdm = denom;
  T inc = el[4], capomega = el[5];
  T coscapomega = Mth<T>::cos(capomega), sincapomega = Mth<T>::sin(capomega);
  T cosomega = (ecc != T(0)) ? ecosomega / ecc : T(1);
  T sinomega = (ecc != T(0)) ? esinomega / ecc : T(0);
  T cosinc = Mth<T>::cos(inc), sininc = Mth<T>::sin(inc);
  M3<T> P1 = mk3<T>(cosomega, -sinomega, 0, sinomega, cosomega, 0, 0, 0, 1);
  M3<T> P2 = mk3<T>(1, 0, 0, 0, cosinc, -sininc, 0, sininc, cosinc);
  M3<T> P3 = mk3<T>(coscapomega, -sincapomega, 0, sincapomega, coscapomega, 0, 0, 0, 1);
  M3<T> P32 = mm3(P3, P2);
  M3<T> P321 = mm3(P32, P1);
  T xplane[3] = {semi * (cosekep - ecc), semi * (sqrt1mecc2 * sinekep), T(0)};
  T vplane[3] = {-sinekep, sqrt1mecc2 * cosekep, T(0)};
  mv3(P321, xplane, x);
  T dxda[3], dxdekep[3], dxdecc[3], dxdecos[3], dxdesin[3], dxdinc[3], dxdcom[3], tmp[3], tmp2[3];
  for (int q = 0; q < 3; q++) dxda[q] = x[q] / semi;
  mv3(ms3(P321, semi), vplane, dxdekep);
  {
    T vv[3] = {cosekep, sinekep / sqrt1mecc2, T(0)};
    M3<T> A = md3(ms3(ms3(P321, T(-1)), semi), ecc);
    mv3(A, vv, dxdecc);
  }
  mv3(md3(P32, ecc), xplane, tmp);
  for (int q = 0; q < 3; q++) dxdecos[q] = dxdecc[q] * deccdecos + tmp[q];
  {
    T vv[3] = {-xplane[1], xplane[0], T(0)};
    mv3(md3(P32, ecc), vv, tmp);
  }
  for (int q = 0; q < 3; q++) dxdesin[q] = dxdecc[q] * deccdesin + tmp[q];
  M3<T> Dinc = mk3<T>(0, 0, 0, 0, -sininc, -cosinc, 0, cosinc, -sininc);
  M3<T> Dcom = mk3<T>(-sincapomega, -coscapomega, 0, coscapomega, -sincapomega, 0, 0, 0, 0);
  mv3(mm3(mm3(P3, Dinc), P1), xplane, dxdinc);
  mv3(mm3(mm3(Dcom, P2), P1), xplane, dxdcom);
  T nsd = n * semi * denom;
  mv3(ms3(P321, nsd), vplane, v);
  T dvda[3], dvdp[3], dvdekep[3], dvdecc[3], dvdecos[3], dvdesin[3], dvdinc[3], dvdcom[3];
  for (int q = 0; q < 3; q++) { dvda[q] = v[q] / semi; dvdp[q] = -v[q] / period; }
  {
    T vv[3] = {-cosekep, -sqrt1mecc2 * sinekep, T(0)};
    mv3(ms3(P321, nsd), vv, tmp);
    for (int q = 0; q < 3; q++) dvdekep[q] = (-v[q]) * ecc * sinekep * denom + tmp[q];
  }
  {
    T vv[3] = {T(0), -ecc / sqrt1mecc2 * cosekep, T(0)};
    mv3(ms3(P321, nsd), vv, tmp);
    for (int q = 0; q < 3; q++) dvdecc[q] = -v[q] / ecc + v[q] * cosekep * denom + tmp[q];
  }
  mv3(md3(ms3(P32, nsd), ecc), vplane, tmp);
  for (int q = 0; q < 3; q++) dvdecos[q] = dvdecc[q] * deccdecos + tmp[q];
  {
    T vv[3] = {-vplane[1], vplane[0], T(0)};
    mv3(md3(ms3(P32, nsd), ecc), vv, tmp);
  }
  for (int q = 0; q < 3; q++) dvdesin[q] = dvdecc[q] * deccdesin + tmp[q];
  mv3(ms3(mm3(mm3(P3, Dinc), P1), nsd), vplane, dvdinc);
  mv3(ms3(mm3(mm3(Dcom, P2), P1), nsd), vplane, dvdcom);
  (void)tmp2;
  for (int q = 0; q < 49; q++) jac[q] = T(0);
  auto J = [&](int a, int b) -> T& { return jac[a + 7 * b]; };
  for (int q = 0; q < 3; q++) {
    J(q, 0) = dxda[q] * dsemidp + dxdekep[q] * dekepdm * (dmdp + dmdtp * dtpdp);
    J(q, 1) = dxdekep[q] * dekepdm * dmdtp * dtpdt0;
    J(q, 2) = (ecc != T(0)) ? dxdecos[q] + dxdekep[q] * (dekepdm * dmdtp * dtpdecos + dekepdecos) : T(0);
    J(q, 3) = (ecc != T(0)) ? dxdesin[q] + dxdekep[q] * (dekepdm * dmdtp * dtpdesin + dekepdesin) : T(0);
    J(q, 4) = dxdinc[q];
    J(q, 5) = dxdcom[q];
    J(q, 6) = dxda[q] * dsemidm;
    J(3 + q, 0) = dvdp[q] + dvda[q] * dsemidp + dvdekep[q] * dekepdm * (dmdp + dmdtp * dtpdp);
    J(3 + q, 1) = dvdekep[q] * dekepdm * dmdtp * dtpdt0;
    J(3 + q, 2) = (ecc != T(0)) ? dvdecos[q] + dvdekep[q] * (dekepdm * dmdtp * dtpdecos + dekepdecos) : T(0);
    J(3 + q, 3) = (ecc != T(0)) ? dvdesin[q] + dvdekep[q] * (dekepdm * dmdtp * dtpdesin + dekepdesin) : T(0);
    J(3 + q, 4) = dvdinc[q];
    J(3 + q, 5) = dvdcom[q];
    J(3 + q, 6) = dvda[q] * dsemidm;
  }
  J(6, 6) = T(1);
}

// Fully nested hierarchy matrix, as hierarchy([N, 1, ..., 1]) returns it
// (setup_hierarchy.jl:9-145): row i < N has -1 on bodies 1..i and +1 on body
// i+1; the last row is all -1.  H is N x N col-major.
template <class T> void hierarchy_nested(int N, T* H) {
  for (int q = 0; q < N * N; q++) H[q] = T(0);
  for (int i = 0; i < N - 1; i++) {
    for (int j = 0; j <= i; j++) H[i + N * j] = T(-1);
    H[i + N * (i + 1)] = T(1);
  }
  for (int j = 0; j < N; j++) H[(N - 1) + N * j] = T(-1);
}

// Sigma_m (init_nbody.jl:203-210) and amatrix (:176-184)
template <class T> T sigma_m(const T* m, int N, int i, int j, const T* H) {
  T s = T(0);
  for (int l = 0; l < N; l++) s = s + m[l] * ((H[i + N * j] == H[i + N * l]) ? T(1) : T(0));
  return s;
}
template <class T> void amatrix(const T* H, const T* m, int N, T* A) {
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) A[i + N * j] = (H[i + N * j] * m[j]) / sigma_m(m, N, i, j, H);
}
// inv(A) by Gauss-Jordan elimination with partial pivoting (the reference
// calls LAPACK's LU-based inverse; the results agree to rounding).
template <class T> bool inv_matrix(const T* A, int N, T* out) {
  std::vector<T> a(A, A + N * N), b((size_t)N * N, T(0));
  for (int i = 0; i < N; i++) b[i + N * i] = T(1);
  for (int c = 0; c < N; c++) {
    int piv = c;
    for (int r = c + 1; r < N; r++)
      if (Mth<T>::fabs(a[r + N * c]) > Mth<T>::fabs(a[piv + N * c])) piv = r;
    if (a[piv + N * c] == T(0)) return false;
    if (piv != c)
      for (int q = 0; q < N; q++) { std::swap(a[c + N * q], a[piv + N * q]); std::swap(b[c + N * q], b[piv + N * q]); }
    T p = a[c + N * c];
    for (int q = 0; q < N; q++) { a[c + N * q] /= p; b[c + N * q] /= p; }
    for (int r = 0; r < N; r++) {
      if (r == c) continue;
      T f = a[r + N * c];
      if (f == T(0)) continue;
      for (int q = 0; q < N; q++) { a[r + N * q] -= f * a[c + N * q]; b[r + N * q] -= f * b[c + N * q]; }
    }
  }
  for (int q = 0; q < N * N; q++) out[q] = b[q];
  return true;
}

// init_nbody(ic::ElementsIC) (init_nbody.jl:13-27) with kepcalc (:50-105)
// and d_dm (:120-162).  elements is N x 7 col-major (m, P, t0, ecosw, esinw,
// I, Omega); H is the N x N hierarchy matrix.  Outputs x, v (3 x N) and
// jac_init (7N x 7N).
template <class T>
bool init_nbody(int N, T t0, const T* elements, const T* H, T* x, T* v, T* jac_init) {
  int M = 7 * N;
  std::vector<T> m(N), A((size_t)N * N), Ainv((size_t)N * N);
  for (int i = 0; i < N; i++) m[i] = elements[i];
  amatrix(H, m.data(), N, A.data());
  if (!inv_matrix(A.data(), N, Ainv.data())) return false;
  std::vector<T> rk((size_t)N * 3, T(0)), rdk((size_t)N * 3, T(0));  // N x 3 col-major
  std::vector<T> jk((size_t)6 * N * M, T(0));                        // 6N x 7N
  T jac21[49];
  int i = 0, b = 0;
  while (i < N - 1) {
    T mu = T(0);
    for (int l = 0; l < N; l++) if (H[i + N * l] != T(0)) mu = mu + m[l];
    if (H[i + N * 0] == T(0)) b += 1;
    T el[6];
    for (int q = 0; q < 6; q++) el[q] = elements[(i + 1 + b) + N * (1 + q)];
    T r[3], rd[3];
    kepler_init(t0, mu, el, r, rd, jac21);
    for (int q = 0; q < 3; q++) { rk[i + N * q] = r[q]; rdk[i + N * q] = rd[q]; }
    for (int j = 0; j < 6; j++)
      for (int k = 0; k < 6; k++) jk[(6 * i + j) + (size_t)6 * N * (7 * (i + 1) + k)] = jac21[j + 7 * k];
    for (int j = 0; j < N; j++)
      if (H[i + N * j] != T(0))
        for (int k = 0; k < 6; k++) jk[(6 * i + k) + (size_t)6 * N * (7 * j + 6)] = jac21[k + 7 * 6];
    if (b > 0) b -= 2;
    else if (b < 0) b = 0;
    i += 1;
  }
  // d_dm
  for (int q = 0; q < M * M; q++) jac_init[q] = T(0);
  std::vector<T> dAdm((size_t)N * N * N), dAinvdm((size_t)N * N * N);
  for (int k = 0; k < N; k++)
    for (int ii = 0; ii < N; ii++)
      for (int j = 0; j < N; j++) {
        T eij = H[ii + N * j], sm = sigma_m(m.data(), N, ii, j, H);
        T dkj = (k == j) ? T(1) : T(0);
        T dee = (H[ii + N * j] == H[ii + N * k]) ? T(1) : T(0);
        dAdm[ii + N * (j + N * k)] = (dkj * eij) / sm - dee * eij * m[j] / (sm * sm);
      }
  std::vector<T> t1((size_t)N * N);
  for (int k = 0; k < N; k++) {
    const T* D = &dAdm[(size_t)N * N * k];
    for (int ii = 0; ii < N; ii++)
      for (int j = 0; j < N; j++) {
        T acc = T(0);
        for (int q = 0; q < N; q++) acc = acc + (-Ainv[ii + N * q]) * D[q + N * j];
        t1[ii + N * j] = acc;
      }
    for (int ii = 0; ii < N; ii++)
      for (int j = 0; j < N; j++) {
        T acc = T(0);
        for (int q = 0; q < N; q++) acc = acc + t1[ii + N * q] * Ainv[q + N * j];
        dAinvdm[ii + N * (j + N * k)] = acc;
      }
  }
  for (int ii = 0; ii < N; ii++) {
    for (int k = 0; k < N; k++)
      for (int l = 0; l < M; l++)
        for (int j = 0; j < 3; j++) {
          jac_init[(7 * ii + j) + (size_t)M * l] += Ainv[ii + N * k] * jk[(6 * k + j) + (size_t)6 * N * l];
          jac_init[(7 * ii + 3 + j) + (size_t)M * l] += Ainv[ii + N * k] * jk[(6 * k + 3 + j) + (size_t)6 * N * l];
        }
    for (int k = 0; k < N; k++) {
      const T* D = &dAinvdm[(size_t)N * N * k];
      for (int j = 0; j < 3; j++) {
        T dx = T(0), dv = T(0);
        for (int q = 0; q < N; q++) {
          dx = dx + D[ii + N * q] * rk[q + N * j];
          dv = dv + D[ii + N * q] * rdk[q + N * j];
        }
        jac_init[(7 * ii + j) + (size_t)M * (7 * k + 6)] += dx;
        jac_init[(7 * ii + 3 + j) + (size_t)M * (7 * k + 6)] += dv;
      }
    }
    jac_init[(7 * ii + 6) + (size_t)M * (7 * ii + 6)] = T(1);
  }
  // x = permutedims(Ainv * r)
  for (int ii = 0; ii < N; ii++)
    for (int k = 0; k < 3; k++) {
      T ax = T(0), av = T(0);
      for (int q = 0; q < N; q++) {
        ax = ax + Ainv[ii + N * q] * rk[q + N * k];
        av = av + Ainv[ii + N * q] * rdk[q + N * k];
      }
      x[k + 3 * ii] = ax;
      v[k + 3 * ii] = av;
    }
  return true;
}

}  // namespace nbgo
