// nbg_ics.cu -- initial conditions on the GPU: ElementsIC -> init_nbody for
// many systems at once (x, v and jac_init from orbital elements), so that a
// batch or a request stream built from elements needs no host-side setup.
//
// Restates, one lane per Keplerian / per body:
//   kepler_init with its 7x7 Jacobian   src/ics/kepler_init.jl:66-210
//   ekepler                             src/ics/kepler.jl:1-41
//   init_nbody (kepcalc, amatrix, d_dm)  src/ics/init_nbody.jl:13-229
//   hierarchy([N, 1, ..., 1])           src/ics/setup_hierarchy.jl:9-145
// Kernel 1 (one thread per system and Keplerian) solves the Kepler
// problems and their element Jacobians -- the transcendental part; kernel 2
// (one thread per system and body) forms A, its inverse, d A^-1 / d m and
// the body's rows of x, v and jac_init.  Built with --fmad=false: products
// and sums round one by one, as the reference evaluates them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/nbg.h"
#include "nbg_internal.cuh"

using namespace nbg;

namespace {

constexpr double kG = 39.4845 / (365.242 * 365.242);  // src/NbodyGradient.jl:13-17
constexpr double kThird = 1.0 / 3.0;
constexpr double kPi = 3.141592653589793;

struct IcOff {
  long long el, H, x, J, kep;  // elements (N x 7), H (N x N), x / v (3 x N), jac_init (M x M), Keplerian scratch
  int n, pad;
  double t0;
};

// Per Keplerian: r (3), rdot (3), the 7x7 Jacobian of kepler_init (49).
constexpr int KREC = 55;

__device__ __forceinline__ double dsign(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : x); }

// Julia mod(x, y) for floats
__device__ __forceinline__ double jmod(double x, double y) {
  double r = fmod(x, y);
  if (r == 0.0) return (y < 0.0) ? -0.0 : 0.0;
  if ((r > 0.0) != (y > 0.0)) return r + y;
  return r;
}

// ekepler (kepler.jl:1-41)
__device__ double ekepler(double m, double ecc) {
  if (m == 0.0) return 0.0;
  const double pi2 = 2.0 * kPi;
  const double ms = jmod(m, pi2);
  double de0 = ecc * 0.85 * dsign(ms);
  double de1 = 2.0 * de0, de2 = 3.0 * de0;
  int iter = 0;
  while (true) {
    de2 = de1;
    de1 = de0;
    const double f3 = ecc * cos(de0 + ms);
    const double f2 = ecc * sin(de0 + ms);
    de0 = (f2 - de1 * f3) / (1.0 - f3);
    iter += 1;
    if (iter >= 20 || de0 == de1 || de0 == de2) break;
  }
  return de0 + m;
}

struct Mat3 {
  double a[9];  // column-major
  __device__ double& operator()(int i, int j) { return a[i + 3 * j]; }
  __device__ double operator()(int i, int j) const { return a[i + 3 * j]; }
};
__device__ Mat3 mk(double a11, double a12, double a13, double a21, double a22, double a23, double a31, double a32,
                   double a33) {
  Mat3 c;
  c(0, 0) = a11; c(0, 1) = a12; c(0, 2) = a13;
  c(1, 0) = a21; c(1, 1) = a22; c(1, 2) = a23;
  c(2, 0) = a31; c(2, 1) = a32; c(2, 2) = a33;
  return c;
}
__device__ Mat3 mul(const Mat3& A, const Mat3& B) {
  Mat3 c;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) c(i, j) = A(i, 0) * B(0, j) + A(i, 1) * B(1, j) + A(i, 2) * B(2, j);
  return c;
}
__device__ Mat3 scale(const Mat3& A, double s) {
  Mat3 c;
  for (int q = 0; q < 9; q++) c.a[q] = A.a[q] * s;
  return c;
}
__device__ Mat3 divide(const Mat3& A, double s) {
  Mat3 c;
  for (int q = 0; q < 9; q++) c.a[q] = A.a[q] / s;
  return c;
}
__device__ void apply(const Mat3& A, const double* x, double* y) {
  for (int i = 0; i < 3; i++) y[i] = A(i, 0) * x[0] + A(i, 1) * x[1] + A(i, 2) * x[2];
}

// kepler_init with its Jacobian (kepler_init.jl:66-210): el = (P, t0, e cos w,
// e sin w, I, Omega); jac is 7x7 column-major d(x, v, m) / d(el, m).
__device__ void kepler_init(double time, double mass, const double* el, double* x, double* v, double* jac) {
  const double G = kG, third = kThird, pi = kPi;
  const double period = el[0];
  const double n = 2.0 * pi / period;
  const double t0 = el[1];
  const double semi = cbrt(G * mass * (period * period) / 4.0 / (pi * pi));
  const double dsemidp = 2.0 * third * semi / period;
  const double dsemidm = third * semi / mass;
  const double ecosomega = el[2], esinomega = el[3];
  const double ecc = sqrt(esinomega * esinomega + ecosomega * ecosomega);
  const double deccdecos = (ecc != 0.0) ? ecosomega / ecc : 0.0;
  const double deccdesin = (ecc != 0.0) ? esinomega / ecc : 0.0;
  const double sqrt1mecc2 = sqrt(1.0 - ecc * ecc);
  const double den1 = esinomega - ecosomega - ecc;
  double tp;
  if (ecc == 0.0) tp = t0 - 3.0 * period / 4.0;
  else
    tp = (t0 - sqrt1mecc2 / n * ecosomega / (1.0 - esinomega) -
          2.0 / n * atan2(sqrt(1.0 - ecc) * (esinomega + ecosomega + ecc), sqrt(1.0 + ecc) * den1));
  const double dtpdp = (tp - t0) / period;
  const double fac = sqrt((1.0 - ecc) / (1.0 + ecc));
  const double den2 = 1.0 / (den1 * den1);
  const double theta = fac * (esinomega + ecosomega + ecc) / den1;
  const double dthetadecc = ((ecc + ecosomega) * (ecc + ecosomega) + 2.0 * (1.0 - ecc * ecc) * esinomega -
                             esinomega * esinomega) /
                            (sqrt1mecc2 * (1.0 + ecc)) * den2;
  const double dthetadecos = 2.0 * fac * esinomega * den2;
  const double dthetadesin = (-(2.0 * fac)) * (ecosomega + ecc) * den2;
  const double dtpdecc =
      ecc / sqrt1mecc2 / n * ecosomega / (1.0 - esinomega) - 2.0 / n / (1.0 + theta * theta) * dthetadecc;
  const double dtpdecos =
      dtpdecc * deccdecos - sqrt1mecc2 / n / (1.0 - esinomega) - 2.0 / n / (1.0 + theta * theta) * dthetadecos;
  const double dtpdesin = dtpdecc * deccdesin - sqrt1mecc2 / n * ecosomega / ((1.0 - esinomega) * (1.0 - esinomega)) -
                          2.0 / n / (1.0 + theta * theta) * dthetadesin;
  const double dtpdt0 = 1.0;
  const double m = n * (time - tp);
  const double dmdp = -m / period;
  const double dmdtp = -n;
  const double ekep = ekepler(m, ecc);
  const double cosekep = cos(ekep), sinekep = sin(ekep);
  const double r = semi * (1.0 - ecc * cosekep);
  const double denom = semi / r;
  const double dekepdecos = sinekep * denom * deccdecos;
  const double dekepdesin = sinekep * denom * deccdesin;
  const double dekepdm = denom;
  const double inc = el[4], capomega = el[5];
  const double coscapomega = cos(capomega), sincapomega = sin(capomega);
  const double cosomega = (ecc != 0.0) ? ecosomega / ecc : 1.0;
  const double sinomega = (ecc != 0.0) ? esinomega / ecc : 0.0;
  const double cosinc = cos(inc), sininc = sin(inc);
  const Mat3 P1 = mk(cosomega, -sinomega, 0, sinomega, cosomega, 0, 0, 0, 1);
  const Mat3 P2 = mk(1, 0, 0, 0, cosinc, -sininc, 0, sininc, cosinc);
  const Mat3 P3 = mk(coscapomega, -sincapomega, 0, sincapomega, coscapomega, 0, 0, 0, 1);
  const Mat3 P32 = mul(P3, P2);
  const Mat3 P321 = mul(P32, P1);
  const double xplane[3] = {semi * (cosekep - ecc), semi * (sqrt1mecc2 * sinekep), 0.0};
  const double vplane[3] = {-sinekep, sqrt1mecc2 * cosekep, 0.0};
  apply(P321, xplane, x);
  double dxda[3], dxdekep[3], dxdecc[3], dxdecos[3], dxdesin[3], dxdinc[3], dxdcom[3], tmp[3];
  for (int q = 0; q < 3; q++) dxda[q] = x[q] / semi;
  apply(scale(P321, semi), vplane, dxdekep);
  {
    const double vv[3] = {cosekep, sinekep / sqrt1mecc2, 0.0};
    apply(divide(scale(scale(P321, -1.0), semi), ecc), vv, dxdecc);
  }
  apply(divide(P32, ecc), xplane, tmp);
  for (int q = 0; q < 3; q++) dxdecos[q] = dxdecc[q] * deccdecos + tmp[q];
  {
    const double vv[3] = {-xplane[1], xplane[0], 0.0};
    apply(divide(P32, ecc), vv, tmp);
  }
  for (int q = 0; q < 3; q++) dxdesin[q] = dxdecc[q] * deccdesin + tmp[q];
  const Mat3 Dinc = mk(0, 0, 0, 0, -sininc, -cosinc, 0, cosinc, -sininc);
  const Mat3 Dcom = mk(-sincapomega, -coscapomega, 0, coscapomega, -sincapomega, 0, 0, 0, 0);
  apply(mul(mul(P3, Dinc), P1), xplane, dxdinc);
  apply(mul(mul(Dcom, P2), P1), xplane, dxdcom);
  const double nsd = n * semi * denom;
  apply(scale(P321, nsd), vplane, v);
  double dvda[3], dvdp[3], dvdekep[3], dvdecc[3], dvdecos[3], dvdesin[3], dvdinc[3], dvdcom[3];
  for (int q = 0; q < 3; q++) {
    dvda[q] = v[q] / semi;
    dvdp[q] = -v[q] / period;
  }
  {
    const double vv[3] = {-cosekep, -sqrt1mecc2 * sinekep, 0.0};
    apply(scale(P321, nsd), vv, tmp);
    for (int q = 0; q < 3; q++) dvdekep[q] = (-v[q]) * ecc * sinekep * denom + tmp[q];
  }
  {
    const double vv[3] = {0.0, -ecc / sqrt1mecc2 * cosekep, 0.0};
    apply(scale(P321, nsd), vv, tmp);
    for (int q = 0; q < 3; q++) dvdecc[q] = -v[q] / ecc + v[q] * cosekep * denom + tmp[q];
  }
  apply(divide(scale(P32, nsd), ecc), vplane, tmp);
  for (int q = 0; q < 3; q++) dvdecos[q] = dvdecc[q] * deccdecos + tmp[q];
  {
    const double vv[3] = {-vplane[1], vplane[0], 0.0};
    apply(divide(scale(P32, nsd), ecc), vv, tmp);
  }
  for (int q = 0; q < 3; q++) dvdesin[q] = dvdecc[q] * deccdesin + tmp[q];
  apply(scale(mul(mul(P3, Dinc), P1), nsd), vplane, dvdinc);
  apply(scale(mul(mul(Dcom, P2), P1), nsd), vplane, dvdcom);
  for (int q = 0; q < 49; q++) jac[q] = 0.0;
  for (int q = 0; q < 3; q++) {
    jac[q + 7 * 0] = dxda[q] * dsemidp + dxdekep[q] * dekepdm * (dmdp + dmdtp * dtpdp);
    jac[q + 7 * 1] = dxdekep[q] * dekepdm * dmdtp * dtpdt0;
    jac[q + 7 * 2] = (ecc != 0.0) ? dxdecos[q] + dxdekep[q] * (dekepdm * dmdtp * dtpdecos + dekepdecos) : 0.0;
    jac[q + 7 * 3] = (ecc != 0.0) ? dxdesin[q] + dxdekep[q] * (dekepdm * dmdtp * dtpdesin + dekepdesin) : 0.0;
    jac[q + 7 * 4] = dxdinc[q];
    jac[q + 7 * 5] = dxdcom[q];
    jac[q + 7 * 6] = dxda[q] * dsemidm;
    jac[3 + q + 7 * 0] = dvdp[q] + dvda[q] * dsemidp + dvdekep[q] * dekepdm * (dmdp + dmdtp * dtpdp);
    jac[3 + q + 7 * 1] = dvdekep[q] * dekepdm * dmdtp * dtpdt0;
    jac[3 + q + 7 * 2] = (ecc != 0.0) ? dvdecos[q] + dvdekep[q] * (dekepdm * dmdtp * dtpdecos + dekepdecos) : 0.0;
    jac[3 + q + 7 * 3] = (ecc != 0.0) ? dvdesin[q] + dvdekep[q] * (dekepdm * dmdtp * dtpdesin + dekepdesin) : 0.0;
    jac[3 + q + 7 * 4] = dvdinc[q];
    jac[3 + q + 7 * 5] = dvdcom[q];
    jac[3 + q + 7 * 6] = dvda[q] * dsemidm;
  }
  jac[6 + 7 * 6] = 1.0;
}

// The element row of Keplerian i (init_nbody.jl:56-104: the counter b steps
// past rows that start a new sub-hierarchy).
__device__ int kepler_row(const double* H, int N, int i) {
  int b = 0;
  for (int q = 0; q <= i; q++) {
    if (H[q + N * 0] == 0.0) b += 1;
    if (q == i) return i + 1 + b;
    if (b > 0) b -= 2;
    else if (b < 0) b = 0;
  }
  return i + 1 + b;
}

__device__ void nested_hierarchy(int N, double* H) {
  for (int q = 0; q < N * N; q++) H[q] = 0.0;
  for (int i = 0; i < N - 1; i++) {
    for (int j = 0; j <= i; j++) H[i + N * j] = -1.0;
    H[i + N * (i + 1)] = 1.0;
  }
  for (int j = 0; j < N; j++) H[(N - 1) + N * j] = -1.0;
}

__device__ void load_h(const IcOff& o, const double* Hin, double* H) {
  const int N = o.n;
  if (Hin)
    for (int q = 0; q < N * N; q++) H[q] = Hin[o.H + q];
  else
    nested_hierarchy(N, H);
}

// Kernel 1: one thread per (system, Keplerian i < N-1).
__global__ void kepler_init_kernel(int nsys, int maxk, const IcOff* off, const double* elements, const double* Hin,
                                   double* kep, int* bad) {
  const long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= (long long)nsys * maxk) return;
  const int sys = (int)(f / maxk), i = (int)(f % maxk);
  const IcOff o = off[sys];
  const int N = o.n;
  if (i >= N - 1) return;
  double H[NBG_MAX_BODIES * NBG_MAX_BODIES];
  load_h(o, Hin, H);
  const double* el = elements + o.el;  // N x 7 column-major
  double mu = 0.0;
  for (int l = 0; l < N; l++)
    if (H[i + N * l] != 0.0) mu = mu + el[l];
  const int row = kepler_row(H, N, i);
  if (row < 0 || row >= N) {  // a hierarchy matrix that init_nbody cannot read
    atomicOr(bad, 2);
    return;
  }
  double e6[6];
  for (int q = 0; q < 6; q++) e6[q] = el[row + N * (1 + q)];
  double* out = kep + o.kep + (long long)KREC * i;
  kepler_init(o.t0, mu, e6, out, out + 3, out + 6);
}

// Gauss-Jordan inverse with partial pivoting (the reference inverts with
// LAPACK's LU; both agree to rounding).  Returns false when singular.
__device__ bool invert(double* a, int N, double* b) {
  for (int q = 0; q < N * N; q++) b[q] = 0.0;
  for (int i = 0; i < N; i++) b[i + N * i] = 1.0;
  for (int c = 0; c < N; c++) {
    int piv = c;
    for (int r = c + 1; r < N; r++)
      if (fabs(a[r + N * c]) > fabs(a[piv + N * c])) piv = r;
    if (a[piv + N * c] == 0.0) return false;
    if (piv != c)
      for (int q = 0; q < N; q++) {
        double t = a[c + N * q]; a[c + N * q] = a[piv + N * q]; a[piv + N * q] = t;
        t = b[c + N * q]; b[c + N * q] = b[piv + N * q]; b[piv + N * q] = t;
      }
    const double p = a[c + N * c];
    for (int q = 0; q < N; q++) {
      a[c + N * q] /= p;
      b[c + N * q] /= p;
    }
    for (int r = 0; r < N; r++) {
      if (r == c) continue;
      const double f = a[r + N * c];
      if (f == 0.0) continue;
      for (int q = 0; q < N; q++) {
        a[r + N * q] -= f * a[c + N * q];
        b[r + N * q] -= f * b[c + N * q];
      }
    }
  }
  return true;
}

__device__ double sigma_m(const double* m, int N, int i, int j, const double* H) {
  double s = 0.0;
  for (int l = 0; l < N; l++) s = s + m[l] * ((H[i + N * j] == H[i + N * l]) ? 1.0 : 0.0);
  return s;
}

// Kernel 2: one thread per (system, body ii): rows 7 ii .. 7 ii + 6 of
// jac_init and column ii of x and v (init_nbody.jl:13-27, d_dm at :120-162).
__global__ void assemble_kernel(int nsys, const IcOff* off, const double* elements, const double* Hin,
                                const double* kep, double* x, double* v, double* jac_init, int* bad) {
  const long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= (long long)nsys * NBG_MAX_BODIES) return;
  const int sys = (int)(f / NBG_MAX_BODIES), ii = (int)(f % NBG_MAX_BODIES);
  const IcOff o = off[sys];
  const int N = o.n, M = 7 * N;
  if (ii >= N) return;
  double H[NBG_MAX_BODIES * NBG_MAX_BODIES], A[NBG_MAX_BODIES * NBG_MAX_BODIES], Ai[NBG_MAX_BODIES * NBG_MAX_BODIES];
  double m[NBG_MAX_BODIES];
  load_h(o, Hin, H);
  const double* el = elements + o.el;
  for (int i = 0; i < N; i++) m[i] = el[i];
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) A[i + N * j] = (H[i + N * j] * m[j]) / sigma_m(m, N, i, j, H);
  if (!invert(A, N, Ai)) {
    atomicOr(bad, 1);
    return;
  }
  const double* kp = kep + o.kep;  // Keplerian k: r at kp[KREC k], rdot at +3, jac21 at +6
  double* J = jac_init + o.J;
  for (int r = 0; r < 7; r++)
    for (int l = 0; l < M; l++) J[(7 * ii + r) + (long long)M * l] = 0.0;
  // jac_init[x, v rows of ii, :] += Ainv[ii, k] * jk[6k + j, :], k ascending;
  // the non-zero columns of jk's block k are body k+1's element columns and
  // the mass columns of the bodies in Keplerian k
  for (int k = 0; k < N - 1; k++) {
    const double aik = Ai[ii + N * k];
    const double* jac21 = kp + KREC * k + 6;
    for (int l = 0; l < M; l++) {
      const int lb = l / 7, lk = l % 7;
      int src = -1;
      if (lb == k + 1 && lk < 6) src = lk;
      else if (lk == 6 && H[k + N * lb] != 0.0) src = 6;
      if (src < 0) continue;
      for (int j = 0; j < 6; j++) {
        double& e = J[(7 * ii + j) + (long long)M * l];
        e = e + aik * jac21[j + 7 * src];
      }
    }
  }
  // the last row of jk is zero (no Keplerian N-1): Ainv[ii, N-1] * 0 adds
  // exact zeros.  Mass columns: += (d Ainv / d m_k)[ii, :] * (r, rdot)
  double t1[NBG_MAX_BODIES], dai[NBG_MAX_BODIES];
  for (int k = 0; k < N; k++) {
    // t1 = -Ainv[ii, :] * dA_k, then row ii of dA_k^inv = t1 * Ainv
    for (int j = 0; j < N; j++) {
      double acc = 0.0;
      for (int q = 0; q < N; q++) {
        const double eqj = H[q + N * j], sm = sigma_m(m, N, q, j, H);
        const double dkj = (k == j) ? 1.0 : 0.0;
        const double dee = (H[q + N * j] == H[q + N * k]) ? 1.0 : 0.0;
        const double d = (dkj * eqj) / sm - dee * eqj * m[j] / (sm * sm);
        acc = acc + (-Ai[ii + N * q]) * d;
      }
      t1[j] = acc;
    }
    for (int j = 0; j < N; j++) {
      double acc = 0.0;
      for (int q = 0; q < N; q++) acc = acc + t1[q] * Ai[q + N * j];
      dai[j] = acc;
    }
    for (int j = 0; j < 3; j++) {
      double dx = 0.0, dv = 0.0;
      for (int q = 0; q < N; q++) {
        const double rq = (q < N - 1) ? kp[KREC * q + j] : 0.0;
        const double vq = (q < N - 1) ? kp[KREC * q + 3 + j] : 0.0;
        dx = dx + dai[q] * rq;
        dv = dv + dai[q] * vq;
      }
      J[(7 * ii + j) + (long long)M * (7 * k + 6)] += dx;
      J[(7 * ii + 3 + j) + (long long)M * (7 * k + 6)] += dv;
    }
  }
  J[(7 * ii + 6) + (long long)M * (7 * ii + 6)] = 1.0;
  // x = (Ainv * r)^T, v = (Ainv * rdot)^T
  for (int k = 0; k < 3; k++) {
    double ax = 0.0, av = 0.0;
    for (int q = 0; q < N; q++) {
      const double rq = (q < N - 1) ? kp[KREC * q + k] : 0.0;
      const double vq = (q < N - 1) ? kp[KREC * q + 3 + k] : 0.0;
      ax = ax + Ai[ii + N * q] * rq;
      av = av + Ai[ii + N * q] * vq;
    }
    x[o.x + k + 3 * ii] = ax;
    v[o.x + k + 3 * ii] = av;
  }
}

}  // namespace

namespace nbg {

// Device-side init_nbody for nsys systems; all array pointers are device
// pointers; n and t0 are host arrays.  scratch is taken from the context.
int init_nbody_device(int device, cudaStream_t st, int nsys, const int32_t* n, const double* t0,
                      const double* d_elements, const double* d_H, double* d_x, double* d_v, double* d_jinit,
                      void* (*get)(void* ctx, const char* name, size_t bytes), void* ctx) {
  std::vector<IcOff> off(nsys);
  long long ael = 0, aH = 0, ax = 0, aJ = 0, ak = 0;
  for (int s = 0; s < nsys; s++) {
    if (n[s] < NBG_MIN_BODIES || n[s] > NBG_MAX_BODIES)
      return set_error(NBG_EUNSUPPORTED, "system %d: n = %d outside %d..%d", s, n[s], NBG_MIN_BODIES, NBG_MAX_BODIES);
    if (!std::isfinite(t0[s])) return set_error(NBG_EINVAL, "system %d: t0 = %g", s, t0[s]);
    const int N = n[s], M = 7 * N;
    IcOff& o = off[s];
    o.el = ael; o.H = aH; o.x = ax; o.J = aJ; o.kep = ak; o.n = N; o.pad = 0; o.t0 = t0[s];
    ael += 7LL * N; aH += (long long)N * N; ax += 3LL * N; aJ += (long long)M * M; ak += (long long)KREC * (N - 1);
  }
  IcOff* d_off = (IcOff*)get(ctx, "ic_off", sizeof(IcOff) * nsys);
  double* d_kep = (double*)get(ctx, "ic_kep", sizeof(double) * std::max<long long>(ak, 1));
  int* d_bad = (int*)get(ctx, "ic_bad", sizeof(int));
  if (!d_off || !d_kep || !d_bad) return NBG_ENOMEM;
  NBG_CUDA(cudaMemcpyAsync(d_off, off.data(), sizeof(IcOff) * nsys, cudaMemcpyHostToDevice, st));
  NBG_CUDA(cudaMemsetAsync(d_bad, 0, sizeof(int), st));
  const long long t1 = (long long)nsys * (NBG_MAX_BODIES - 1);
  kepler_init_kernel<<<(unsigned)((t1 + 63) / 64), 64, 0, st>>>(nsys, NBG_MAX_BODIES - 1, d_off, d_elements, d_H,
                                                                 d_kep, d_bad);
  const long long t2 = (long long)nsys * NBG_MAX_BODIES;
  assemble_kernel<<<(unsigned)((t2 + 63) / 64), 64, 0, st>>>(nsys, d_off, d_elements, d_H, d_kep, d_x, d_v, d_jinit,
                                                              d_bad);
  NBG_CUDA(cudaGetLastError());
  int bad = 0;
  NBG_CUDA(cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, st));
  NBG_CUDA(cudaStreamSynchronize(st));
  if (bad & 2) return set_error(NBG_EINVAL, "init_nbody: a hierarchy matrix names an element row beyond N");
  if (bad) return set_error(NBG_EINVAL, "init_nbody: the hierarchy's A matrix is singular for some system");
  (void)device;
  return NBG_OK;
}

}  // namespace nbg
