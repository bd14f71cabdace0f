// nbg_oracle.hpp -- CPU restatement of NbodyGradient.jl's AHL21 integrator with
// forward Jacobian propagation, its transit-timing driver and its initial
// conditions.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA path
// of the nbodygradient.jl_gb300 package.  Only tests/, __graft_entry__.smoke()
// and the CPU-baseline leg of bench.py may build, load or call it.  The
// product never links it.
//
// Every function cites the reference file:line it restates (paths are
// relative to the NbodyGradient.jl repository root).  The code is templated
// on the real type T so that the same arithmetic runs in double (the parity
// oracle) and in __float128 (the finite-difference pins that stand in for the
// reference's BigFloat tests).
//
// Arithmetic conventions that follow Julia's semantics:
//   * no FMA contraction in scalar code (build with -ffp-contract=off);
//   * n-ary a*b*c and a+b+c are left folds;
//   * x^2 -> x*x and x^3 -> x*x*x (Base.literal_pow); x^4 uses the
//     compensated power-by-squaring of Base.:^(::Float64, ::Integer);
//   * LinearAlgebra.mul! (BLAS gemm/gemv) is evaluated as one FMA chain per
//     output element in index order.  The reference's BLAS (Julia-bundled
//     OpenBLAS, version unpinned) fixes no order, so this is one admissible
//     evaluation; it is not claimed to be bit-identical to OpenBLAS.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <atomic>
#if defined(__x86_64__) || defined(__i386__)
#include <quadmath.h>
#define NBGO_QUADMATH 1
#endif

namespace nbgo {

// The quad type of the finite-difference pins: __float128 (libquadmath) on
// x86-64, long double (IEEE binary128 under the AArch64 Linux ABI) on Arm.
#ifdef NBGO_QUADMATH
typedef __float128 quad;
#else
typedef long double quad;
#endif

// ---------------------------------------------------------------- math traits
template <class T> struct Mth;
template <> struct Mth<double> {
  static double sin(double x) { return std::sin(x); }
  static double cos(double x) { return std::cos(x); }
  static double tan(double x) { return std::tan(x); }
  static double sinh(double x) { return std::sinh(x); }
  static double cosh(double x) { return std::cosh(x); }
  static double exp(double x) { return std::exp(x); }
  static double sqrt(double x) { return std::sqrt(x); }
  static double cbrt(double x) { return std::cbrt(x); }
  static double atan2(double y, double x) { return std::atan2(y, x); }
  static double fabs(double x) { return std::fabs(x); }
  static double fmod(double x, double y) { return std::fmod(x, y); }
  static double fma(double a, double b, double c) { return std::fma(a, b, c); }
  static double pi() { return 3.141592653589793; }
  static bool isfinite(double x) { return std::isfinite(x); }
};
#ifdef NBGO_QUADMATH
template <> struct Mth<quad> {
  static quad sin(quad x) { return sinq(x); }
  static quad cos(quad x) { return cosq(x); }
  static quad tan(quad x) { return tanq(x); }
  static quad sinh(quad x) { return sinhq(x); }
  static quad cosh(quad x) { return coshq(x); }
  static quad exp(quad x) { return expq(x); }
  static quad sqrt(quad x) { return sqrtq(x); }
  static quad cbrt(quad x) { return cbrtq(x); }
  static quad atan2(quad y, quad x) { return atan2q(y, x); }
  static quad fabs(quad x) { return fabsq(x); }
  static quad fmod(quad x, quad y) { return fmodq(x, y); }
  static quad fma(quad a, quad b, quad c) { return fmaq(a, b, c); }
  static quad pi() { return strtoflt128("3.14159265358979323846264338327950288", nullptr); }
  static bool isfinite(quad x) { return finiteq(x); }
};
#else
template <> struct Mth<quad> {
  static quad sin(quad x) { return std::sin(x); }
  static quad cos(quad x) { return std::cos(x); }
  static quad tan(quad x) { return std::tan(x); }
  static quad sinh(quad x) { return std::sinh(x); }
  static quad cosh(quad x) { return std::cosh(x); }
  static quad exp(quad x) { return std::exp(x); }
  static quad sqrt(quad x) { return std::sqrt(x); }
  static quad cbrt(quad x) { return std::cbrt(x); }
  static quad atan2(quad y, quad x) { return std::atan2(y, x); }
  static quad fabs(quad x) { return std::fabs(x); }
  static quad fmod(quad x, quad y) { return std::fmod(x, y); }
  static quad fma(quad a, quad b, quad c) { return std::fma(a, b, c); }
  static quad pi() { return 3.14159265358979323846264338327950288L; }
  static bool isfinite(quad x) { return std::isfinite(x); }
};
#endif

// Julia's sign(x) for floats: -1, 0 or +1 (NaN stays NaN).
template <class T> inline T jsign(T x) {
  if (x > T(0)) return T(1);
  if (x < T(0)) return T(-1);
  return x;  // +-0 or NaN
}

// Base.:^(x::Float64, n::Integer) for n == 4: compensated power by squaring
// (two_mul on each squaring, error carried in a low word).  For quad the
// plain product is used (the reference's BigFloat runs use MPFR powers).
template <class T> inline T pow4(T x) {
  T x2 = x * x;
  return x2 * x2;
}
template <> inline double pow4<double>(double x) {
  double x2 = x * x;
  double x2lo = std::fma(x, x, -x2);
  double err = x2 * 2.0 * x2lo;
  double x4 = x2 * x2;
  double x4lo = std::fma(x2, x2, -x4);
  double lo = x4lo + err;
  if (std::isfinite(x4) && std::isfinite(lo)) return x4 + lo;
  return x4;
}

// Constants of src/NbodyGradient.jl:13-17.  They are Float64 constants in
// the reference and stay Float64 (promoted) inside BigFloat computations.
static const double YEAR_D = 365.242;
static const double GNEWT_D = 39.4845 / (365.242 * 365.242);
static const double THIRD_D = 1.0 / 3.0;

// ------------------------------------------------------------ state & scratch
// State (src/integrator/Integrator.jl:49-103).  Column-major as in Julia:
//   x[k + 3 i], J[r + 7n c], pair[i + n j].
template <class T> struct State {
  int n = 0;
  std::vector<T> x, v, xerror, verror, a;
  T t = T(0);
  std::vector<T> m;
  std::vector<T> jac_step, jac_error, jac_init;
  std::vector<T> dqdt, dqdt_error;
  std::vector<uint8_t> pair;
  T rij[3], aij[3], x0[3], v0[3], delxv[6], rtmp[3];

  void alloc(int n_) {
    n = n_;
    int M = 7 * n;
    x.assign(3 * n, T(0)); v.assign(3 * n, T(0));
    xerror.assign(3 * n, T(0)); verror.assign(3 * n, T(0)); a.assign(3 * n, T(0));
    m.assign(n, T(0));
    jac_step.assign((size_t)M * M, T(0)); jac_error.assign((size_t)M * M, T(0));
    jac_init.assign((size_t)M * M, T(0));
    for (int i = 0; i < M; i++) jac_step[i + (size_t)M * i] = T(1);  // :87
    dqdt.assign(M, T(0)); dqdt_error.assign(M, T(0));
    pair.assign((size_t)n * n, 0);
    for (int k = 0; k < 3; k++) rij[k] = aij[k] = x0[k] = v0[k] = rtmp[k] = T(0);
    for (int k = 0; k < 6; k++) delxv[k] = T(0);
  }
  T& X(int k, int i) { return x[k + 3 * i]; }
  T& V(int k, int i) { return v[k + 3 * i]; }
  T& XE(int k, int i) { return xerror[k + 3 * i]; }
  T& VE(int k, int i) { return verror[k + 3 * i]; }
  T& A(int k, int i) { return a[k + 3 * i]; }
  T& J(int r, int c) { return jac_step[r + (size_t)7 * n * c]; }
  T& JE(int r, int c) { return jac_error[r + (size_t)7 * n * c]; }
  bool P(int i, int j) const { return pair[i + n * j] != 0; }
};

// set_state! (src/integrator/Integrator.jl:123-134)
template <class T> void set_state(State<T>& dst, const State<T>& src) {
  dst.t = src.t;
  dst.x = src.x; dst.v = src.v;
  dst.jac_step = src.jac_step;
  dst.xerror = src.xerror; dst.verror = src.verror;
  dst.jac_error = src.jac_error;
  dst.dqdt = src.dqdt; dst.dqdt_error = src.dqdt_error;
}

// Derivatives (src/PreAllocArrays.jl:65-113)
template <class T> struct Derivs {
  int n = 0, M = 0;
  std::vector<T> jac_phi, jac_kick, jac_copy, jac_ij, jac_tmp1, jac_tmp2, jac_err1;
  std::vector<T> dqdt_phi, dqdt_kick, dqdt_ij, dqdt_tmp1, dqdt_tmp2, jac_kepler, jac_mass;
  std::vector<T> dadq, dotdadq, tmp7n, tmp14;
  void alloc(int n_) {
    n = n_; M = 7 * n;
    jac_phi.assign((size_t)M * M, T(0)); jac_kick.assign((size_t)M * M, T(0));
    jac_copy.assign((size_t)M * M, T(0)); jac_ij.assign(196, T(0));
    jac_tmp1.assign(14 * M, T(0)); jac_tmp2.assign(14 * M, T(0)); jac_err1.assign(14 * M, T(0));
    dqdt_phi.assign(M, T(0)); dqdt_kick.assign(M, T(0)); dqdt_ij.assign(14, T(0));
    dqdt_tmp1.assign(14, T(0)); dqdt_tmp2.assign(14, T(0));
    jac_kepler.assign(48, T(0)); jac_mass.assign(6, T(0));
    dadq.assign((size_t)3 * n * 4 * n, T(0)); dotdadq.assign(4 * n, T(0));
    tmp7n.assign(M, T(0)); tmp14.assign(14, T(0));
  }
  // zero_out! (src/PreAllocArrays.jl:116-123)
  void zero() {
    for (auto* p : {&jac_phi, &jac_kick, &jac_copy, &jac_ij, &jac_tmp1, &jac_tmp2, &jac_err1,
                    &dqdt_phi, &dqdt_kick, &dqdt_ij, &dqdt_tmp1, &dqdt_tmp2, &jac_kepler,
                    &jac_mass, &dadq, &dotdadq, &tmp7n, &tmp14})
      std::fill(p->begin(), p->end(), T(0));
  }
  T& phi(int r, int c) { return jac_phi[r + (size_t)M * c]; }
  T& kick(int r, int c) { return jac_kick[r + (size_t)M * c]; }
  T& ij(int r, int c) { return jac_ij[r + 14 * c]; }
  T& kep(int r, int c) { return jac_kepler[r + 6 * c]; }
  T& DA(int k, int i, int p, int di) { return dadq[k + 3 * (i + n * (p + 4 * di))]; }
  T& DOT(int p, int di) { return dotdadq[p + 4 * di]; }
};

// Products skip the exact-zero entries of A when this flag is set (process
// wide; off by default, so the CPU baseline multiplies every zero as the
// reference's dense mul! does).  For finite B the skipped term is
// fma(+-0, b, acc) = acc exactly, and acc is never -0 (it starts at +0 and
// an FMA whose product is a signed zero and whose addend is +0 rounds to
// +0), so both modes give bitwise the same C; tests/test_oracle_pins.py
// checks that on whole integrations.  The long parity runs use it: the
// operators of ahl21! are mostly structural zeros.
inline std::atomic<bool>& skip_zero_products_flag() {
  static std::atomic<bool> on(false);
  return on;
}
inline bool skip_zero_products() { return skip_zero_products_flag().load(std::memory_order_relaxed); }

// LinearAlgebra.mul!(C, A, B): C (m x p) = A (m x q) * B (q x p), col-major.
template <class T>
void mul(T* C, const T* A, const T* B, int m, int q, int p) {
  if (skip_zero_products()) {
    for (int j = 0; j < p; j++)
      for (int i = 0; i < m; i++) {
        T acc = T(0);
        for (int k = 0; k < q; k++) {
          const T a = A[i + (size_t)m * k];
          if (a == T(0)) continue;
          acc = Mth<T>::fma(a, B[k + (size_t)q * j], acc);
        }
        C[i + (size_t)m * j] = acc;
      }
    return;
  }
  for (int j = 0; j < p; j++)
    for (int i = 0; i < m; i++) {
      T acc = T(0);
      for (int k = 0; k < q; k++) acc = Mth<T>::fma(A[i + (size_t)m * k], B[k + (size_t)q * j], acc);
      C[i + (size_t)m * j] = acc;
    }
}

// ---------------------------------------------------------------- src/utils.jl
// comp_sum (utils.jl:16-23)
template <class T> inline void comp_sum(T& s, T& e, T addend) {
  e = e + addend;
  T tmp = s + e;
  e = (s - tmp) + e;
  s = tmp;
}
// comp_sum_matrix! (utils.jl:36-46)
template <class T> void comp_sum_matrix(T* s, T* e, const T* add, size_t len) {
  for (size_t i = 0; i < len; i++) {
    e[i] = e[i] + add[i];
    T tmp = s[i] + e[i];
    e[i] = e[i] + (s[i] - tmp);
    s[i] = tmp;
  }
}
// copy_submatrix! (utils.jl:51-73); indi, indj are 0-based row offsets 7i, 7j
template <class T> void copy_submatrix(State<T>& s, Derivs<T>& d, int indi, int indj) {
  int M = 7 * s.n;
  for (int k2 = 0; k2 < M; k2++)
    for (int k1 = 0; k1 < 7; k1++) {
      d.jac_tmp1[k1 + 14 * k2] = s.J(indi + k1, k2);
      d.jac_err1[k1 + 14 * k2] = s.JE(indi + k1, k2);
      d.jac_tmp1[7 + k1 + 14 * k2] = s.J(indj + k1, k2);
      d.jac_err1[7 + k1 + 14 * k2] = s.JE(indj + k1, k2);
    }
  for (int k1 = 0; k1 < 7; k1++) {
    d.dqdt_tmp1[k1] = s.dqdt[indi + k1];
    d.dqdt_tmp1[7 + k1] = s.dqdt[indj + k1];
  }
}
// ypoc_submatrix! (utils.jl:78-100)
template <class T> void ypoc_submatrix(State<T>& s, Derivs<T>& d, int indi, int indj) {
  int M = 7 * s.n;
  for (int k2 = 0; k2 < M; k2++)
    for (int k1 = 0; k1 < 7; k1++) {
      s.J(indi + k1, k2) = d.jac_tmp1[k1 + 14 * k2];
      s.JE(indi + k1, k2) = d.jac_err1[k1 + 14 * k2];
      s.J(indj + k1, k2) = d.jac_tmp1[7 + k1 + 14 * k2];
      s.JE(indj + k1, k2) = d.jac_err1[7 + k1 + 14 * k2];
    }
  for (int k1 = 0; k1 < 7; k1++) {
    s.dqdt[indi + k1] = d.dqdt_ij[k1];
    s.dqdt[indj + k1] = d.dqdt_ij[7 + k1];
  }
}

// cubic1 (utils.jl:103-122)
template <class T> T cubic1(T a, T b, T c) {
  const T third = T(THIRD_D);
  T a3 = a * third;
  T Q = a3 * a3 - b * third;
  T R = a3 * a3 * a3 + T(0.5) * ((-a3) * b + c);
  T R2 = R * R, Q3 = Q * Q * Q;
  if (R2 < Q3) return -c / b;
  T A = (-jsign(R)) * Mth<T>::cbrt(Mth<T>::fabs(R) + Mth<T>::sqrt(R2 - Q3));
  T B = (A == T(0)) ? T(0) : Q / A;
  return A + B - a3;
}

// G3 and the H functions with their series (utils.jl:124-396).  gc = 0.5.
template <class T> T G3_series(T gamma, T beta, T sqb) {  // utils.jl:137-165
  T x2 = (-jsign(beta)) * (gamma * gamma);
  T term = T(1), g3 = T(1), g31 = T(2), g32 = T(2);
  int n = 0, iter = 0;
  while (true) {
    g32 = g31; g31 = g3; n += 1;
    term = term * (x2 / T((2 * n + 3) * (2 * n + 2)));
    g3 = g3 + term;
    iter += 1;
    if (iter >= 100 || g3 == g32 || g3 == g31) break;
  }
  g3 = g3 * (((-x2) * gamma) / ((T(6) * beta) * sqb));
  return g3;
}
template <class T> T G3(T gamma, T beta, T sqb) {  // utils.jl:124-135
  if (gamma < T(0.5)) return G3_series(gamma, beta, sqb);
  if (beta >= T(0)) return (gamma - Mth<T>::sin(gamma)) / (sqb * beta);
  return (gamma - Mth<T>::sinh(gamma)) / (sqb * beta);
}
template <class T> T H1_series(T gamma, T beta) {  // utils.jl:180-209
  T x2 = (-jsign(beta)) * (gamma * gamma);
  T term = T(1), h1 = T(1), h11 = T(2), h12 = T(2);
  int n = 0, iter = 0;
  while (true) {
    h12 = h11; h11 = h1; n += 1;
    term = term * (x2 * T(n + 1));
    term = term / T((2 * n + 4) * (2 * n + 3) * n);
    h1 = h1 + term;
    iter += 1;
    if (iter >= 100 || h1 == h12 || h1 == h11) break;
  }
  h1 = h1 * ((x2 * x2) / (T(12) * (beta * beta)));
  return h1;
}
template <class T> T H1(T gamma, T beta) {  // utils.jl:167-178
  if (gamma < T(0.5)) return H1_series(gamma, beta);
  if (beta >= T(0)) {
    T s = Mth<T>::sin(T(0.5) * gamma);
    return (T(4) * (s * s) - gamma * Mth<T>::sin(gamma)) / (beta * beta);
  }
  T s = Mth<T>::sinh(T(0.5) * gamma);
  return (T(-4) * (s * s) + gamma * Mth<T>::sinh(gamma)) / (beta * beta);
}
template <class T> T H2_series(T gamma, T beta, T sqb) {  // utils.jl:225-254
  T x2 = (-jsign(beta)) * (gamma * gamma);
  T term = T(1), h2 = T(1), h21 = T(2), h22 = T(2);
  int n = 0, iter = 0;
  while (true) {
    h22 = h21; h21 = h2; n += 1;
    term = term * x2;
    term = term / T((4 * n + 6) * n);
    h2 = h2 + term;
    iter += 1;
    if (iter >= 100 || h2 == h22 || h2 == h21) break;
  }
  h2 = h2 * (((-x2) * gamma) / ((T(3) * beta) * sqb));
  return h2;
}
template <class T> T H2(T gamma, T beta, T sqb) {  // utils.jl:211-223
  if (gamma < T(0.5)) return H2_series(gamma, beta, sqb);
  if (beta >= T(0)) return (Mth<T>::sin(gamma) - gamma * Mth<T>::cos(gamma)) / (sqb * beta);
  return (Mth<T>::sinh(gamma) - gamma * Mth<T>::cosh(gamma)) / (sqb * beta);
}
template <class T> T H3_series(T gamma, T beta, T sqb) {  // utils.jl:271-303
  T x2 = (-jsign(beta)) * (gamma * gamma);
  T term = T(1) / T(30), h3 = T(1) / T(10);
  T h31 = T(2) * h3, h32 = T(2) * h3;
  int n = 0, iter = 0;
  T four2n = T(4);
  while (true) {
    h32 = h31; h31 = h3; n += 1;
    term = term * x2;
    term = term / T((2 * n + 4) * (2 * n + 5));
    four2n = four2n * T(4);
    h3 = h3 + term * (four2n - T(1));
    iter += 1;
    if (iter >= 100 || h3 == h32 || h3 == h31) break;
  }
  h3 = h3 * (((-(x2 * x2)) * gamma) / (beta * sqb));
  return h3;
}
template <class T> T H3(T gamma, T beta, T sqb) {  // utils.jl:256-269
  if (gamma < T(0.5)) return H3_series(gamma, beta, sqb);
  if (beta >= T(0)) {
    T s = Mth<T>::sin(gamma), c = Mth<T>::cos(gamma);
    return (T(4) * s - s * c - T(3) * gamma) / (beta * sqb);
  }
  T s = Mth<T>::sinh(gamma), c = Mth<T>::cosh(gamma);
  return (T(4) * s - s * c - T(3) * gamma) / (beta * sqb);
}
template <class T> T H5_series(T gamma, T beta, T sqb) {  // utils.jl:320-349
  T x2 = (-jsign(beta)) * (gamma * gamma);
  T term = T(1) / T(60), h5 = term;
  T h51 = T(2) * h5, h52 = T(2) * h5;
  int n = 0, iter = 0;
  while (true) {
    h52 = h51; h51 = h5; n += 1;
    term = term * (x2 * T(n + 1));
    term = term / T((2 * n + 5) * (2 * n + 4) * n);
    h5 = h5 + term;
    iter += 1;
    if (iter >= 100 || h5 == h52 || h5 == h51) break;
  }
  h5 = h5 * (((-(x2 * x2)) * gamma) / (beta * sqb));
  return h5;
}
template <class T> T H5(T gamma, T beta, T sqb) {  // utils.jl:305-318
  if (gamma < T(0.5)) return H5_series(gamma, beta, sqb);
  if (beta >= T(0))
    return (T(3) * Mth<T>::sin(gamma) - T(2) * gamma - gamma * Mth<T>::cos(gamma)) / (beta * sqb);
  return (T(3) * Mth<T>::sinh(gamma) - T(2) * gamma - gamma * Mth<T>::cosh(gamma)) / (beta * sqb);
}
template <class T> T H6_series(T gamma, T beta) {  // utils.jl:364-396
  T x2 = (-jsign(beta)) * (gamma * gamma);
  T term = T(1) / T(360), h6 = T(1) / T(40);
  T h61 = T(2) * h6, h62 = T(2) * h6;
  int n = 0, iter = 0;
  T four2n = T(16);
  while (true) {
    h62 = h61; h61 = h6; n += 1;
    term = term * x2;
    term = term / T((2 * n + 5) * (2 * n + 6));
    four2n = four2n * T(4);
    h6 = h6 + term * (four2n - T(3 * n) - T(7));
    iter += 1;
    if (iter >= 100 || h6 == h62 || h6 == h61) break;
  }
  h6 = h6 * ((-(x2 * x2 * x2)) / (beta * beta));
  return h6;
}
template <class T> T H6(T gamma, T beta) {  // utils.jl:351-362
  if (gamma < T(0.5)) return H6_series(gamma, beta);
  if (beta >= T(0))
    return (T(9) - T(8) * Mth<T>::cos(gamma) - Mth<T>::cos(T(2) * gamma) -
            (T(6) * gamma) * Mth<T>::sin(gamma)) / (T(2) * (beta * beta));
  return (T(9) - T(8) * Mth<T>::cosh(gamma) - Mth<T>::cosh(T(2) * gamma) +
          (T(6) * gamma) * Mth<T>::sinh(gamma)) / (T(2) * (beta * beta));
}

// dot_fast (utils.jl:500-506)
template <class T> inline T dot3(const T* a, const T* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

}  // namespace nbgo

#include "nbg_oracle_step.hpp"
#include "nbg_oracle_transit.hpp"
#include "nbg_oracle_ics.hpp"
