// nbg_kepler.cuh -- device-side universal-variable Kepler drift for one body
// pair and its analytic Jacobian, FP64.
//
// Restates, for one lane = one system, NbodyGradient.jl's
//   jac_delxv_gamma!        src/integrator/ahl21/ahl21.jl:766-890
//   compute_jacobian_gamma! src/integrator/ahl21/ahl21.jl:896-1139
//   cubic1, G3, H1, H2, H3, H5, H6 and their series  src/utils.jl:103-396
// The translation unit is compiled with --fmad=false: every product and sum
// rounds on its own, as Julia evaluates them; fma() appears only where the
// reference itself takes a fused product (Base.:^(x, 4)).
//
// GPU-specific structure: the six G/H series are evaluated as fixed-degree
// polynomials with precomputed exact coefficients (gh_functions), which
// removes the series' chains of dependent FP64 divisions from the per-pair
// critical path.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace nbg {

// src/NbodyGradient.jl:13-17
constexpr double GNEWT = 39.4845 / (365.242 * 365.242);
constexpr double THIRD = 1.0 / 3.0;

__device__ __forceinline__ double jsign(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : x); }

// comp_sum (src/utils.jl:16-23)
__device__ __forceinline__ void kahan(double& s, double& e, double a) {
  e = e + a;
  double t = s + e;
  e = (s - t) + e;
  s = t;
}

// Base.:^(x::Float64, 4): compensated power by squaring
__device__ __forceinline__ double pow4(double x) {
  double x2 = x * x;
  double x2lo = fma(x, x, -x2);
  double err = x2 * 2.0 * x2lo;
  double x4 = x2 * x2;
  double x4lo = fma(x2, x2, -x4);
  double lo = x4lo + err;
  if (isfinite(x4) && isfinite(lo)) return x4 + lo;
  return x4;
}

// cubic1 (src/utils.jl:103-122)
__device__ __forceinline__ double cubic1(double a, double b, double c) {
  double a3 = a * THIRD;
  double Q = a3 * a3 - b * THIRD;
  double R = a3 * a3 * a3 + 0.5 * ((-a3) * b + c);
  double R2 = R * R, Q3 = Q * Q * Q;
  if (R2 < Q3) return -c / b;
  double A = (-jsign(R)) * cbrt(fabs(R) + sqrt(R2 - Q3));
  double B = (A == 0.0) ? 0.0 : Q / A;
  return A + B - a3;
}

// sin and cos of |x| <= pi/4 from their Taylor series about 0 (coefficients
// (-1)^k / (2k+1)! up to x^17 and (-1)^k / (2k)! up to x^18, Horner scheme in
// x^2).  The truncation error at |x| = pi/4 is below 1e-19, the evaluation
// error about one ulp; the result is checked against CUDA's sin and cos
// (tests/test_gpu_math.py).  Outside |x| <= pi/4 CUDA's sincos is used.
// The half-angle x = gamma / 2 of the Kepler solve is far below pi/4 for
// bound orbits stepped at a fraction of their period.
__device__ __forceinline__ void sincos_kepler(double x, double* s, double* c) {
  if (fabs(x) > 0.78539816339744831) {
    sincos(x, s, c);
    return;
  }
  const double x2 = x * x;
  double ps = 0x1.952c77030ad4ap-49;
  ps = fma(ps, x2, -0x1.ae7f3e733b81fp-41);
  ps = fma(ps, x2, 0x1.6124613a86d09p-33);
  ps = fma(ps, x2, -0x1.ae64567f544e4p-26);
  ps = fma(ps, x2, 0x1.71de3a556c734p-19);
  ps = fma(ps, x2, -0x1.a01a01a01a01ap-13);
  ps = fma(ps, x2, 0x1.1111111111111p-7);
  ps = fma(ps, x2, -0x1.5555555555555p-3);
  *s = fma(x * x2, ps, x);
  double pc = -0x1.6827863b97d97p-53;
  pc = fma(pc, x2, 0x1.ae7f3e733b81fp-45);
  pc = fma(pc, x2, -0x1.93974a8c07c9dp-37);
  pc = fma(pc, x2, 0x1.1eed8eff8d898p-29);
  pc = fma(pc, x2, -0x1.27e4fb7789f5cp-22);
  pc = fma(pc, x2, 0x1.a01a01a01a01ap-16);
  pc = fma(pc, x2, -0x1.6c16c16c16c17p-10);
  pc = fma(pc, x2, 0x1.5555555555555p-5);
  *c = fma(x2 * x2, pc, fma(-0.5, x2, 1.0));
}

enum : int { GH_G3 = 1, GH_H1 = 2, GH_H2 = 4, GH_H3 = 8, GH_H5 = 16, GH_H6 = 32 };

struct GH {
  double g3, h1, h2, h3, h5, h6;
};

// Coefficients c_n of the G3, H1, H2, H3, H5, H6 series in x2 = -sign(beta) gamma^2
// (src/utils.jl:137-396), exact rationals rounded to double, n = 0..10.
__device__ __constant__ double kGHCoef[6][11] = {
    {0x1.0000000000000p+0, 0x1.999999999999ap-5, 0x1.3813813813814p-10, 0x1.1566abc011567p-16, 0x1.42cb40df7f3abp-23, 0x1.08db48ebe51c7p-30, 0x1.42df6ed66ca17p-38, 0x1.2fe15942481f8p-46, 0x1.c6ee8e9c1e203p-55, 0x1.154ab3925b815p-63, 0x1.189470e50aa13p-72},  // G3
    {0x1.0000000000000p+0, 0x1.1111111111111p-4, 0x1.d41d41d41d41dp-10, 0x1.bbd779334ef0bp-16, 0x1.0cfeb60f94b0ep-22, 0x1.c60a33dd88c31p-30, 0x1.1a8380fb9f0d4p-37, 0x1.0e1da4acb1e32p-45, 0x1.99704d261b1cfp-54, 0x1.f82abadb8f19bp-63, 0x1.0132bcd1f4692p-71},  // H1
    {0x1.0000000000000p+0, 0x1.999999999999ap-4, 0x1.d41d41d41d41dp-9, 0x1.1566abc011567p-14, 0x1.937e11175f095p-21, 0x1.8d48ed61d7aabp-28, 0x1.1a8380fb9f0d4p-35, 0x1.2fe15942481f8p-43, 0x1.ffcc606fa1e43p-52, 0x1.5a9d6076f261ap-60, 0x1.81cc1b3aee9dbp-69},  // H2
    {0x1.999999999999ap-4, 0x1.8618618618618p-7, 0x1.6c16c16c16c17p-11, 0x1.acb5f228d4f9fp-16, 0x1.60cc1822382eep-21, 0x1.ae64567f544e4p-27, 0x1.952622512ec88p-33, 0x1.2f48851e5fad6p-39, 0x1.71b892ff937bap-46, 0x1.761b29cfaf6e8p-53, 0x1.3f3cc8d472c34p-60},  // H3
    {0x1.1111111111111p-6, 0x1.a01a01a01a01ap-11, 0x1.1566abc011567p-16, 0x1.ae64567f544e4p-23, 0x1.b96d79892884cp-30, 0x1.42df6ed66ca17p-37, 0x1.6286e822a97a1p-45, 0x1.2f49b46814157p-53, 0x1.9ff00d5b89420p-62, 0x1.d3a2117dbc620p-71, 0x1.b6f39affec388p-80},  // H5
    {0x1.999999999999ap-6, 0x1.5f15f15f15f16p-9, 0x1.18de5ab277f45p-13, 0x1.1a71d8c38f535p-18, 0x1.91b806e381809p-24, 0x1.adeb42b5c3e58p-30, 0x1.68045a5f7c07ap-36, 0x1.e535756d08617p-43, 0x1.0ce18de28b3bep-49, 0x1.f2cdf899367f3p-57, 0x1.88e826fd0f0dep-64},  // H6
};

__device__ __forceinline__ double gh_horner(const double* c, double x2) {
  double p = c[10];
#pragma unroll
  for (int n = 9; n >= 0; n--) p = fma(p, x2, c[n]);
  return p;
}

// G3, H1, H2, H3, H5, H6 at (gamma, beta) -- the subset named by NEED.
// gamma < 0.5: the series of utils.jl:137-396 in x2 = -sign(beta) gamma^2,
// |x2| < 0.25, evaluated as degree-10 polynomials with the exact series
// coefficients (terms beyond n = 10 are below 1e-17 of the leading term).
// The reference sums term by term until the partial sum stops changing;
// the polynomial reaches the same value to rounding, without the series'
// dependent FP64 divisions.  gamma >= 0.5: the closed forms of utils.jl.
template <int NEED>
__device__ __forceinline__ GH gh_functions(double gamma, double beta, double sqb) {
  GH o;
  o.g3 = o.h1 = o.h2 = o.h3 = o.h5 = o.h6 = 0.0;
  if (gamma < 0.5) {
    const double x2 = (-jsign(beta)) * (gamma * gamma);
    if (NEED & GH_G3) o.g3 = gh_horner(kGHCoef[0], x2) * (((-x2) * gamma) / ((6.0 * beta) * sqb));
    if (NEED & GH_H1) o.h1 = gh_horner(kGHCoef[1], x2) * ((x2 * x2) / (12.0 * (beta * beta)));
    if (NEED & GH_H2) o.h2 = gh_horner(kGHCoef[2], x2) * (((-x2) * gamma) / ((3.0 * beta) * sqb));
    if (NEED & GH_H3) o.h3 = gh_horner(kGHCoef[3], x2) * (((-(x2 * x2)) * gamma) / (beta * sqb));
    if (NEED & GH_H5) o.h5 = gh_horner(kGHCoef[4], x2) * (((-(x2 * x2)) * gamma) / (beta * sqb));
    if (NEED & GH_H6) o.h6 = gh_horner(kGHCoef[5], x2) * ((-(x2 * x2 * x2)) / (beta * beta));
  } else if (beta >= 0.0) {
    double s, c;
    sincos(gamma, &s, &c);
    if (NEED & GH_G3) o.g3 = (gamma - s) / (sqb * beta);
    if (NEED & GH_H1) {
      double sh = sin(0.5 * gamma);
      o.h1 = (4.0 * (sh * sh) - gamma * s) / (beta * beta);
    }
    if (NEED & GH_H2) o.h2 = (s - gamma * c) / (sqb * beta);
    if (NEED & GH_H3) o.h3 = (4.0 * s - s * c - 3.0 * gamma) / (beta * sqb);
    if (NEED & GH_H5) o.h5 = (3.0 * s - 2.0 * gamma - gamma * c) / (beta * sqb);
    if (NEED & GH_H6) o.h6 = (9.0 - 8.0 * c - cos(2.0 * gamma) - (6.0 * gamma) * s) / (2.0 * (beta * beta));
  } else {
    double s = sinh(gamma), c = cosh(gamma);
    if (NEED & GH_G3) o.g3 = (gamma - s) / (sqb * beta);
    if (NEED & GH_H1) {
      double sh = sinh(0.5 * gamma);
      o.h1 = (-4.0 * (sh * sh) + gamma * s) / (beta * beta);
    }
    if (NEED & GH_H2) o.h2 = (s - gamma * c) / (sqb * beta);
    if (NEED & GH_H3) o.h3 = (4.0 * s - s * c - 3.0 * gamma) / (beta * sqb);
    if (NEED & GH_H5) o.h5 = (3.0 * s - 2.0 * gamma - gamma * c) / (beta * sqb);
    if (NEED & GH_H6) o.h6 = (9.0 - 8.0 * c - cosh(2.0 * gamma) + (6.0 * gamma) * s) / (2.0 * (beta * beta));
  }
  return o;
}

// Parameters jac_delxv_gamma! hands to compute_jacobian_gamma! (ahl21.jl:888)
// plus the H values the Jacobian needs.
struct KepParams {
  double gamma, g0, g1, g2, g3, h1, h2, dfdt, fm1, gmh, dgdtm1, r0, r, r0inv, rinv, k, h, beta, betainv, eta, sqb,
      zeta;
  double H1v, H2v, H3v, H5v, H6v;
  int newton_iter;
};

// jac_delxv_gamma! (ahl21.jl:766-890): Kepler drift of the relative orbit
// (x0, v0) with k = G (m_i + m_j) over h; writes delxv (position and velocity
// differences, finish - start minus the drift terms).
template <bool DRIFT_FIRST, bool JAC>
__device__ __noinline__ void kep_delxv(const double* x0, const double* v0, double k, double h, double* delxv,
                                          KepParams& P) {
  double rt0 = x0[0] - h * v0[0], rt1 = x0[1] - h * v0[1], rt2 = x0[2] - h * v0[2];
  double r0 = DRIFT_FIRST ? sqrt(rt0 * rt0 + rt1 * rt1 + rt2 * rt2) : sqrt(x0[0] * x0[0] + x0[1] * x0[1] + x0[2] * x0[2]);
  double r0inv = 1.0 / r0;
  double beta0 = 2.0 * k * r0inv - (v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2]);
  double beta0inv = 1.0 / beta0;
  double signb = jsign(beta0);
  double sqb = sqrt(signb * beta0);
  double zeta = k - r0 * beta0;
  double eta = DRIFT_FIRST ? (rt0 * v0[0] + rt1 * v0[1] + rt2 * v0[2]) : (x0[0] * v0[0] + x0[1] * v0[1] + x0[2] * v0[2]);
  double gamma_guess;
  if (zeta != 0.0) {
    double zinv = 6.0 / zeta;
    gamma_guess = cubic1(0.5 * eta * sqb * zinv, r0 * signb * beta0 * zinv, (-h) * signb * beta0 * sqb * zinv);
  } else if (eta != 0.0) {
    double reta = r0 / eta;
    double disc = reta * reta + 2.0 * h / eta;
    gamma_guess = (disc > 0.0) ? sqb * ((-reta) + sqrt(disc)) : h * r0inv * sqb;
  } else {
    gamma_guess = h * r0inv * sqb;
  }
  double gamma = gamma_guess;
  double gamma1 = 2.0 * gamma, gamma2 = 3.0 * gamma;
  double c2 = -2.0 * zeta, c3 = 2.0 * eta * signb * sqb, c4 = (-sqb) * h * beta0, c5 = 2.0 * eta * signb * sqb;
  double sx, cx;
  int iter = 0;
  while (iter < 20) {
    gamma2 = gamma1;
    gamma1 = gamma;
    double xx = 0.5 * gamma;
    if (beta0 > 0.0) {
      sincos_kepler(xx, &sx, &cx);
    } else {
      sx = sinh(xx);
      cx = exp(-xx) + sx;
    }
    gamma = gamma - (k * gamma + c2 * sx * cx + c3 * (sx * sx) + c4) /
                        (2.0 * signb * zeta * (sx * sx) + c5 * sx * cx + r0 * beta0);
    iter += 1;
    if (gamma == gamma2 || gamma == gamma1) break;
  }
  P.newton_iter = iter;
  double xx = 0.5 * gamma;
  if (beta0 > 0.0) {
    sincos_kepler(xx, &sx, &cx);
  } else {
    sx = sinh(xx);
    cx = exp(-xx) + sx;
  }
  double g1bs = 2.0 * sx * cx / sqb;
  double g2bs = 2.0 * signb * (sx * sx) * beta0inv;
  double g0bs = 1.0 - beta0 * g2bs;
  constexpr int NEED = JAC ? (GH_G3 | GH_H1 | GH_H2 | GH_H3 | GH_H5 | GH_H6)
                           : (DRIFT_FIRST ? GH_G3 : (GH_G3 | GH_H1 | GH_H2));
  GH gh = gh_functions<NEED>(gamma, beta0, sqb);
  double g3bs = gh.g3;
  double h1 = 0.0, h2 = 0.0;
  double r = r0 * g0bs + eta * g1bs + k * g2bs;
  double rinv = 1.0 / r;
  double dfdt = (-k) * g1bs * rinv * r0inv;
  double fm1, gmh, dgdtm1;
  if (DRIFT_FIRST) {
    fm1 = (-k) * r0inv * g2bs;
    gmh = k * r0inv * (h * g2bs - r0 * g3bs);
    dgdtm1 = k * r0inv * rinv * (h * g1bs - r0 * g2bs);
  } else {
    h1 = gh.h1;
    h2 = gh.h2;
    fm1 = k * rinv * (g2bs - k * r0inv * h1);
    gmh = k * rinv * (r0 * h2 + eta * h1);
    dgdtm1 = (-k) * rinv * g2bs;
  }
  for (int j = 0; j < 3; j++) delxv[j] = fm1 * x0[j] + gmh * v0[j];
  for (int j = 0; j < 3; j++) delxv[3 + j] = dfdt * x0[j] + dgdtm1 * v0[j];
  P.gamma = gamma; P.g0 = g0bs; P.g1 = g1bs; P.g2 = g2bs; P.g3 = g3bs; P.h1 = h1; P.h2 = h2;
  P.dfdt = dfdt; P.fm1 = fm1; P.gmh = gmh; P.dgdtm1 = dgdtm1; P.r0 = r0; P.r = r; P.r0inv = r0inv; P.rinv = rinv;
  P.k = k; P.h = h; P.beta = beta0; P.betainv = beta0inv; P.eta = eta; P.sqb = sqb; P.zeta = zeta;
  P.H1v = gh.h1; P.H2v = gh.h2; P.H3v = gh.h3; P.H5v = gh.h5; P.H6v = gh.h6;
}

// ---------------------------------------------------------------- two lanes
// The wide form of the team producer runs each pair solve on two adjacent
// lanes of one warp (role 0 and role 1; `mask` names both, `base` is role
// 0's lane).  Both lanes execute the same instructions.  Where the solve has
// two independent pieces of FP64 work of one shape -- the sin and cos
// series, the Newton update's numerator and denominator, G3 and H1 -- each
// lane evaluates one of them with its own coefficients or operands, and a
// shuffle (no FP64 instruction) hands each result to both.  Every value is
// formed by the same operations in the same order as in kep_delxv, so the
// results are bitwise the same.  A warp issues one FP64 instruction per 64
// cycles however many of them are independent, so one system's step takes
// as long as the FP64 instructions its warp issues; splitting them over two
// lanes removes about a fifth of a drift solve's.

// sincos_kepler on two lanes: role 0 evaluates the sine series, role 1 the
// cosine series; both lanes receive both.
__device__ __forceinline__ void sincos_kepler2(double x, double* s, double* c, int role, unsigned mask, int base) {
  if (fabs(x) > 0.78539816339744831) {
    sincos(x, s, c);
    return;
  }
  const double x2 = x * x;
  double p = role ? -0x1.6827863b97d97p-53 : 0x1.952c77030ad4ap-49;
  p = fma(p, x2, role ? 0x1.ae7f3e733b81fp-45 : -0x1.ae7f3e733b81fp-41);
  p = fma(p, x2, role ? -0x1.93974a8c07c9dp-37 : 0x1.6124613a86d09p-33);
  p = fma(p, x2, role ? 0x1.1eed8eff8d898p-29 : -0x1.ae64567f544e4p-26);
  p = fma(p, x2, role ? -0x1.27e4fb7789f5cp-22 : 0x1.71de3a556c734p-19);
  p = fma(p, x2, role ? 0x1.a01a01a01a01ap-16 : -0x1.a01a01a01a01ap-13);
  p = fma(p, x2, role ? -0x1.6c16c16c16c17p-10 : 0x1.1111111111111p-7);
  p = fma(p, x2, role ? 0x1.5555555555555p-5 : -0x1.5555555555555p-3);
  const double b = x2 * (role ? x2 : x);  // x x2 (sine) or x2 x2 (cosine)
  const double one_minus = fma(-0.5, x2, 1.0);
  const double v = fma(b, p, role ? one_minus : x);
  *s = __shfl_sync(mask, v, base);
  *c = __shfl_sync(mask, v, base + 1);
}

// kep_delxv<DRIFT_FIRST, false> on two lanes (see above); both lanes return
// the same delxv and P.
template <bool DRIFT_FIRST>
__device__ __noinline__ void kep_delxv2(const double* x0, const double* v0, double k, double h, double* delxv,
                                        KepParams& P, int role, unsigned mask, int base) {
  double rt0 = x0[0] - h * v0[0], rt1 = x0[1] - h * v0[1], rt2 = x0[2] - h * v0[2];
  double r0 = DRIFT_FIRST ? sqrt(rt0 * rt0 + rt1 * rt1 + rt2 * rt2) : sqrt(x0[0] * x0[0] + x0[1] * x0[1] + x0[2] * x0[2]);
  double r0inv = 1.0 / r0;
  double beta0 = 2.0 * k * r0inv - (v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2]);
  double beta0inv = 1.0 / beta0;
  double signb = jsign(beta0);
  double sqb = sqrt(signb * beta0);
  double zeta = k - r0 * beta0;
  double eta = DRIFT_FIRST ? (rt0 * v0[0] + rt1 * v0[1] + rt2 * v0[2]) : (x0[0] * v0[0] + x0[1] * v0[1] + x0[2] * v0[2]);
  double gamma_guess;
  if (zeta != 0.0) {
    double zinv = 6.0 / zeta;
    gamma_guess = cubic1(0.5 * eta * sqb * zinv, r0 * signb * beta0 * zinv, (-h) * signb * beta0 * sqb * zinv);
  } else if (eta != 0.0) {
    double reta = r0 / eta;
    double disc = reta * reta + 2.0 * h / eta;
    gamma_guess = (disc > 0.0) ? sqb * ((-reta) + sqrt(disc)) : h * r0inv * sqb;
  } else {
    gamma_guess = h * r0inv * sqb;
  }
  double gamma = gamma_guess;
  double gamma1 = 2.0 * gamma, gamma2 = 3.0 * gamma;
  double c2 = -2.0 * zeta, c3 = 2.0 * eta * signb * sqb, c4 = (-sqb) * h * beta0, c5 = 2.0 * eta * signb * sqb;
  // the update's numerator k gamma + c2 sx cx + c3 sx^2 + c4 (role 0) and
  // denominator 2 signb zeta sx^2 + c5 sx cx + r0 beta0 (role 1), term by term
  const double kz = 2.0 * signb * zeta, rb = r0 * beta0;
  const double a1 = role ? kz : k, a2 = role ? c5 : c2, a3 = role ? 1.0 : c3, a4 = role ? 0.0 : c4;
  double sx, cx;
  int iter = 0;
  while (iter < 20) {
    gamma2 = gamma1;
    gamma1 = gamma;
    double xx = 0.5 * gamma;
    if (beta0 > 0.0) {
      sincos_kepler2(xx, &sx, &cx, role, mask, base);
    } else {
      sx = sinh(xx);
      cx = exp(-xx) + sx;
    }
    const double ss = sx * sx;
    double acc = a1 * (role ? ss : gamma) + (a2 * sx) * cx;
    acc = acc + a3 * (role ? rb : ss);  // 1.0 * (r0 beta0) is r0 beta0 exactly
    const double acc4 = acc + a4;
    acc = role ? acc : acc4;
    const double num = __shfl_sync(mask, acc, base);
    const double den = __shfl_sync(mask, acc, base + 1);
    gamma = gamma - num / den;
    iter += 1;
    if (gamma == gamma2 || gamma == gamma1) break;
  }
  P.newton_iter = iter;
  double xx = 0.5 * gamma;
  if (beta0 > 0.0) {
    sincos_kepler2(xx, &sx, &cx, role, mask, base);
  } else {
    sx = sinh(xx);
    cx = exp(-xx) + sx;
  }
  double g1bs = 2.0 * sx * cx / sqb;
  double g2bs = 2.0 * signb * (sx * sx) * beta0inv;
  double g0bs = 1.0 - beta0 * g2bs;
  GH gh;
  if (DRIFT_FIRST) {
    gh = gh_functions<GH_G3>(gamma, beta0, sqb);
  } else if (gamma < 0.5) {
    // G3 (role 0) and H1 (role 1) as gh_functions forms them; H2 on both
    const double x2 = (-jsign(beta0)) * (gamma * gamma);
    const double poly = gh_horner(kGHCoef[role ? 1 : 0], x2);
    const double pn = (role ? x2 : -x2) * (role ? x2 : gamma);          // (-x2) gamma | x2 x2
    const double pd = ((role ? beta0 : 6.0) * beta0) * (role ? 12.0 : sqb);  // (6 beta) sqb | 12 (beta beta)
    const double v = poly * (pn / pd);
    gh.g3 = __shfl_sync(mask, v, base);
    gh.h1 = __shfl_sync(mask, v, base + 1);
    gh.h2 = gh_horner(kGHCoef[2], x2) * (((-x2) * gamma) / ((3.0 * beta0) * sqb));
    gh.h3 = gh.h5 = gh.h6 = 0.0;
  } else {
    gh = gh_functions<GH_G3 | GH_H1 | GH_H2>(gamma, beta0, sqb);
  }
  double g3bs = gh.g3;
  double h1 = 0.0, h2 = 0.0;
  double r = r0 * g0bs + eta * g1bs + k * g2bs;
  double rinv = 1.0 / r;
  double dfdt = (-k) * g1bs * rinv * r0inv;
  double fm1, gmh, dgdtm1;
  if (DRIFT_FIRST) {
    fm1 = (-k) * r0inv * g2bs;
    gmh = k * r0inv * (h * g2bs - r0 * g3bs);
    dgdtm1 = k * r0inv * rinv * (h * g1bs - r0 * g2bs);
  } else {
    h1 = gh.h1;
    h2 = gh.h2;
    fm1 = k * rinv * (g2bs - k * r0inv * h1);
    gmh = k * rinv * (r0 * h2 + eta * h1);
    dgdtm1 = (-k) * rinv * g2bs;
  }
  for (int j = 0; j < 3; j++) delxv[j] = fm1 * x0[j] + gmh * v0[j];
  for (int j = 0; j < 3; j++) delxv[3 + j] = dfdt * x0[j] + dgdtm1 * v0[j];
  P.gamma = gamma; P.g0 = g0bs; P.g1 = g1bs; P.g2 = g2bs; P.g3 = g3bs; P.h1 = h1; P.h2 = h2;
  P.dfdt = dfdt; P.fm1 = fm1; P.gmh = gmh; P.dgdtm1 = dgdtm1; P.r0 = r0; P.r = r; P.r0inv = r0inv; P.rinv = rinv;
  P.k = k; P.h = h; P.beta = beta0; P.betainv = beta0inv; P.eta = eta; P.sqb = sqb; P.zeta = zeta;
  P.H1v = gh.h1; P.H2v = gh.h2; P.H3v = gh.h3; P.H5v = gh.h5; P.H6v = gh.h6;
}

// compute_jacobian_gamma! (ahl21.jl:896-1139, debug = false).  jk is the 6x8
// jac_kepler (col-major: jk[row + 6 col]); jm the 6-vector jac_mass.
template <bool DRIFT_FIRST>
__device__ __noinline__ void kep_jacobian(const KepParams& P, const double* x0, const double* v0, double* jk,
                                             double* jm) {
  const double G = GNEWT;
  const double gamma = P.gamma, g0 = P.g0, g1 = P.g1, g2 = P.g2, g3 = P.g3, h1 = P.h1;
  const double dfdt = P.dfdt, fm1 = P.fm1, gmh = P.gmh, dgdtm1 = P.dgdtm1, r0 = P.r0, r = P.r;
  const double r0inv = P.r0inv, rinv = P.rinv, k = P.k, h = P.h, beta = P.beta, betainv = P.betainv;
  const double eta = P.eta, sqb = P.sqb, zeta = P.zeta;
  // repeated divisors of the reference's expressions, inverted once
  const double g1inv = 1.0 / g1, g2inv = 1.0 / g2, kinv = 1.0 / k;
  double r0inv2 = r0inv * r0inv;
  double r0inv3 = r0inv2 * r0inv;
  double rinv2 = rinv * rinv;
  double rinv3 = rinv2 * rinv;
  double hsq = h * h;
  double ksq = k * k;
  double d = (h + eta * g2 + 2.0 * k * g3) * betainv;
  double c1 = d - r0 * g3;
  double c2 = eta * g0 + g1 * zeta;
  double c3 = d * k + g1 * (r0 * r0);
  double h6 = P.H6v, h3 = P.H3v, h5 = P.H5v;
  double h8 = (-(2.0 * h3)) + 3.0 * h5;
  double dfm1dxx, dfm1dxv, dfm1dvx, dfm1dvv, dfm1dh, dfm1dk, dfm1dk2;
  double dgmhdxx, dgmhdxv, dgmhdvx, dgmhdvv, dgmhdh, dgmhdk, dgmhdk2;
  double ddfdtdxx, ddfdtdxv, ddfdtdvx, ddfdtdvv, ddfdtdk, ddfdtdk2, ddfdtdh;
  double dgdxx, dgdxv, dgdvx, dgdvv, dgdk, dgdk2, dgdh;
  if (DRIFT_FIRST) {
    double c13 = g1 * h - g2 * r0;
    double c9 = 2.0 * g2 * h - 3.0 * g3 * r0;
    double c10 = k * (r0inv2 * r0inv2) * ((-g2) * r0 * h + k * c9 * betainv - c3 * c13 * rinv);
    double c24 = r0inv3 * (r0 * (2.0 * k * r0inv - beta) * betainv - g1 * c3 * rinv * g2inv);
    dfm1dxx = fm1 * c24;
    dfm1dxv = (-fm1) * (g1 * rinv + h * c24);
    dfm1dvx = dfm1dxv;
    dfm1dvv = fm1 * rinv * ((-r0) * g2 + k * h6 * betainv * g2inv + h * (2.0 * g1 + h * r * c24));
    dfm1dh = fm1 * (g1 * rinv * (g2inv + 2.0 * k * r0inv - beta) - eta * c24);
    dfm1dk = fm1 * (kinv + g1 * c1 * rinv * r0inv * g2inv - 2.0 * betainv * r0inv);
    double h4 = (-P.H1v) * beta;
    dfm1dk2 = (r0 * h4 + k * h6);
    dgmhdxx = c10;
    dgmhdxv = (-g2) * k * c13 * rinv * r0inv - h * c10;
    dgmhdvx = dgmhdxv;
    dgmhdvv = 2.0 * g2 * h * k * c13 * rinv * r0inv + hsq * c10 +
              k * betainv * rinv * r0inv * ((r0 * r0) * h8 - beta * h * r0 * (g2 * g2) + (h * k + eta * r0) * h6);
    dgmhdh = g2 * k * r0inv + k * c13 * rinv * r0inv + g2 * k * (2.0 * k * r0inv - beta) * c13 * rinv * r0inv -
             eta * c10;
    dgmhdk = r0inv * (k * c1 * c13 * rinv * r0inv + g2 * h - g3 * r0 - k * c9 * betainv * r0inv);
    dgmhdk2 = (h6 * g3 * ksq + eta * r0 * (h6 + g2 * h4) + (r0 * r0) * g0 * h5 + k * eta * g2 * h6 +
               (g1 * h6 + g3 * h4) * k * r0);
    double c12 = g0 * h - g1 * r0;
    double c17 = r0 - r - g2 * k;
    double c21 = (g2 * k - r0) * (beta * c3 - k * g1 * r) * betainv * rinv2 * r0inv3 * g1inv +
                 eta * g1 * rinv * r0inv2 - 2.0 * r0inv2;
    double c22 = rinv * ((-g1) - g0 * g2 * g1inv + g2 * c2 * rinv);
    double c25 = k * rinv * r0inv2 *
                 ((-g2) + k * (c13 - g2 * r0) * betainv * r0inv2 - c13 * r0inv - c12 * c3 * rinv * r0inv2 +
                  c13 * c2 * c3 * rinv2 * r0inv2 - c13 * (k * (g2 * k + r) - g0 * r0 * zeta) * betainv * rinv * r0inv2);
    double c26 = k * rinv2 * r0inv * ((-g2) * c12 - g1 * c13 + g2 * c13 * c2 * rinv);
    ddfdtdxx = dfdt * c21;
    ddfdtdxv = dfdt * (c22 - h * c21);
    ddfdtdvx = ddfdtdxv;
    double c34 = ((-beta) * (eta * eta) * (g2 * g2) - eta * k * h8 - h6 * ksq - 2.0 * beta * eta * r0 * g1 * g2 +
                  ((g2 * g2) - 3.0 * g1 * g3) * beta * k * r0 - beta * (g1 * g1) * (r0 * r0)) *
                     betainv * rinv2 +
                 (eta * (g2 * g2)) * rinv * g1inv + (k * h8) * betainv * rinv * g1inv;
    ddfdtdvv = dfdt * (c34 - 2.0 * h * c22 + hsq * c21);
    ddfdtdk = dfdt * (kinv - betainv * r0inv - c17 * betainv * rinv * r0inv -
                      c1 * (g1 * c2 - g0 * r) * rinv2 * r0inv * g1inv);
    ddfdtdk2 = (-(g2 * k - r0)) * (beta * r0 * (g3 - g1 * g2) - beta * eta * (g2 * g2) + k * h3) * betainv * rinv2 *
               r0inv;
    ddfdtdh = dfdt * (g0 * rinv * g1inv - c2 * rinv2 - (2.0 * k * r0inv - beta) * c22 - eta * c21);
    dgdxx = c25;
    dgdxv = c26 - h * c25;
    dgdvx = c26 - h * c25;
    double h2 = P.H2v;
    double c33 = d * k * rinv3 * r0inv * k * (h * g2 - r0 * g3) +
                 k *
                     ((-eta) * k * g1 * (g2 * g2) - g1 * g2 * g3 * ksq - r0 * eta * beta * g1 * (g2 * g2) -
                      r0 * k * g1 * h2 - beta * (g2 * g2) * g0 * (r0 * r0)) *
                     betainv * rinv2 * r0inv;
    dgdvv = c33 - 2.0 * h * c26 + hsq * c25;
    dgdk = rinv * r0inv *
           ((-k) * (c13 - g2 * r0) * betainv * r0inv + c13 - k * c13 * c17 * betainv * rinv * r0inv +
            k * c1 * c12 * rinv * r0inv - k * c1 * c2 * c13 * rinv2 * r0inv);
    dgdk2 = k * betainv * rinv2 * r0inv *
            ((-beta) * (eta * eta) * pow4(g2) + eta * g2 * (g1 * (g2 * g2) + (g1 * g1) * g3 - 5.0 * g2 * g3) * k +
             g2 * g3 * h3 * ksq + 2.0 * eta * r0 * beta * (g2 * g2) * (g3 - g1 * g2) +
             (4.0 * g3 - g0 * g3 - g1 * g2) * (g3 - g1 * g2) * r0 * k +
             beta * (2.0 * g1 * g3 * g2 - (g1 * g1) * (g2 * g2) - (g3 * g3)) * (r0 * r0));
    dgdh = g1 * k * rinv * r0inv + k * c12 * rinv2 * r0inv - k * c2 * c13 * rinv3 * r0inv -
           (2.0 * k * r0inv - beta) * c26 - eta * c25;
  } else {
    const double h2 = P.h2;
    double c14 = r0 * g2 - k * h1;
    double c15 = eta * h1 + h2 * r0;
    double c16 = eta * h2 + g1 * gamma * r0 * (1.0 / sqb);
    double c17 = r0 - r - g2 * k;
    double c19 = 4.0 * eta * h1 + 3.0 * h2 * r0;
    double c23 = h2 * k - r0 * g1;
    dfm1dxx = k * rinv3 * betainv * pow4(r0inv) *
              (k * h1 * (r * r) * r0 * (beta - 2.0 * k * r0inv) + beta * c3 * (r * c23 + c14 * c2) +
               c14 * r * (k * (r - g2 * k) + g0 * r0 * zeta));
    dfm1dxv = k * rinv2 * r0inv * (k * (g2 * h2 + g1 * h1) - 2.0 * g1 * g2 * r0 + g2 * c14 * c2 * rinv);
    dfm1dvx = dfm1dxv;
    dfm1dvv = k * r0inv * rinv2 * betainv *
              (2.0 * eta * k * (g2 * g3 - g1 * h1) + (3.0 * g3 * h2 - 4.0 * h1 * g2) * ksq +
               beta * g2 * r0 * (3.0 * h1 * k - g2 * r0) +
               c14 * rinv *
                   ((-beta) * (g2 * g2) * (eta * eta) + eta * k * (2.0 * g0 * g3 - h2) - h6 * ksq +
                    ((-(2.0 * eta)) * g1 * g2 + k * (h1 - 2.0 * g1 * g3)) * beta * r0 - beta * (g1 * g1) * (r0 * r0)));
    dfm1dh = (g1 * k - h2 * ksq * r0inv - k * c14 * c2 * rinv * r0inv) * rinv2;
    dfm1dk = rinv * r0inv *
             (4.0 * h1 * ksq * betainv * r0inv - k * h1 - 2.0 * g2 * k * betainv + c14 -
              k * c14 * c17 * betainv * rinv * r0inv + k * (g1 * r0 - k * h2) * c1 * rinv * r0inv -
              k * c14 * c1 * c2 * rinv2 * r0inv);
    dfm1dk2 = betainv * r0inv * rinv2 *
              (r * (2.0 * eta * k * (g1 * h1 - g3 * g2) + (4.0 * g2 * h1 - 3.0 * g3 * h2) * ksq -
                    eta * r0 * beta * g1 * h1 + (g3 * h2 - 4.0 * g2 * h1) * beta * k * r0 +
                    g2 * h1 * (beta * beta) * (r0 * r0)) -
               c14 * ((-(eta * eta)) * beta * (g2 * g2) - k * eta * h8 - ksq * h6 -
                      eta * r0 * beta * (g1 * g2 + g0 * g3) + 2.0 * (h1 - g1 * g3) * beta * k * r0 -
                      (g2 - beta * g1 * g3) * beta * (r0 * r0)));
    dgmhdxx = k * rinv * r0inv *
              (h2 + k * c19 * betainv * r0inv2 - c16 * c3 * rinv * r0inv2 +
               c2 * c3 * c15 * ((rinv * r0inv) * (rinv * r0inv)) -
               c15 * (k * (g2 * k + r) - g0 * r0 * zeta) * betainv * rinv * r0inv2);
    dgmhdxv = k * rinv2 * (h1 * r - g2 * c16 - g1 * c15 + g2 * c2 * c15 * rinv);
    dgmhdvx = dgmhdxv;
    dgmhdvv = k * betainv * rinv2 *
              (2.0 * (eta * eta) * (g1 * h1 - g2 * g3) + eta * k * (4.0 * g2 * h1 - 3.0 * h2 * g3) +
               r0 * eta * (4.0 * g0 * h1 - 2.0 * g1 * g3) + 3.0 * r0 * k * ((g1 + beta * g3) * h1 - g3 * g2) +
               (g0 * h8 - beta * g1 * ((g2 * g2) + g1 * g3)) * (r0 * r0) -
               c15 * rinv *
                   (beta * (g2 * g2) * (eta * eta) + eta * k * h8 + h6 * ksq +
                    (2.0 * eta * g1 * g2 - k * ((g2 * g2) - 3.0 * g1 * g3)) * beta * r0 + beta * (g1 * g1) * (r0 * r0)));
    dgmhdk = rinv * (k * c1 * c16 * rinv * r0inv + c15 - k * c15 * c17 * betainv * rinv * r0inv -
                     k * c19 * betainv * r0inv - k * c1 * c2 * c15 * rinv2 * r0inv);
    double h7 = beta * g1 * (g2 * g2) - g0 * h8;
    dgmhdk2 = betainv * rinv2 *
              (r * (2.0 * (eta * eta) * (g3 * g2 - g1 * h1) + eta * k * (3.0 * g3 * h2 - 4.0 * g2 * h1) +
                    r0 * eta * (beta * g3 * (g1 * g2 + g0 * g3) - 2.0 * g0 * h6) +
                    ((-h6) * (g1 + beta * g3) + g2 * (2.0 * g3 - h2)) * r0 * k +
                    (h7 - (beta * beta) * g1 * (g3 * g3)) * (r0 * r0)) -
               c15 * ((-beta) * (eta * eta) * (g2 * g2) + eta * k * ((-h2) + 2.0 * g0 * g3) - h6 * ksq -
                      r0 * eta * beta * (h2 + 2.0 * g0 * g3) + 2.0 * beta * (2.0 * h1 - (g2 * g2)) * r0 * k +
                      beta * (beta * g1 * g3 - g2) * (r0 * r0)));
    dgmhdh = k * rinv3 * (r * c16 - c2 * c15);
    ddfdtdxx = dfdt *
               (eta * g1 * rinv - 2.0 - g0 * c3 * rinv * r0inv * g1inv + c2 * c3 * r0inv * rinv2 -
                k * (k * g2 - r0) * betainv * rinv * r0inv) *
               r0inv2;
    ddfdtdxv = (-dfdt) * (g0 * g2 * g1inv + (r0 * g1 + eta * g2) * rinv) * rinv;
    ddfdtdvx = ddfdtdxv;
    ddfdtdvv = (-k) * rinv3 * r0inv * betainv *
               ((beta * eta * (g2 * g2) + k * h8) * (r0 * g0 + k * g2) +
                g1 * ((-h6) * ksq + ((-(2.0 * eta)) * g1 * g2 + (h1 - 2.0 * g1 * g3) * k) * beta * r0 -
                      beta * (g1 * g1) * (r0 * r0)));
    ddfdtdk = dfdt * (kinv + c1 * (r0 - g2 * k) * r0inv * rinv2 * g1inv - betainv * r0inv * (1.0 + c17 * rinv));
    ddfdtdk2 = (r0 - g2 * k) * betainv * r0inv * rinv2 * ((-eta) * beta * (g2 * g2) + h3 * k + (g3 - g1 * g2) * beta * r0);
    ddfdtdh = dfdt * (r0 - g2 * k) * rinv2 * g1inv;
    dgdxx = rinv2 * r0inv3 *
            ((eta * g2 + g1 * r0) * k * c3 * rinv + g2 * k * (k * (g2 * k - r) - g0 * r0 * zeta) * betainv);
    dgdxv = k * g2 * rinv3 * (r * g1 + r0 * g1 + eta * g2);
    dgdvx = dgdxv;
    dgdvv = k * betainv * rinv3 *
            ((eta * eta) * beta * (g2 * g2 * g2) - eta * k * g2 * h3 + 3.0 * r0 * eta * beta * g1 * (g2 * g2) +
             r0 * k * ((-g0) * h6 + 3.0 * beta * g1 * g2 * g3) + beta * g2 * (g0 * g2 + (g1 * g1)) * (r0 * r0));
    dgdk = rinv * r0inv *
           ((-r0) * g2 + g2 * k * (r + r0 - g2 * k) * betainv * rinv - k * g1 * c1 * rinv + k * g2 * c1 * c2 * rinv2);
    dgdk2 = betainv * rinv2 *
            ((-beta) * (eta * eta) * (g2 * g2 * g2) + eta * k * g2 * h3 + eta * r0 * beta * g2 * (g3 - 2.0 * g1 * g2) +
             (h6 - beta * (g2 * g2 * g2)) * r0 * k + beta * g1 * (g3 - g1 * g2) * (r0 * r0));
    dgdh = k * rinv3 * (g2 * c2 - r * g1);
  }
  for (int q = 0; q < 48; q++) jk[q] = 0.0;
  for (int j = 0; j < 3; j++) {
    jk[j + 6 * j] = fm1;
    jk[j + 6 * (3 + j)] = gmh;
    for (int i = 0; i < 3; i++) {
      jk[j + 6 * i] = jk[j + 6 * i] + ((dfm1dxx * x0[i] + dfm1dxv * v0[i]) * x0[j] +
                                       (dgmhdxx * x0[i] + dgmhdxv * v0[i]) * v0[j]);
      jk[j + 6 * (3 + i)] = jk[j + 6 * (3 + i)] + ((dfm1dvx * x0[i] + dfm1dvv * v0[i]) * x0[j] +
                                                   (dgmhdvx * x0[i] + dgmhdvv * v0[i]) * v0[j]);
    }
    jk[j + 6 * 6] = dfm1dk * x0[j] + dgmhdk * v0[j];
    jk[j + 6 * 7] = dfm1dh * x0[j] + dgmhdh * v0[j];
    if (DRIFT_FIRST)
      jm[j] = (G * r0inv) * (G * r0inv) * betainv * rinv * (dfm1dk2 * x0[j] - dgmhdk2 * v0[j]);
    else
      jm[j] = G * G * rinv * r0inv * (dfm1dk2 * x0[j] + dgmhdk2 * v0[j]);
  }
  for (int j = 0; j < 3; j++) {
    jk[3 + j + 6 * j] = dfdt;
    jk[3 + j + 6 * (3 + j)] = dgdtm1;
    for (int i = 0; i < 3; i++) {
      jk[3 + j + 6 * i] = jk[3 + j + 6 * i] + ((ddfdtdxx * x0[i] + ddfdtdxv * v0[i]) * x0[j] +
                                               (dgdxx * x0[i] + dgdxv * v0[i]) * v0[j]);
      jk[3 + j + 6 * (3 + i)] = jk[3 + j + 6 * (3 + i)] + ((ddfdtdvx * x0[i] + ddfdtdvv * v0[i]) * x0[j] +
                                                           (dgdvx * x0[i] + dgdvv * v0[i]) * v0[j]);
    }
    jk[3 + j + 6 * 6] = ddfdtdk * x0[j] + dgdk * v0[j];
    jk[3 + j + 6 * 7] = ddfdtdh * x0[j] + dgdh * v0[j];
    if (DRIFT_FIRST)
      jm[3 + j] = G * G * r0inv * rinv * (ddfdtdk2 * x0[j] + dgdk2 * v0[j]);
    else
      jm[3 + j] = G * G * rinv * r0inv * (ddfdtdk2 * x0[j] + dgdk2 * v0[j]);
  }
}

}  // namespace nbg
