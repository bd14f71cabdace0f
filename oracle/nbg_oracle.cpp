// nbg_oracle.cpp -- C-ABI of the CPU oracle (TEST INFRASTRUCTURE ONLY).
//
// Built by oracle/Makefile into oracle/_build/liboracle.so.  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.  All array
// arguments follow the reference's Julia column-major layouts (see
// nbg_oracle.hpp); body indices passed in are 0-based.
//
// The oracle_fd_* entry points restate the reference's finite-difference
// tests.  They run the no-gradient map in __float128 (standing in for the
// reference's BigFloat) and return double-rounded numerical derivatives.
#include "nbg_oracle.hpp"

#include <thread>
#include <atomic>

using namespace nbgo;

namespace {

template <class T> void load_state(State<T>& s, int n, const double* x, const double* v, const double* m,
                                   const double* xerr, const double* verr, const double* jac_step,
                                   const double* jac_err, const double* dqdt, const uint8_t* pair,
                                   const double* jac_init) {
  s.alloc(n);
  int M = 7 * n;
  for (int q = 0; q < 3 * n; q++) {
    s.x[q] = T(x[q]); s.v[q] = T(v[q]);
    s.xerror[q] = xerr ? T(xerr[q]) : T(0);
    s.verror[q] = verr ? T(verr[q]) : T(0);
  }
  for (int q = 0; q < n; q++) s.m[q] = T(m[q]);
  if (jac_step) for (size_t q = 0; q < (size_t)M * M; q++) s.jac_step[q] = T(jac_step[q]);
  if (jac_err) for (size_t q = 0; q < (size_t)M * M; q++) s.jac_error[q] = T(jac_err[q]);
  if (jac_init) for (size_t q = 0; q < (size_t)M * M; q++) s.jac_init[q] = T(jac_init[q]);
  if (dqdt) for (int q = 0; q < M; q++) s.dqdt[q] = T(dqdt[q]);
  if (pair) for (int q = 0; q < n * n; q++) s.pair[q] = pair[q];
}

template <class T> void store_state(const State<T>& s, double* x, double* v, double* xerr, double* verr,
                                    double* jac_step, double* jac_err, double* dqdt) {
  int n = s.n, M = 7 * n;
  for (int q = 0; q < 3 * n; q++) {
    if (x) x[q] = (double)s.x[q];
    if (v) v[q] = (double)s.v[q];
    if (xerr) xerr[q] = (double)s.xerror[q];
    if (verr) verr[q] = (double)s.verror[q];
  }
  if (jac_step) for (size_t q = 0; q < (size_t)M * M; q++) jac_step[q] = (double)s.jac_step[q];
  if (jac_err) for (size_t q = 0; q < (size_t)M * M; q++) jac_err[q] = (double)s.jac_error[q];
  if (dqdt) for (int q = 0; q < M; q++) dqdt[q] = (double)s.dqdt[q];
}

// Perturbation of the reference's tests: dq = dlnq*q (dlnq when q == 0).
// BigFloat's 256-bit precision absorbs a relative step on a coordinate that is
// zero up to rounding (~1e-19 next to 1e-2); binary128 does not, so the step
// is floored at 1e-6 of the array's scale.
static inline quad fd_step(quad q, quad dlnq, quad scale) {
  quad a = (q < quad(0)) ? -q : q;
  quad fl = quad(1e-6) * scale;
  return dlnq * (a > fl ? a : (fl > quad(0) ? fl : quad(1)));
}
template <class T> static quad absmax(const std::vector<T>& a) {
  quad s = quad(0);
  for (auto q : a) { quad b = (q < T(0)) ? -quad(q) : quad(q); if (b > s) s = b; }
  return s;
}

}  // namespace

// R: the arithmetic type (double for parity; quad for the rounding-error
// reference the parity tests use to size their tolerances).
template <class R>
static int integrate_transits_nr(int nr, int n, int ti, double h, double tmax, int grad, double* t, double* x,
                                 double* v, const double* m, double* xerr, double* verr, double* jac_step,
                                 double* jac_err, double* dqdt, const uint8_t* pair, const double* jac_init, int ntt,
                                 double* tt, double* dtdq0, double* dtdelements, int64_t* count) {
  if (n < 2 || ti < 0 || ti >= n || ntt < 1) return -1;
  State<R> s;
  load_state(s, n, x, v, m, xerr, verr, jac_step, jac_err, dqdt, pair, jac_init);
  s.t = R(*t);
  TransitTiming<R> T;
  T.alloc(n, ntt, ti, nr);
  size_t n4 = (size_t)nr * n * ntt * 7 * n;
  for (size_t q = 0; q < (size_t)nr * n * ntt; q++) T.tt[q] = R(tt[q]);
  for (size_t q = 0; q < n4; q++) {
    T.dtdq0[q] = R(dtdq0[q]);
    T.dtdelements[q] = R(dtdelements[q]);
  }
  for (int q = 0; q < n; q++) T.count[q] = count[q];
  T.s_prior.alloc(n);
  intr_transits(s, T, R(h), R(tmax), grad != 0);
  store_state(s, x, v, xerr, verr, jac_step, jac_err, dqdt);
  *t = (double)s.t;
  for (size_t q = 0; q < T.tt.size(); q++) tt[q] = (double)T.tt[q];
  for (size_t q = 0; q < n4; q++) {
    dtdq0[q] = (double)T.dtdq0[q];
    dtdelements[q] = (double)T.dtdelements[q];
  }
  for (int q = 0; q < n; q++) count[q] = T.count[q];
  return 0;
}

extern "C" {

int oracle_version(void) { return 1; }

// Exact-zero entries of the operators skipped in the dense products (1) or
// multiplied as the reference's mul! does (0, the default); both give
// bitwise the same results for finite inputs.  Returns the previous setting.
int oracle_set_skip_zero_products(int on) {
  return skip_zero_products_flag().exchange(on != 0) ? 1 : 0;
}

// Transit Newton searches that stopped at ITMAX on this thread so far.
long long oracle_newton_itmax_hits(void) { return newton_itmax_hits(); }

// ElementsIC(t0, H, elements) -> init_nbody.  H may be NULL (fully nested).
int oracle_init_nbody(int n, double t0, const double* elements, const double* H, double* x, double* v,
                      double* jac_init) {
  std::vector<double> Hn((size_t)n * n);
  if (H) std::copy(H, H + (size_t)n * n, Hn.begin());
  else hierarchy_nested<double>(n, Hn.data());
  return init_nbody<double>(n, t0, elements, Hn.data(), x, v, jac_init) ? 0 : -1;
}

// intr(s, tt; grad) on one system (Transits.jl:140-180).  State arrays are
// updated in place; tt, dtdq0, dtdelements and count are in/out as in the
// reference's TransitTiming.  t is in/out (s.t).
int oracle_integrate_transits(int n, int ti, double h, double tmax, int grad, double* t, double* x, double* v,
                              const double* m, double* xerr, double* verr, double* jac_step, double* jac_err,
                              double* dqdt, const uint8_t* pair, const double* jac_init, int ntt, double* tt,
                              double* dtdq0, double* dtdelements, int64_t* count) {
  return integrate_transits_nr<double>(1, n, ti, h, tmax, grad, t, x, v, m, xerr, verr, jac_step, jac_err, dqdt, pair,
                               jac_init, ntt, tt, dtdq0, dtdelements, count);
}

// intr(s, ttbv::TransitParameters; grad) (Transits.jl:140-180 with the
// TransitParameters branch of timing.jl:82-98): ttbv 3 x n x ntt,
// dtbvdq0 / dtbvdelements 3 x n x ntt x 7 x n.
int oracle_integrate_transit_parameters(int n, int ti, double h, double tmax, int grad, double* t, double* x,
                                        double* v, const double* m, double* xerr, double* verr, double* jac_step,
                                        double* jac_err, double* dqdt, const uint8_t* pair, const double* jac_init,
                                        int ntt, double* ttbv, double* dtbvdq0, double* dtbvdelements,
                                        int64_t* count) {
  return integrate_transits_nr<double>(3, n, ti, h, tmax, grad, t, x, v, m, xerr, verr, jac_step, jac_err, dqdt,
                                       pair, jac_init, ntt, ttbv, dtbvdq0, dtbvdelements, count);
}

// The same in quad precision (outputs rounded to double): the rounding-error
// reference for the parity tolerances of the v_sky and b_sky^2 rows.
int oracle_integrate_transit_parameters_quad(int n, int ti, double h, double tmax, int grad, double* t, double* x,
                                             double* v, const double* m, double* xerr, double* verr,
                                             double* jac_step, double* jac_err, double* dqdt, const uint8_t* pair,
                                             const double* jac_init, int ntt, double* ttbv, double* dtbvdq0,
                                             double* dtbvdelements, int64_t* count) {
  return integrate_transits_nr<quad>(3, n, ti, h, tmax, grad, t, x, v, m, xerr, verr, jac_step, jac_err, dqdt,
                                     pair, jac_init, ntt, ttbv, dtbvdq0, dtbvdelements, count);
}

// Batched CPU baseline: nsys independent systems of equal n, packed
// system-major (x: 3n per system, J: (7n)^2 per system, ...).  Uses up to
// nthreads host threads, one system at a time per thread.
int oracle_integrate_transits_batch(int nsys, int nthreads, int n, int ti, const double* h, const double* tmax,
                                    int grad, double* t, double* x, double* v, const double* m, double* xerr,
                                    double* verr, double* jac_step, double* jac_err, double* dqdt,
                                    const uint8_t* pair, const double* jac_init, int ntt, double* tt,
                                    double* dtdq0, double* dtdelements, int64_t* count) {
  if (nthreads < 1) nthreads = 1;
  int M = 7 * n;
  size_t MM = (size_t)M * M, n4 = (size_t)n * ntt * 7 * n;
  std::atomic<int> next(0), fail(0);
  auto work = [&]() {
    while (true) {
      int s = next.fetch_add(1);
      if (s >= nsys) break;
      int rc = oracle_integrate_transits(
          n, ti, h[s], tmax[s], grad, t + s, x + (size_t)3 * n * s, v + (size_t)3 * n * s, m + (size_t)n * s,
          xerr + (size_t)3 * n * s, verr + (size_t)3 * n * s, jac_step + MM * s, jac_err + MM * s,
          dqdt + (size_t)M * s, pair ? pair + (size_t)n * n * s : nullptr, jac_init + MM * s, ntt,
          tt + (size_t)n * ntt * s, dtdq0 + n4 * s, dtdelements + n4 * s, count + (size_t)n * s);
      if (rc) fail.store(rc);
    }
  };
  std::vector<std::thread> th;
  for (int q = 1; q < nthreads; q++) th.emplace_back(work);
  work();
  for (auto& q : th) q.join();
  return fail.load();
}

// intr(s, time; grad) (Integrator.jl:159-197)
int oracle_integrate_time(int n, double h, double time, int grad, double* t, double* x, double* v,
                          const double* m, double* xerr, double* verr, double* jac_step, double* jac_err,
                          double* dqdt, const uint8_t* pair) {
  State<double> s;
  load_state(s, n, x, v, m, xerr, verr, jac_step, jac_err, dqdt, pair, nullptr);
  s.t = *t;
  intr_time(s, h, time, grad != 0);
  store_state(s, x, v, xerr, verr, jac_step, jac_err, dqdt);
  *t = s.t;
  return 0;
}

// intr(s, N; grad) (Integrator.jl:211-234)
int oracle_integrate_nsteps(int n, double h, int64_t nsteps, int grad, double* t, double* x, double* v,
                            const double* m, double* xerr, double* verr, double* jac_step, double* jac_err,
                            double* dqdt, const uint8_t* pair) {
  State<double> s;
  load_state(s, n, x, v, m, xerr, verr, jac_step, jac_err, dqdt, pair, nullptr);
  s.t = *t;
  double hh = h;
  intr_nsteps(s, hh, nsteps, grad != 0);
  store_state(s, x, v, xerr, verr, jac_step, jac_err, dqdt);
  *t = s.t;
  return 0;
}

// One ahl21! step (grad: ahl21.jl:5-95; no grad: ahl21_no_grad.jl:6-18).
int oracle_ahl21_step(int n, double h, int grad, double* x, double* v, const double* m, double* xerr, double* verr,
                      double* jac_step, double* jac_err, double* dqdt, const uint8_t* pair) {
  State<double> s;
  load_state(s, n, x, v, m, xerr, verr, jac_step, jac_err, dqdt, pair, nullptr);
  if (grad) {
    Derivs<double> d;
    d.alloc(n);
    ahl21(s, d, h);
  } else {
    ahl21_ng(s, h);
  }
  store_state(s, x, v, xerr, verr, jac_step, jac_err, dqdt);
  return 0;
}

// kepler_driftij_gamma! with Jacobian for one pair (ahl21.jl:706-760).
int oracle_kepler_driftij(int n, int i, int j, double h, int drift_first, double* x, double* v, const double* m,
                          double* xerr, double* verr, double* jac_ij, double* dqdt_ij) {
  State<double> s;
  load_state(s, n, x, v, m, xerr, verr, nullptr, nullptr, nullptr, nullptr, nullptr);
  Derivs<double> d;
  d.alloc(n);
  kepler_driftij_gamma(s, d, i, j, h, drift_first != 0);
  store_state(s, x, v, xerr, verr, nullptr, nullptr, nullptr);
  std::copy(d.jac_ij.begin(), d.jac_ij.end(), jac_ij);
  std::copy(d.dqdt_ij.begin(), d.dqdt_ij.end(), dqdt_ij);
  return 0;
}

// kickfast! (ahl21.jl:337-386) -> jac_kick (7n x 7n), dqdt_kick (7n)
int oracle_kickfast(int n, double h, double* x, double* v, const double* m, double* xerr, double* verr,
                    const uint8_t* pair, double* jac_kick, double* dqdt_kick) {
  State<double> s;
  load_state(s, n, x, v, m, xerr, verr, nullptr, nullptr, nullptr, pair, nullptr);
  Derivs<double> d;
  d.alloc(n);
  kickfast(s, d, h);
  store_state(s, x, v, xerr, verr, nullptr, nullptr, nullptr);
  std::copy(d.jac_kick.begin(), d.jac_kick.end(), jac_kick);
  std::copy(d.dqdt_kick.begin(), d.dqdt_kick.end(), dqdt_kick);
  return 0;
}

// phic! then phisalpha!(alpha) as ahl21! calls them (ahl21.jl:46-47);
// which == 1: phic! only, which == 2: phisalpha! only, else both.
int oracle_phi(int n, double h, double alpha, int which, double* x, double* v, const double* m, double* xerr,
               double* verr, const uint8_t* pair, double* jac_phi, double* dqdt_phi) {
  State<double> s;
  load_state(s, n, x, v, m, xerr, verr, nullptr, nullptr, nullptr, pair, nullptr);
  Derivs<double> d;
  d.alloc(n);
  if (which != 2) phic(s, d, h);
  if (which != 1) phisalpha(s, d, h, alpha);
  store_state(s, x, v, xerr, verr, nullptr, nullptr, nullptr);
  std::copy(d.jac_phi.begin(), d.jac_phi.end(), jac_phi);
  std::copy(d.dqdt_phi.begin(), d.dqdt_phi.end(), dqdt_phi);
  return 0;
}

// ------------------------------------------------------ quad-precision pins



// Numerical 14x14 Jacobian and 14 dq/dt of one no-grad kepler_driftij_gamma!
// call (test/test_kepler_driftij_gamma.jl:60-282).  Columns follow jac_ij:
// (x_i, v_i, m_i, x_j, v_j, m_j); the mass rows are identity.
int oracle_fd_kepler_driftij(int n, int i, int j, double h, int drift_first, const double* x, const double* v,
                             const double* m, double dlnq_d, double* jac_num, double* dqdt_num) {
  quad dlnq = quad(dlnq_d);
  auto run = [&](int which, int comp, quad sign, quad& dq, State<quad>& out) {
    load_state(out, n, x, v, m, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    quad hh = quad(h);
    int bodies[2] = {i, j};
    if (which == 0) { dq = dlnq * hh; hh = hh + sign * dq; }
    else {
      int b = bodies[(which - 1) / 3];
      int kind = (which - 1) % 3;  // 0: x, 1: v, 2: m
      quad& q = (kind == 0) ? out.X(comp, b) : (kind == 1) ? out.V(comp, b) : out.m[b];
      quad scale = (kind == 0) ? absmax(out.x) : (kind == 1) ? absmax(out.v) : absmax(out.m);
      dq = fd_step(q, dlnq, scale);
      q = q + sign * dq;
    }
    kepler_driftij_ng(out, i, j, hh, drift_first != 0);
  };
  for (int q = 0; q < 196; q++) jac_num[q] = 0.0;
  State<quad> sp, sm;
  quad dq;
  run(0, 0, quad(1), dq, sp);
  run(0, 0, quad(-1), dq, sm);
  int bodies[2] = {i, j};
  for (int bb = 0; bb < 2; bb++)
    for (int k = 0; k < 3; k++) {
      dqdt_num[7 * bb + k] = (double)(quad(0.5) * (sp.X(k, bodies[bb]) - sm.X(k, bodies[bb])) / dq);
      dqdt_num[7 * bb + 3 + k] = (double)(quad(0.5) * (sp.V(k, bodies[bb]) - sm.V(k, bodies[bb])) / dq);
    }
  dqdt_num[6] = dqdt_num[13] = 0.0;
  for (int bcol = 0; bcol < 2; bcol++)
    for (int kind = 0; kind < 3; kind++)
      for (int comp = 0; comp < (kind == 2 ? 1 : 3); comp++) {
        int which = 1 + 3 * bcol + kind;
        run(which, comp, quad(1), dq, sp);
        run(which, comp, quad(-1), dq, sm);
        int col = 7 * bcol + (kind == 2 ? 6 : 3 * kind + comp);
        for (int brow = 0; brow < 2; brow++)
          for (int k = 0; k < 3; k++) {
            jac_num[(7 * brow + k) + 14 * col] = (double)(quad(0.5) * (sp.X(k, bodies[brow]) - sm.X(k, bodies[brow])) / dq);
            jac_num[(7 * brow + 3 + k) + 14 * col] =
                (double)(quad(0.5) * (sp.V(k, bodies[brow]) - sm.V(k, bodies[brow])) / dq);
          }
      }
  jac_num[6 + 14 * 6] = 1.0;
  jac_num[13 + 14 * 13] = 1.0;
  return 0;
}

// Order-of-accuracy run of the no-gradient map, restating the energy study
// of examples/energy_conservation.jl:96-183: nsteps of ahl21!(s, h) in
// binary128 from (x, v), with the outer kick fraction 1/kick_den and
// phisalpha!'s alpha (the method's values are 6 and 2; the pin passes others
// to show that its test rejects them).  Returns the final x and v as
// double-double pairs (hi = the rounded value, lo = the rest), so that end
// states of different step sizes can be differenced far below double
// precision, and the largest |E(t) - E(0)| / |E(0)| over the steps, E the
// kinetic plus potential energy of compute_energy (:96-113).
int oracle_order_run_quad(int n, double h, int64_t nsteps, const double* x, const double* v, const double* m,
                          const uint8_t* pair, double kick_den, double alpha, double* x_hi, double* x_lo,
                          double* v_hi, double* v_lo, double* max_rel_denergy) {
  if (n < 2 || nsteps < 0) return -1;
  State<quad> s;
  load_state(s, n, x, v, m, nullptr, nullptr, nullptr, nullptr, nullptr, pair, nullptr);
  const quad G = quad(GNEWT_D);
  auto energy = [&]() {
    quad ke = quad(0), pe = quad(0);
    for (int j = 0; j < n; j++)
      ke += quad(0.5) * s.m[j] * (s.V(0, j) * s.V(0, j) + s.V(1, j) * s.V(1, j) + s.V(2, j) * s.V(2, j));
    for (int j = 0; j < n - 1; j++)
      for (int k = j + 1; k < n; k++) {
        quad dx = s.X(0, j) - s.X(0, k), dy = s.X(1, j) - s.X(1, k), dz = s.X(2, j) - s.X(2, k);
        pe -= G * s.m[j] * s.m[k] / Mth<quad>::sqrt(dx * dx + dy * dy + dz * dz);
      }
    return ke + pe;
  };
  const quad e0 = energy();
  quad worst = quad(0);
  const quad hh = quad(h), kd = quad(kick_den), al = quad(alpha);
  for (int64_t q = 0; q < nsteps; q++) {
    ahl21_ng(s, hh, kd, al);
    quad de = (energy() - e0) / e0;
    if (de < quad(0)) de = -de;
    if (de > worst) worst = de;
  }
  for (int q = 0; q < 3 * n; q++) {
    x_hi[q] = (double)s.x[q];
    x_lo[q] = (double)(s.x[q] - quad(x_hi[q]));
    v_hi[q] = (double)s.v[q];
    v_lo[q] = (double)(s.v[q] - quad(v_hi[q]));
  }
  *max_rel_denergy = (double)worst;
  return 0;
}

// Numerical d(x,v)/d(x0,v0,m) of a no-grad map, for the operator tests
// (test/test_kickfast.jl, test_phic.jl, test_phisalpha.jl) and the full
// step sequence (test/test_integrator.jl:55-144).  op: 0 = nsteps ahl21!
// steps of size h; 1 = kickfast!(h); 2 = phic!(h) then phisalpha!(h, 2);
// 3 = phisalpha!(h, 2) only; 4 = phic!(h) only.  Output is the full 7n x 7n
// Jacobian of the map including the identity.
int oracle_fd_map_jacobian(int n, int op, double h, int64_t nsteps, const double* x, const double* v,
                           const double* m, const uint8_t* pair, double dlnq_d, int nthreads, double* jac_num) {
  int M = 7 * n;
  quad dlnq = quad(dlnq_d);
  auto apply = [&](State<quad>& s) {
    quad hh = quad(h);
    switch (op) {
      case 0: for (int64_t q = 0; q < nsteps; q++) ahl21_ng(s, hh); break;
      case 1: kickfast_ng(s, hh); break;
      case 2: phic_ng(s, hh); phisalpha_ng(s, hh, quad(2)); break;
      case 3: phisalpha_ng(s, hh, quad(2)); break;
      case 4: phic_ng(s, hh); break;
    }
  };
  for (size_t q = 0; q < (size_t)M * M; q++) jac_num[q] = 0.0;
  std::atomic<int> next(0);
  auto work = [&]() {
    while (true) {
      int col = next.fetch_add(1);
      if (col >= M) break;
      int b = col / 7, kk = col % 7;
      State<quad> sp, sm;
      load_state(sp, n, x, v, m, nullptr, nullptr, nullptr, nullptr, nullptr, pair, nullptr);
      load_state(sm, n, x, v, m, nullptr, nullptr, nullptr, nullptr, nullptr, pair, nullptr);
      quad* qp = (kk < 3) ? &sp.X(kk, b) : (kk < 6) ? &sp.V(kk - 3, b) : &sp.m[b];
      quad* qm = (kk < 3) ? &sm.X(kk, b) : (kk < 6) ? &sm.V(kk - 3, b) : &sm.m[b];
      quad scale = (kk < 3) ? absmax(sp.x) : (kk < 6) ? absmax(sp.v) : absmax(sp.m);
      quad dq = fd_step(*qp, dlnq, scale);
      *qp = *qp + dq;
      *qm = *qm - dq;
      apply(sp);
      apply(sm);
      for (int i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) {
          jac_num[(7 * i + k) + (size_t)M * col] = (double)(quad(0.5) * (sp.X(k, i) - sm.X(k, i)) / dq);
          jac_num[(7 * i + 3 + k) + (size_t)M * col] = (double)(quad(0.5) * (sp.V(k, i) - sm.V(k, i)) / dq);
        }
      if (kk == 6) jac_num[(7 * b + 6) + (size_t)M * col] = 1.0;
    }
  };
  std::vector<std::thread> th;
  for (int q = 1; q < nthreads; q++) th.emplace_back(work);
  work();
  for (auto& q : th) q.join();
  return 0;
}

// Numerical dq/dh of one no-grad ahl21! step (test/test_integrator.jl:146-169).
int oracle_fd_dqdt(int n, double h, const double* x, const double* v, const double* m, const uint8_t* pair,
                   double dlnq_d, double* dqdt_num) {
  quad dq = quad(h) * quad(dlnq_d);
  State<quad> sp, sm;
  load_state(sp, n, x, v, m, nullptr, nullptr, nullptr, nullptr, nullptr, pair, nullptr);
  load_state(sm, n, x, v, m, nullptr, nullptr, nullptr, nullptr, nullptr, pair, nullptr);
  ahl21_ng(sp, quad(h) + dq);
  ahl21_ng(sm, quad(h) - dq);
  for (int i = 0; i < n; i++) {
    for (int k = 0; k < 3; k++) {
      dqdt_num[7 * i + k] = (double)(quad(0.5) * (sp.X(k, i) - sm.X(k, i)) / dq);
      dqdt_num[7 * i + 3 + k] = (double)(quad(0.5) * (sp.V(k, i) - sm.V(k, i)) / dq);
    }
    dqdt_num[7 * i + 6] = 0.0;
  }
  return 0;
}

// Numerical d tt / d elements (test/test_transit_timing.jl:31-66): elements
// are perturbed by +-dq0 (absolute), initial conditions are recomputed with
// init_nbody and the grad = false transit integration is repeated in quad.
// H may be NULL (fully nested).  Output layout matches dtdelements.
static int fd_dtdelements_nr(int nr, int n, double t0, const double* elements, const double* H, double h,
                             double tmax, int ti, int ntt, double dq0_d, int nthreads, double* dtde_num) {
  quad dq0 = quad(dq0_d);
  std::vector<quad> Hq((size_t)n * n), el0((size_t)n * 7);
  if (H) for (int q = 0; q < n * n; q++) Hq[q] = quad(H[q]);
  else hierarchy_nested<quad>(n, Hq.data());
  for (int q = 0; q < n * 7; q++) el0[q] = quad(elements[q]);
  size_t n4 = (size_t)nr * n * ntt * 7 * n;
  for (size_t q = 0; q < n4; q++) dtde_num[q] = 0.0;
  auto run = [&](int jq, int ivary, quad delta, TransitTiming<quad>& T) {
    std::vector<quad> el(el0);
    el[jq + n * ivary] = el[jq + n * ivary] + delta;
    State<quad> s;
    s.alloc(n);
    init_nbody<quad>(n, quad(t0), el.data(), Hq.data(), s.x.data(), s.v.data(), s.jac_init.data());
    for (int q = 0; q < n; q++) s.m[q] = el[q];
    s.t = quad(t0);
    T.alloc(n, ntt, ti, nr);
    T.s_prior.alloc(n);
    intr_transits(s, T, quad(h), quad(tmax), false);
  };
  std::atomic<int> next(0);
  auto work = [&]() {
    while (true) {
      int task = next.fetch_add(1);
      if (task >= 7 * n) break;
      int jq = task / 7, iq = task % 7;  // iq 0..5: elements 2..7; 6: mass
      int ivary = (iq == 6) ? 0 : iq + 1;
      TransitTiming<quad> tp, tm;
      run(jq, ivary, dq0, tp);
      run(jq, ivary, -dq0, tm);
      for (int i : tm.occs)
        for (int64_t k = 0; k < tm.count[i] && k < ntt && k < tp.count[i]; k++)
          for (int r = 0; r < nr; r++)
            dtde_num[tm.idx4(i, (int)k, iq, jq, r)] =
                (double)((tp.tt[tp.idx2(i, (int)k, r)] - tm.tt[tm.idx2(i, (int)k, r)]) / (quad(2) * dq0));
    }
  };
  std::vector<std::thread> th;
  for (int q = 1; q < nthreads; q++) th.emplace_back(work);
  work();
  for (auto& q : th) q.join();
  return 0;
}

int oracle_fd_dtdelements(int n, double t0, const double* elements, const double* H, double h, double tmax,
                          int ti, int ntt, double dq0_d, int nthreads, double* dtde_num) {
  return fd_dtdelements_nr(1, n, t0, elements, H, h, tmax, ti, ntt, dq0_d, nthreads, dtde_num);
}

// Numerical d(t, v_sky, b_sky^2) / d elements for TransitParameters
// (test/test_transit_parameters.jl:47-82); layout of dtbvdelements.
int oracle_fd_dtbvdelements(int n, double t0, const double* elements, const double* H, double h, double tmax,
                            int ti, int ntt, double dq0_d, int nthreads, double* dtde_num) {
  return fd_dtdelements_nr(3, n, t0, elements, H, h, tmax, ti, ntt, dq0_d, nthreads, dtde_num);
}

// Numerical jac_init (test/test_init_nbody.jl): two-sided differences in quad
// with per-element absolute steps dq[7] (mass step for the central body:
// dq_star_mass).
int oracle_fd_init_nbody(int n, double t0, const double* elements, const double* H, const double* dq,
                         double dq_star_mass, double* jac_num) {
  int M = 7 * n;
  std::vector<quad> Hq((size_t)n * n), el0((size_t)n * 7);
  if (H) for (int q = 0; q < n * n; q++) Hq[q] = quad(H[q]);
  else hierarchy_nested<quad>(n, Hq.data());
  for (int q = 0; q < n * 7; q++) el0[q] = quad(elements[q]);
  for (size_t q = 0; q < (size_t)M * M; q++) jac_num[q] = 0.0;
  std::vector<quad> xp(3 * n), vp(3 * n), xm(3 * n), vm(3 * n), jtmp((size_t)M * M);
  for (int j = 0; j < n; j++)
    for (int k = 0; k < 7; k++) {
      int ivary = (k == 6) ? 0 : k + 1;  // jac_init column order: P,t0,ecos,esin,I,Omega,m
      quad d = quad((j == 0 && k == 6) ? dq_star_mass : dq[k]);
      std::vector<quad> el(el0);
      el[j + n * ivary] = el0[j + n * ivary] + d;
      init_nbody<quad>(n, quad(t0), el.data(), Hq.data(), xp.data(), vp.data(), jtmp.data());
      el[j + n * ivary] = el0[j + n * ivary] - d;
      init_nbody<quad>(n, quad(t0), el.data(), Hq.data(), xm.data(), vm.data(), jtmp.data());
      int col = 7 * j + k;
      for (int i = 0; i < n; i++)
        for (int q = 0; q < 3; q++) {
          jac_num[(7 * i + q) + (size_t)M * col] = (double)((xp[q + 3 * i] - xm[q + 3 * i]) / (quad(2) * d));
          jac_num[(7 * i + 3 + q) + (size_t)M * col] = (double)((vp[q + 3 * i] - vm[q + 3 * i]) / (quad(2) * d));
        }
      if (k == 6) jac_num[(7 * j + 6) + (size_t)M * col] = 1.0;
    }
  return 0;
}

// kepler_init with its 7x7 Jacobian (kepler_init.jl:66-210) for one
// Keplerian, in double (quad = 0) or in quad precision (quad = 1, outputs
// rounded to double).  el = (P, t0, e cos w, e sin w, I, Omega).
int oracle_kepler_init(double time, double mass, const double* el, int quad_prec, double* x, double* v,
                       double* jac) {
  if (quad_prec) {
    quad e[6], xq[3], vq[3], jq[49];
    for (int q = 0; q < 6; q++) e[q] = quad(el[q]);
    kepler_init<quad>(quad(time), quad(mass), e, xq, vq, jq);
    for (int q = 0; q < 3; q++) { x[q] = (double)xq[q]; v[q] = (double)vq[q]; }
    for (int q = 0; q < 49; q++) jac[q] = (double)jq[q];
  } else {
    kepler_init<double>(time, mass, el, x, v, jac);
  }
  return 0;
}

// Numerical d(x, v, m) / d(elements, m) of kepler_init
// (test/test_kepler_init.jl:34-76): two-sided differences in quad precision
// with absolute steps dq[7] (P, t0, e cos w, e sin w, I, Omega, mass).
int oracle_fd_kepler_init(double time, double mass, const double* el, const double* dq, double* jac_num) {
  for (int q = 0; q < 49; q++) jac_num[q] = 0.0;
  for (int j = 0; j < 7; j++) {
    quad ep[6], em[6], mp = quad(mass), mm = quad(mass), xp[3], vp[3], xm[3], vm[3], jt[49];
    for (int q = 0; q < 6; q++) ep[q] = em[q] = quad(el[q]);
    const quad d = quad(dq[j]);
    if (j < 6) { ep[j] = ep[j] + d; em[j] = em[j] - d; }
    else { mp = mp + d; mm = mm - d; }
    kepler_init<quad>(quad(time), mp, ep, xp, vp, jt);
    kepler_init<quad>(quad(time), mm, em, xm, vm, jt);
    for (int k = 0; k < 3; k++) {
      jac_num[k + 7 * j] = (double)(quad(0.5) * (xp[k] - xm[k]) / d);
      jac_num[3 + k + 7 * j] = (double)(quad(0.5) * (vp[k] - vm[k]) / d);
    }
  }
  jac_num[6 + 7 * 6] = 1.0;
  return 0;
}

}  // extern "C"
