// nbg_oracle_transit.hpp -- TEST INFRASTRUCTURE ONLY (parity oracle; see
// nbg_oracle.hpp).  Restates src/transits/Transits.jl:14-110,140-180 and
// src/transits/timing.jl:3-193 for TransitTiming and TransitParameters
// outputs, plus the plain drivers of src/integrator/Integrator.jl:159-247.
#pragma once

namespace nbgo {

// TransitTiming (Transits.jl:14-56, nr = 1) and TransitParameters
// (Transits.jl:68-110, nr = 3: rows t, v_sky, b_sky^2).  Arrays are Julia
// column-major with the row index first:
//   tt[r + nr (j + n c)], dtdq0[r + nr (j + n (c + ntt (k + 7 p)))],
//   dtdelements likewise, dtdq[r + nr (k + 7 p)]; nr = 1 is TransitTiming's
//   tt[j + n c], dtdq0[j + n (c + ntt (k + 7 p))].
template <class T> struct TransitTiming {
  int n = 0, ntt = 0, ti = 0;  // ti is 0-based
  int nr = 1;
  std::vector<T> tt, dtdq0, dtdelements, dtdq, gsave;
  std::vector<int64_t> count;
  std::vector<int> occs;
  State<T> s_prior, s_transit;
  void alloc(int n_, int ntt_, int ti_, int nr_ = 1) {
    n = n_; ntt = ntt_; ti = ti_; nr = nr_;
    tt.assign((size_t)nr * n * ntt, T(0));
    dtdq0.assign((size_t)nr * n * ntt * 7 * n, T(0));
    dtdelements.assign((size_t)nr * n * ntt * 7 * n, T(0));
    dtdq.assign((size_t)nr * 7 * n, T(0));
    gsave.assign(n, T(0));
    count.assign(n, 0);
    occs.clear();
    for (int i = 0; i < n; i++) if (i != ti) occs.push_back(i);  // setdiff(1:n, ti)
  }
  size_t idx4(int j, int c, int k, int p, int r = 0) const {
    return r + (size_t)nr * (j + (size_t)n * (c + (size_t)ntt * (k + 7 * (size_t)p)));
  }
  size_t idx2(int j, int c, int r = 0) const { return r + (size_t)nr * (j + (size_t)n * c); }
};

// g! (timing.jl:141-144): sky-plane relative position dotted with velocity
template <class T> T gsky(State<T>& s, int i, int j) {
  return (s.X(0, j) - s.X(0, i)) * (s.V(0, j) - s.V(0, i)) + (s.X(1, j) - s.X(1, i)) * (s.V(1, j) - s.V(1, i));
}
// gd! (timing.jl:147-150)
template <class T> T gdot(State<T>& s, int i, int j) {
  const std::vector<T>& q = s.dqdt;
  return ((s.X(0, j) - s.X(0, i)) * (q[7 * j + 3] - q[7 * i + 3]) +
          (s.X(1, j) - s.X(1, i)) * (q[7 * j + 4] - q[7 * i + 4]) +
          (s.V(0, j) - s.V(0, i)) * (q[7 * j + 0] - q[7 * i + 0]) +
          (s.V(1, j) - s.V(1, i)) * (q[7 * j + 1] - q[7 * i + 1]));
}
// dtbvdq! row 1 (timing.jl:155-171): dtdq[k + 7 p]
template <class T> void dtbvdq1(State<T>& s, int i, int j, std::vector<T>& dtdq) {
  T gd = gdot(s, i, j);
  std::fill(dtdq.begin(), dtdq.end(), T(0));
  int indj = 7 * j, indi = 7 * i;
  for (int p = 0; p < s.n; p++) {
    int indp = 7 * p;
    for (int k = 0; k < 7; k++) {
      int c = indp + k;
      dtdq[k + 7 * p] = -((s.J(indj, c) - s.J(indi, c)) * (s.V(0, j) - s.V(0, i)) +
                          (s.J(indj + 1, c) - s.J(indi + 1, c)) * (s.V(1, j) - s.V(1, i)) +
                          (s.J(indj + 3, c) - s.J(indi + 3, c)) * (s.X(0, j) - s.X(0, i)) +
                          (s.J(indj + 4, c) - s.J(indi + 4, c)) * (s.X(1, j) - s.X(1, i))) /
                        gd;
    }
  }
}

// calc_bsky2, calc_vsky (timing.jl:152-153)
template <class T> T calc_bsky2(State<T>& s, int i, int j) {
  return (s.X(0, j) - s.X(0, i)) * (s.X(0, j) - s.X(0, i)) + (s.X(1, j) - s.X(1, i)) * (s.X(1, j) - s.X(1, i));
}
template <class T> T calc_vsky(State<T>& s, int i, int j) {
  return Mth<T>::sqrt((s.V(0, j) - s.V(0, i)) * (s.V(0, j) - s.V(0, i)) +
                      (s.V(1, j) - s.V(1, i)) * (s.V(1, j) - s.V(1, i)));
}

// dtbvdq! with three rows (timing.jl:155-193): dtbvdq[r + 3 (k + 7 p)];
// returns v_sky and b_sky^2.
template <class T> void dtbvdq3(State<T>& s, int i, int j, std::vector<T>& dq, T* vsky_out, T* bsky2_out) {
  T gd = gdot(s, i, j);
  std::fill(dq.begin(), dq.end(), T(0));
  int indj = 7 * j, indi = 7 * i;
  for (int p = 0; p < s.n; p++) {
    int indp = 7 * p;
    for (int k = 0; k < 7; k++) {
      int c = indp + k;
      dq[0 + 3 * (k + 7 * p)] = -((s.J(indj, c) - s.J(indi, c)) * (s.V(0, j) - s.V(0, i)) +
                                  (s.J(indj + 1, c) - s.J(indi + 1, c)) * (s.V(1, j) - s.V(1, i)) +
                                  (s.J(indj + 3, c) - s.J(indi + 3, c)) * (s.X(0, j) - s.X(0, i)) +
                                  (s.J(indj + 4, c) - s.J(indi + 4, c)) * (s.X(1, j) - s.X(1, i))) /
                                gd;
    }
  }
  T vsky = calc_vsky(s, i, j);
  T bsky2 = calc_bsky2(s, i, j);
  const std::vector<T>& q = s.dqdt;
  T dvdt = ((s.V(0, j) - s.V(0, i)) * (q[7 * j + 3] - q[7 * i + 3]) +
            (s.V(1, j) - s.V(1, i)) * (q[7 * j + 4] - q[7 * i + 4])) /
           vsky;
  for (int p = 0; p < s.n; p++) {
    int indp = 7 * p;
    for (int k = 0; k < 7; k++) {
      int c = indp + k;
      dq[1 + 3 * (k + 7 * p)] = ((s.J(indj + 3, c) - s.J(indi + 3, c)) * (s.V(0, j) - s.V(0, i)) +
                                 (s.J(indj + 4, c) - s.J(indi + 4, c)) * (s.V(1, j) - s.V(1, i))) /
                                    vsky +
                                dvdt * dq[0 + 3 * (k + 7 * p)];
      dq[2 + 3 * (k + 7 * p)] = T(2) * ((s.J(indj, c) - s.J(indi, c)) * (s.X(0, j) - s.X(0, i)) +
                                        (s.J(indj + 1, c) - s.J(indi + 1, c)) * (s.X(1, j) - s.X(1, i)));
    }
  }
  *vsky_out = vsky;
  *bsky2_out = bsky2;
}

// Number of transit Newton searches that stopped at ITMAX (diagnostics only;
// the reference continues silently).
inline long long& newton_itmax_hits() {
  static thread_local long long n = 0;
  return n;
}

// findtransit! (timing.jl:31-109), TransitTiming branch
template <class T>
void findtransit(int i, int j, T dt0, State<T>& s, Derivs<T>& d, TransitTiming<T>& tt, bool grad) {
  std::fill(s.dqdt.begin(), s.dqdt.end(), T(0));
  T dt = T(1);
  int iter = 0;
  T stmp = T(0);
  T tt1 = dt0 + T(1), tt2 = dt0 + T(2);
  const int ITMAX = 20;
  while (true) {
    tt2 = tt1;
    tt1 = dt0;
    set_state(s, tt.s_prior);
    d.zero();
    ahl21(s, d, dt0);
    T gs = gsky(s, i, j);
    T gd = gdot(s, i, j);
    dt = -gs / gd;
    comp_sum(dt0, stmp, dt);
    iter += 1;
    if (iter >= ITMAX || dt0 == tt1 || dt0 == tt2) break;
  }
  if (iter >= ITMAX) newton_itmax_hits() += 1;
  if (grad) {
    set_state(s, tt.s_prior);
    d.zero();
    ahl21(s, d, dt0);
  }
  int64_t c = tt.count[j] - 1;
  if (tt.nr == 3) {
    // TransitParameters branch (timing.jl:82-98): t, v_sky, b_sky^2; without
    // grad v_sky and b_sky^2 come from the last Newton iteration's state
    tt.tt[tt.idx2(j, (int)c, 0)] = s.t + dt0;
    if (grad) {
      T vsky, bsky2;
      dtbvdq3(s, i, j, tt.dtdq, &vsky, &bsky2);
      tt.tt[tt.idx2(j, (int)c, 1)] = vsky;
      tt.tt[tt.idx2(j, (int)c, 2)] = bsky2;
      for (int r = 0; r < 3; r++)
        for (int k = 0; k < 7; k++)
          for (int p = 0; p < s.n; p++) tt.dtdq0[tt.idx4(j, (int)c, k, p, r)] = tt.dtdq[r + 3 * (k + 7 * p)];
      return;
    }
    tt.tt[tt.idx2(j, (int)c, 1)] = calc_vsky(s, i, j);
    tt.tt[tt.idx2(j, (int)c, 2)] = calc_bsky2(s, i, j);
    return;
  }
  tt.tt[j + (size_t)tt.n * c] = s.t + dt0;
  if (grad) {
    dtbvdq1(s, i, j, tt.dtdq);
    for (int k = 0; k < 7; k++)
      for (int p = 0; p < s.n; p++) tt.dtdq0[tt.idx4(j, (int)c, k, p)] = tt.dtdq[k + 7 * p];
  }
}

// detect_transits! (timing.jl:3-28)
// ih is the integrator's (unsigned) step intr.h, as read at timing.jl:20.
template <class T> void detect_transits(State<T>& s, Derivs<T>& d, TransitTiming<T>& tt, T ih, bool grad) {
  const T rstar = T(1e12);
  set_state(tt.s_prior, s);
  for (int i : tt.occs) {
    T gi = gsky(s, i, tt.ti);
    T ri = Mth<T>::sqrt(s.X(0, i) * s.X(0, i) + s.X(1, i) * s.X(1, i) + s.X(2, i) * s.X(2, i));
    if (gi > T(0) && tt.gsave[i] < T(0) && -s.X(2, i) > T(0.25) * ri && ri < rstar) {
      tt.count[i] += 1;
      if (tt.count[i] <= tt.ntt) {
        T dt0 = -gi * ih / (gi - tt.gsave[i]);
        set_state(s, tt.s_prior);
        findtransit(tt.ti, i, dt0, s, d, tt, grad);
      }
    }
    tt.gsave[i] = gi;
    set_state(s, tt.s_prior);
  }
}

// calc_dtdelements! (timing.jl:112-123; TransitParameters: :126-138, per row)
template <class T> void calc_dtdelements(State<T>& s, TransitTiming<T>& tt) {
  int n = s.n, M = 7 * n;
  for (int r = 0; r < tt.nr; r++)
    for (int i = 0; i < n; i++)
      for (int64_t j = 0; j < tt.count[i]; j++) {
        if (j + 1 > tt.ntt) continue;
        for (int k = 0; k < n; k++)
          for (int l = 0; l < 7; l++) {
            T acc = T(0);
            for (int p = 0; p < n; p++)
              for (int q = 0; q < 7; q++)
                acc = acc + tt.dtdq0[tt.idx4(i, (int)j, q, p, r)] * s.jac_init[(7 * p + q) + (size_t)M * (7 * k + l)];
            tt.dtdelements[tt.idx4(i, (int)j, l, k, r)] = acc;
          }
      }
}

// check_step (Integrator.jl:249-259)
template <class T> T check_step(T t0, T tmax) {
  if (Mth<T>::fabs(tmax) > Mth<T>::fabs(t0)) return jsign(tmax);
  if (jsign(tmax) != jsign(t0)) return jsign(tmax);
  return T(-1) * jsign(tmax);
}

// Julia round(Int64, x): nearest, ties to even.
template <class T> int64_t jround(T x) { return (int64_t)std::nearbyint((double)x); }

// (intr::Integrator)(s, tt, d; grad) (Transits.jl:140-170).  The integrator's
// own t0 is not read on this path; the start time is s.t.
template <class T> void intr_transits(State<T>& s, TransitTiming<T>& tt, T ih, T itmax, bool grad) {
  Derivs<T> d;
  d.alloc(s.n);
  T t0 = s.t;
  int64_t nsteps = jround(itmax / ih);
  if (nsteps < 0) nsteps = -nsteps;
  T h = ih * check_step(t0, itmax + t0);
  for (int i : tt.occs) tt.gsave[i] = gsky(s, i, tt.ti);
  int64_t istep = 0;
  for (int64_t q = 0; q < nsteps; q++) {
    if (grad) ahl21(s, d, h);
    else ahl21_ng(s, h);
    istep += 1;
    s.t = t0 + T(istep) * h;
    detect_transits(s, d, tt, ih, grad);
  }
  if (grad) calc_dtdelements(s, tt);
}

// (intr::Integrator)(s, time; grad) (Integrator.jl:159-197)
template <class T> void intr_time(State<T>& s, T ih, T time, bool grad) {
  T t0 = s.t;
  int64_t nsteps = jround((time - t0) / ih);
  if (nsteps < 0) nsteps = -nsteps;
  T h = ih * check_step(t0, time);
  T tmax = t0 + (h * T(nsteps));
  Derivs<T> d;
  if (grad) d.alloc(s.n);
  for (int64_t q = 0; q < nsteps; q++) {
    if (grad) ahl21(s, d, h);
    else ahl21_ng(s, h);
  }
  if (tmax != time) {
    T hf = time - tmax;
    if (grad) ahl21(s, d, hf);
    else ahl21_ng(s, hf);
  }
  s.t = time;
}

// (intr::Integrator)(s, N; grad) (Integrator.jl:211-234)
template <class T> void intr_nsteps(State<T>& s, T& ih, int64_t N, bool grad) {
  T s2 = T(0);
  Derivs<T> d;
  if (grad) d.alloc(s.n);
  if (N < 0) { ih = -ih; N = -N; }
  T h = ih;
  for (int64_t q = 0; q < N; q++) {
    if (grad) ahl21(s, d, h);
    else ahl21_ng(s, h);
    comp_sum(s.t, s2, ih);
  }
  if (ih < T(0)) ih = -ih;
}

}  // namespace nbgo
