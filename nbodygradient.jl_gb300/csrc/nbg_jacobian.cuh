// nbg_jacobian.cuh -- the Jacobian consumer: one GPU lane owns one column of
// jac_step (and of jac_error) of one system and applies the operator stream
// the orbit producer recorded, with the reference's compensated summation.
//
// Every update of ahl21! on jac_step (src/integrator/ahl21/ahl21.jl:5-95) has
// the form J <- J + A J followed by comp_sum_matrix!(J, J_err, A J)
// (src/utils.jl:36-46); columns of J never mix, so a column is a complete
// unit of work.  The consumer keeps the 6N non-mass rows of its column in
// shared memory ([row][lane], conflict-free); the mass rows of J are unit
// rows that no operator touches (the library checks this on entry).
//
// The pair update uses the structure of jac_ij (ahl21.jl:734-750): rows of
// body i are mj*K, -mj*K on (x,v)_i, (x,v)_j and rows of body j are -mi*K,
// mi*K, so jac_ij * [J_i; J_j] = [mj u; -mi u] with u = K (J_i - J_j), plus
// the two mass columns (fused into the scaling FMA).  That is 54 FP64
// operations per column instead of 144 for the dense 12x12 block; the
// product is rounded differently from a dense BLAS product, which the
// reference's BLAS leaves unspecified anyway.
#pragma once
#include "nbg_operators.cuh"

namespace nbg {

// Kahan fold with a zero addend (comp_sum_matrix! on a zero entry).
__device__ __forceinline__ void fold(double& s, double& e) {
  double t = s + e;
  e = (s - t) + e;
  s = t;
}

// Whether fold(s, e) changes s or e.  It leaves both bitwise unchanged exactly
// when s + e rounds to s (same bits), s is finite (else s - s is NaN) and e is
// not -0 ((s - s) + -0 is +0).  After a compensated add the pair is normally
// in that state: the add leaves in e the rounding error of s, which s + e
// rounds away.  The test costs one FP64 add against the fold's three; the
// rest is integer work.
__device__ __forceinline__ bool fold_changes(double s, double e) {
  const unsigned long long sb = __double_as_longlong(s), eb = __double_as_longlong(e);
  const unsigned long long tb = __double_as_longlong(s + e);
  return tb != sb || ((sb >> 52) & 0x7ffull) == 0x7ffull || eb == 0x8000000000000000ull;
}

// fold() on rows 6 b + R0 .. 6 b + R0 + NR - 1 of every body b.  The warp
// first tests its lanes' rows and runs the folds only if one of them would
// change a row, so the result is the folds' result bitwise (each lane skips
// only when no lane of its group, itself included, would change).
template <int N, int BS, int R0, int NR>
__device__ __forceinline__ void fold_rows(double* J, double* E) {
  bool change = false;
#pragma unroll 1
  for (int b = 0; b < N; b++)
#pragma unroll
    for (int r = R0; r < R0 + NR; r++) change |= fold_changes(J[(6 * b + r) * BS], E[(6 * b + r) * BS]);
  if (!__any_sync(__activemask(), change)) return;
#pragma unroll 1
  for (int b = 0; b < N; b++)
#pragma unroll
    for (int r = R0; r < R0 + NR; r++) fold(J[(6 * b + r) * BS], E[(6 * b + r) * BS]);
}

// P[vr] = (A J)[velocity row vr] for the compact operator at record offset
// roff: one FMA chain over the position rows of J, with the exact no-op
// terms (zero operator entries; mass rows of J, which are unit rows) reduced
// to the single mass entry of this column, which starts the chain.  Starting
// from it costs no FP64 instruction, where adding it inside the chain would
// cost a warp-wide issue slot for the few mass-column lanes; the summation
// order of the reference's BLAS product is unspecified, so any order is as
// faithful as another.
template <int N, int BS>
__device__ __forceinline__ void op_product(const double* J, const Rec& rec, int roff, int c, double* P) {
  const int cm = (c % 7 == 6) ? c / 7 : -1;  // body whose mass this column is
#pragma unroll 1
  for (int vr = 0; vr < 3 * N; vr++) {
    const int rb = roff + vr * (4 * N);
    double acc = (cm >= 0) ? rec.get(rb + 4 * cm + 3) : 0.0;
#pragma unroll
    for (int d = 0; d < N; d++)
#pragma unroll
      for (int p = 0; p < 3; p++) acc = fma(rec.get(rb + 4 * d + p), J[(6 * d + p) * BS], acc);
    P[vr] = acc;
  }
}

// One Kepler pair block update (ahl21.jl:31-42 / :64-75) on this column.
// The pair's record is loaded first, all of it, so that its loads go out
// together ahead of this pair's stores to J and E (which a load through the
// record pointer could alias): one trip to memory per pair.  A system alone
// on the GPU waits out every such trip, at ten bodies 90 of them per step.
template <int N, int BS>
__device__ __forceinline__ void pair_apply(double* J, double* E, int c, int i, int j, const Rec& rec, int roff) {
  double K[36];
#pragma unroll
  for (int q = 0; q < 36; q++) K[q] = rec.get(roff + q);
  const double mi = rec.get(roff + PREC_MI), mj = rec.get(roff + PREC_MJ);
  // the mass column of body i or j (at most one of them is this column)
  // takes the pair's mass entries; every other column adds an exact zero
  const int mc = (c == 7 * i + 6) ? PREC_MC6 : (c == 7 * j + 6) ? PREC_MC13 : -1;
  double C[12];
#pragma unroll
  for (int q = 0; q < 12; q++) C[q] = (mc >= 0) ? rec.get(roff + mc + q) : 0.0;
  double D[6];
#pragma unroll
  for (int l = 0; l < 6; l++) D[l] = J[(6 * i + l) * BS] - J[(6 * j + l) * BS];
#pragma unroll
  for (int r = 0; r < 6; r++) {
    double u = K[r * 6] * D[0];
#pragma unroll
    for (int l = 1; l < 6; l++) u = fma(K[r * 6 + l], D[l], u);
    kahan(J[(6 * i + r) * BS], E[(6 * i + r) * BS], fma(mj, u, C[r]));
    kahan(J[(6 * j + r) * BS], E[(6 * j + r) * BS], fma(-mi, u, C[6 + r]));
  }
}

// J <- J + A J on all non-mass rows: velocity rows take the product P,
// position rows a zero addend.  Every row is summed on its own, so the
// position rows' folds may run first.
template <int N, int BS>
__device__ __forceinline__ void add_velocity_rows(double* J, double* E, const double* P) {
  fold_rows<N, BS, 0, 3>(J, E);
#pragma unroll 1
  for (int b = 0; b < N; b++)
#pragma unroll
    for (int k = 0; k < 3; k++) kahan(J[(6 * b + 3 + k) * BS], E[(6 * b + 3 + k) * BS], P[3 * b + k]);
}
template <int N, int BS>
__device__ __forceinline__ void fold_all(double* J, double* E) {
  fold_rows<N, BS, 0, 6>(J, E);
}

// drift_grad! on jac_step (ahl21.jl:318-331): x rows += h * v rows.
template <int N, int BS>
__device__ __forceinline__ void drift_rows(double* J, double* E, double h) {
#pragma unroll 1
  for (int b = 0; b < N; b++)
#pragma unroll
    for (int k = 0; k < 3; k++) kahan(J[(6 * b + k) * BS], E[(6 * b + k) * BS], h * J[(6 * b + 3 + k) * BS]);
}

// One recorded step on this column (ahl21.jl:5-95, the jac_step updates).
template <int N, int BS>
__device__ void apply_step(double* J, double* E, int c, double h, uint64_t kick, const Rec& rec) {
  const double h2 = 0.5 * h;
  double P[3 * N];
  int roff = 0;
  if (kick) {
    op_product<N, BS>(J, rec, roff, c, P);  // jac_kick * jac_step before the drift
    roff += op_size(N);
  }
  drift_rows<N, BS>(J, E, h2);
  if (kick) add_velocity_rows<N, BS>(J, E, P);
  else fold_all<N, BS>(J, E);
#pragma unroll 1
  for (int i = 0; i < N - 1; i++)
#pragma unroll 1
    for (int j = i + 1; j < N; j++) {
      if ((kick >> pair_bit(i, j, N)) & 1) continue;
      pair_apply<N, BS>(J, E, c, i, j, rec, roff);
      roff += PREC;
    }
  op_product<N, BS>(J, rec, roff, c, P);
  roff += op_size(N);
  add_velocity_rows<N, BS>(J, E, P);
#pragma unroll 1
  for (int i = N - 2; i >= 0; i--)
#pragma unroll 1
    for (int j = N - 1; j > i; j--) {
      if ((kick >> pair_bit(i, j, N)) & 1) continue;
      pair_apply<N, BS>(J, E, c, i, j, rec, roff);
      roff += PREC;
    }
  drift_rows<N, BS>(J, E, h2);
  if (kick) {
    op_product<N, BS>(J, rec, roff, c, P);
    add_velocity_rows<N, BS>(J, E, P);
  } else {
    fold_all<N, BS>(J, E);
  }
}

}  // namespace nbg
