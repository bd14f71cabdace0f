"""The consumer's zero-addend Kahan folds skip the work only when it is the identity.

fold_rows (csrc/nbg_jacobian.cuh) tests s + e for every row of the warp's lanes and runs the folds of
comp_sum_matrix! (src/utils.jl:36-46, a zero entry of the added matrix) only if one lane would change.
The probe runs it, and add_velocity_rows, on pairs (s, e) made to hit every branch: compensated pairs
(the usual state, where the warp skips), off-by-an-ulp errors, rounding ties, powers of two, signed
zeros, subnormals, infinities and NaN, whole and partial warps.  numpy restates the plain folds and
Kahan adds, and the device must match them bit for bit (NaN payloads aside).
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import PKG_DIR, has_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not has_gpu(), reason="needs a CUDA GPU")]

N, ROWS, LANES = 3, 18, 32

PROBE = r'''
#include <cstdio>
#include <vector>
#include "nbg_jacobian.cuh"
using namespace nbg;
constexpr int N = 3, R = 6 * N, BS = 32;
// mode 0: fold_all; 1: add_velocity_rows; 2: fold_all on the first act[t] lanes only
__global__ void k(int mode, const int* act, const double* J0, const double* E0, const double* P0,
                  double* Jo, double* Eo) {
  __shared__ double sm[2 * R * BS];
  const int t = blockIdx.x, l = threadIdx.x;
  double* J = sm + l;
  double* E = sm + R * BS + l;
  for (int r = 0; r < R; r++) {
    J[r * BS] = J0[((size_t)t * R + r) * BS + l];
    E[r * BS] = E0[((size_t)t * R + r) * BS + l];
  }
  if (mode == 0 || (mode == 2 && l < act[t])) {
    fold_all<N, BS>(J, E);
  } else if (mode == 1) {
    double P[3 * N];
    for (int q = 0; q < 3 * N; q++) P[q] = P0[((size_t)t * 3 * N + q) * BS + l];
    add_velocity_rows<N, BS>(J, E, P);
  }
  for (int r = 0; r < R; r++) {
    Jo[((size_t)t * R + r) * BS + l] = J[r * BS];
    Eo[((size_t)t * R + r) * BS + l] = E[r * BS];
  }
}
int main(int argc, char** argv) {
  FILE* f = fopen(argv[1], "rb");
  int T = 0;
  if (!f || fread(&T, sizeof(int), 1, f) != 1 || T <= 0 || T > (1 << 16)) return 2;
  const size_t nr = (size_t)T * R * BS, np = (size_t)T * 3 * N * BS;
  std::vector<int> act(T);
  std::vector<double> J(nr), E(nr), P(np), out(2 * nr);
  if (fread(act.data(), sizeof(int), T, f) != (size_t)T || fread(J.data(), 8, nr, f) != nr ||
      fread(E.data(), 8, nr, f) != nr || fread(P.data(), 8, np, f) != np) return 3;
  fclose(f);
  int* dact; double *dJ, *dE, *dP, *dJo, *dEo;
  cudaMalloc(&dact, sizeof(int) * T);
  cudaMalloc(&dJ, 8 * nr); cudaMalloc(&dE, 8 * nr); cudaMalloc(&dP, 8 * np);
  cudaMalloc(&dJo, 8 * nr); cudaMalloc(&dEo, 8 * nr);
  cudaMemcpy(dact, act.data(), sizeof(int) * T, cudaMemcpyHostToDevice);
  cudaMemcpy(dJ, J.data(), 8 * nr, cudaMemcpyHostToDevice);
  cudaMemcpy(dE, E.data(), 8 * nr, cudaMemcpyHostToDevice);
  cudaMemcpy(dP, P.data(), 8 * np, cudaMemcpyHostToDevice);
  FILE* g = fopen(argv[2], "wb");
  for (int mode = 0; mode < 3; mode++) {
    k<<<T, BS>>>(mode, dact, dJ, dE, dP, dJo, dEo);
    if (cudaMemcpy(out.data(), dJo, 8 * nr, cudaMemcpyDeviceToHost) != cudaSuccess) return 4;
    if (cudaMemcpy(out.data() + nr, dEo, 8 * nr, cudaMemcpyDeviceToHost) != cudaSuccess) return 4;
    fwrite(out.data(), 8, 2 * nr, g);
  }
  fclose(g);
  return 0;
}
'''


def _fold(s, e):
    t = s + e
    return t, (s - t) + e


def _kahan(s, e, a):
    e = e + a
    t = s + e
    return t, (s - t) + e


def _specials():
    one = np.float64(1.0)
    ulp1 = np.spacing(one)
    x = np.float64(1.7)
    ux = np.spacing(x)
    return [
        (x, 0.5 * ux), (x + ux, 0.5 * ux),           # ties: to even stays / moves
        (x, 0.75 * ux), (x, -ux), (x, 3.0 * ux),      # errors that s + e does not round away
        (one, -0.25 * ulp1), (one, -0.3 * ulp1),      # power of two: the spacing below is half
        (one, -0.2 * ulp1), (-one, 0.3 * ulp1),
        (np.inf, 0.0), (-np.inf, 1e-300), (np.nan, 0.0), (x, np.nan), (x, np.inf),
        (0.0, -0.0), (-0.0, 0.0), (-0.0, -0.0), (x, -0.0), (0.0, 1e-300),
        (5e-324, 5e-324), (1e-310, -1e-320), (1e300, 1e300), (np.finfo(np.float64).max, 1e292),
    ]


def _make(rng, T):
    J = np.empty((T, ROWS, LANES))
    E = np.empty((T, ROWS, LANES))
    a = rng.standard_normal((T, ROWS, LANES)) * 10.0 ** rng.uniform(-3, 3, (T, ROWS, LANES))
    b = a * rng.standard_normal((T, ROWS, LANES)) * 10.0 ** rng.uniform(-20, -1, (T, ROWS, LANES))
    J[:] = a + b
    E[:] = (a - J) + b  # compensated pairs: the state after a Kahan add
    sp = _specials()
    for t in range(T):
        kind = t % 4
        if kind == 1:  # one odd pair somewhere in the warp
            s, e = sp[rng.integers(len(sp))]
            r, l = rng.integers(ROWS), rng.integers(LANES)
            J[t, r, l], E[t, r, l] = s, e
        elif kind == 2:  # unit and zero entries as in fresh jac_step columns
            J[t] = rng.integers(0, 2, (ROWS, LANES)).astype(np.float64)
            E[t] = 0.0
        elif kind == 3:  # every lane odd in one row
            for l in range(LANES):
                s, e = sp[rng.integers(len(sp))]
                J[t, 3, l], E[t, 3, l] = s, e
    P = rng.standard_normal((T, 3 * N, LANES)) * 1e-3
    act = rng.integers(1, LANES + 1, T).astype(np.int32)
    return act, J, E, P


def _expected(mode, act, J, E, P):
    Jx, Ex = J.copy(), E.copy()
    with np.errstate(all="ignore"):
        if mode in (0, 2):
            Jf, Ef = _fold(J, E)
            if mode == 0:
                return Jf, Ef
            lanes = np.arange(LANES)[None, None, :] < act[:, None, None]
            return np.where(lanes, Jf, J), np.where(lanes, Ef, E)
        for b in range(N):
            for k in range(3):
                Jx[:, 6 * b + k], Ex[:, 6 * b + k] = _fold(J[:, 6 * b + k], E[:, 6 * b + k])
                r = 6 * b + 3 + k
                Jx[:, r], Ex[:, r] = _kahan(J[:, r], E[:, r], P[:, 3 * b + k])
    return Jx, Ex


def _same_bits(a, b):
    both_nan = np.isnan(a) & np.isnan(b)
    return (a.view(np.uint64) == b.view(np.uint64)) | both_nan


def test_skipped_folds_are_bitwise_the_folds():
    rng = np.random.default_rng(20240611)
    T = 2048
    act, J, E, P = _make(rng, T)
    with tempfile.TemporaryDirectory() as tmp:
        src, exe = os.path.join(tmp, "f.cu"), os.path.join(tmp, "f")
        fin, fout = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
        with open(src, "w") as f:
            f.write(PROBE)
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-std=c++17",
                        "-I", os.path.join(PKG_DIR, "csrc"), "-o", exe, src], check=True)
        with open(fin, "wb") as f:
            f.write(np.int32(T).tobytes())
            f.write(act.tobytes())
            for arr in (J, E, P):
                f.write(np.ascontiguousarray(arr, dtype=np.float64).tobytes())
        subprocess.run([exe, fin, fout], check=True)
        out = np.fromfile(fout, dtype=np.float64).reshape(3, 2, T, ROWS, LANES)
    for mode in range(3):
        Jx, Ex = _expected(mode, act, J, E, P)
        okJ, okE = _same_bits(out[mode, 0], Jx), _same_bits(out[mode, 1], Ex)
        assert okJ.all() and okE.all(), (mode, np.argwhere(~(okJ & okE))[:5])
    # the skip and the full path were both taken: compensated warps change nothing, odd ones do
    with np.errstate(all="ignore"):
        Jf, Ef = _fold(J, E)
    changed = ~(_same_bits(Jf, J) & _same_bits(Ef, E))
    warps_changed = changed.any(axis=(1, 2))
    assert warps_changed[0::4].mean() < 0.05
    assert warps_changed[3::4].mean() > 0.5
