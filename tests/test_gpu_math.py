"""Device math of the Kepler solver against CUDA's own functions and the
reference's series recurrences.

* sincos_kepler (Taylor series of sin and cos, |x| <= pi/4) vs CUDA's sin/cos;
* gh_functions' degree-10 polynomials vs the term-by-term series of
  src/utils.jl:137-396 (restated in the probe), over gamma in [0, 0.5) and
  both signs of beta.
The probe is compiled with nvcc for sm_103a at test time and reports the
worst errors.
"""
import os
import subprocess
import tempfile

import pytest

import nbg

from conftest import PKG_DIR, has_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not has_gpu(), reason="needs a CUDA GPU")]

PROBE = r'''
#include <cstdio>
#include <cmath>
#include "nbg_kepler.cuh"
using namespace nbg;
__device__ double ulp_err(double a, double b) {
  if (a == b) return 0.0;
  double u = fabs(b) * 2.220446049250313e-16;
  return fabs(a - b) / (u > 0 ? u : 4.9e-324);
}
// reference series, term by term (src/utils.jl:137-396)
__device__ double series(int which, double x2) {
  double term, h, h1, h2, f = 4.0;
  if (which == 0) { term = 1; h = 1; }
  else if (which == 1) { term = 1; h = 1; }
  else if (which == 2) { term = 1; h = 1; }
  else if (which == 3) { term = 1.0 / 30; h = 0.1; f = 4.0; }
  else if (which == 4) { term = 1.0 / 60; h = term; }
  else { term = 1.0 / 360; h = 1.0 / 40; f = 16.0; }
  h1 = 2 * h; h2 = 2 * h;
  for (int n = 1; n <= 100; n++) {
    h2 = h1; h1 = h;
    if (which == 0) { term = term * (x2 / ((2 * n + 3) * (2 * n + 2))); h = h + term; }
    else if (which == 1) { term = term * (x2 * (n + 1)); term = term / ((2 * n + 4) * (2 * n + 3) * n); h = h + term; }
    else if (which == 2) { term = term * x2; term = term / ((4 * n + 6) * n); h = h + term; }
    else if (which == 3) { term = term * x2; term = term / ((2 * n + 4) * (2 * n + 5)); f = f * 4; h = h + term * (f - 1); }
    else if (which == 4) { term = term * (x2 * (n + 1)); term = term / ((2 * n + 5) * (2 * n + 4) * n); h = h + term; }
    else { term = term * x2; term = term / ((2 * n + 5) * (2 * n + 6)); f = f * 4; h = h + term * (f - 3 * n - 7); }
    if (h == h1 || h == h2) break;
  }
  return h;
}
__global__ void k(int n, double* out) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  double x = -0.78539816339744831 + 1.5707963267948966 * ((double)t + 0.5) / n;
  double s, c;
  sincos_kepler(x, &s, &c);
  out[4 * t + 0] = ulp_err(s, sin(x));
  out[4 * t + 1] = ulp_err(c, cos(x));
  double gamma = 0.5 * ((double)t + 0.5) / n;
  double worst = 0.0;
  for (int sb = -1; sb <= 1; sb += 2) {
    double x2 = -sb * gamma * gamma;
    for (int w = 0; w < 6; w++) {
      double p = gh_horner(kGHCoef[w], x2), r = series(w, x2);
      worst = fmax(worst, fabs(p - r) / fabs(r));
    }
  }
  out[4 * t + 2] = worst;
  out[4 * t + 3] = 0.0;
}
int main() {
  const int n = 1 << 20;
  double* d; cudaMalloc(&d, sizeof(double) * 4 * n);
  k<<<n / 256, 256>>>(n, d);
  double* h = new double[4 * n];
  if (cudaMemcpy(h, d, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost) != cudaSuccess) return 1;
  double ms = 0, mc = 0, mg = 0;
  for (int i = 0; i < n; i++) { ms = fmax(ms, h[4*i]); mc = fmax(mc, h[4*i+1]); mg = fmax(mg, h[4*i+2]); }
  printf("%.6g %.6g %.6g\n", ms, mc, mg);
  return 0;
}
'''


def test_kepler_math_against_cuda_and_series():
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "m.cu")
        exe = os.path.join(tmp, "m")
        with open(src, "w") as f:
            f.write(PROBE)
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false",
                        "-I", os.path.join(PKG_DIR, "csrc"), "-o", exe, src], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    sin_ulp, cos_ulp, series_rel = (float(q) for q in out)
    assert sin_ulp <= 2.0, sin_ulp
    assert cos_ulp <= 2.0, cos_ulp
    assert series_rel <= 1e-15, series_rel  # a few ulp: polynomial vs term-by-term rounding


def test_fp64_tensor_core_probe_runs_and_checks_its_fragments():
    """The DMMA probe checks one exact m8n8k4 f64 product against the documented fragment layout (it
    fails with NBG_EUNSUPPORTED otherwise) and reports positive rates."""
    ctx = nbg.Context(0)
    try:
        mma, share0 = ctx.fp64_mma_peak_tflops(False)
        mixed, share = ctx.fp64_mma_peak_tflops(True)
    finally:
        ctx.close()
    assert mma > 0 and mixed > 0
    assert share0 == 0.0 and 0.0 < share < 1.0


def test_fp64_warp_issue_probe():
    """One warp issues FP64 instructions no faster than its 8 independent chains allow; more warps of
    one block share the SM's FP64 pipe (a warp's interval grows once the pipe is full)."""
    ctx = nbg.Context(0)
    try:
        one = ctx.fp64_warp_issue_cycles(1, 8)
        many = ctx.fp64_warp_issue_cycles(8, 8)
        with pytest.raises(nbg.NbgError):
            ctx.fp64_warp_issue_cycles(33, 8)
    finally:
        ctx.close()
    assert one > 1.0 and many >= one
