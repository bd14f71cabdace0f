// nbg_internal.cuh -- host-side pieces shared by the translation units of
// libnbg_cuda (nbg_cuda.cu: the batched entry points; nbg_server.cu: the
// request server).  Not part of the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/nbg.h"
#include "nbg_layout.cuh"

namespace nbg {

// Offsets of one system into packed arrays in the caller's layout (element
// counts, not bytes).  x/v/xerror/verror share `x`; jac_step/jac_error/
// jac_init share `J`; dtdq0/dtdelements share `dq`.  nr: rows per transit
// of the outputs (1: TransitTiming; 3: TransitParameters' t, v_sky,
// b_sky^2; 0 counts as 1).
struct SysOff {
  long long x, m, J, dqdt, pair, tt, dq, cnt;
  int n, ntt, grad, nr;
};

// Records the calling thread's error message and returns `code`.
int set_error(int code, const char* fmt, ...);

// |round(tmax / h)| with ties to even (Transits.jl:143, round(Int64, tmax/h)).
long long steps_of(double h, double tmax);
// check_step (src/integrator/Integrator.jl:249-259): the sign of the steps.
double check_step(double t0, double tmax);

// Whether a group of N bodies with kick-pair mask `kick` uses the team form
// of the orbit producer (mode: -1 automatic, 0 never, 1 whenever possible).
bool use_team(int mode, int N, unsigned long long kick);
bool use_wide(int mode, bool latency_bound, unsigned long long kick);

// Kernel launchers for body count N (nbg_inst.cu instantiates the kernels).
int launch_group_orbit(int N, const GroupArgs& g, int chunk, cudaStream_t st);
int launch_group_transit(int N, const GroupArgs& g, int chunk, cudaStream_t st);
int launch_group_operators(int N, const GroupArgs& g, int chunk, cudaStream_t st);
int launch_group_jacobian(int N, const GroupArgs& g, int chunk, cudaStream_t st);
int launch_group_seed(int N, const GroupArgs& g, cudaStream_t st);

// Gather / scatter between packed caller-layout arrays and a group's SoA
// state, for the group slots s with sysidx[s] >= 0 (off indexed by sysidx).
void launch_pack_state(int N, int S, const int* sysidx, const SysOff* off, const double* x, const double* v,
                       const double* xe, const double* ve, const double* m, const double* dqdt,
                       const long long* count, const GroupArgs& g, cudaStream_t st);
void launch_unpack_state(int N, int S, int grad, const int* sysidx, const SysOff* off, double* x, double* v,
                         double* xe, double* ve, double* dqdt, long long* count, const GroupArgs& g,
                         cudaStream_t st);
void launch_pack_jac(int N, int S, const int* sysidx, const SysOff* off, const double* J, const double* E,
                     const GroupArgs& g, int* bad, cudaStream_t st);
void launch_unpack_jac(int N, int S, const int* sysidx, const SysOff* off, double* J, double* E,
                       const GroupArgs& g, cudaStream_t st);
// calc_dtdelements! for the systems list[0..nlist) (all of 0..nlist when
// list is null).  With after_dtdq0 the output of a system starts right after
// its dtdq0 block in the same array (dtdel is then the dtdq0 base pointer).
void launch_dtdelements(int nlist, const int* list, const SysOff* off, const double* dtdq0, const double* jac_init,
                        double* dtdel, const long long* count, bool after_dtdq0, cudaStream_t st);

// init_nbody for nsys systems on the device (nbg_ics.cu).  Array pointers
// are device pointers (H may be null: fully nested hierarchies); n and t0
// are host arrays.  get(ctx, name, bytes) returns device scratch.
int init_nbody_device(int device, cudaStream_t st, int nsys, const int32_t* n, const double* t0,
                      const double* d_elements, const double* d_H, double* d_x, double* d_v, double* d_jinit,
                      void* (*get)(void* ctx, const char* name, size_t bytes), void* ctx);

}  // namespace nbg

#define NBG_CUDA(call)                                                                                    \
  do {                                                                                                    \
    cudaError_t e_ = (call);                                                                              \
    if (e_ != cudaSuccess)                                                                                \
      return ::nbg::set_error(NBG_ECUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)
