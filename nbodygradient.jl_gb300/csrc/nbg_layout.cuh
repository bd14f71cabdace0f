// nbg_layout.cuh -- data layout shared by the host orchestration and the
// kernels of libnbg_cuda: operator-record sizes, the per-group argument block
// and the launcher declarations (definitions live in nbg_kernels_impl.cuh and
// are instantiated once per body count by nbg_inst.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace nbg {

// Pair record: K[36] (row-major r*6+l), mi, mj, jac_ij[:,m_i] (12), jac_ij[:,m_j] (12)
constexpr int PREC = 62;
constexpr int PREC_MI = 36, PREC_MJ = 37, PREC_MC6 = 38, PREC_MC13 = 50;

__host__ __device__ constexpr int op_size(int N) { return 12 * N * N; }
__host__ __device__ inline int pair_bit(int i, int j, int N) { return i * N - i * (i + 1) / 2 + (j - i - 1); }

// Record size of one step for N bodies with npk Kepler pairs; kick operators
// only when the group has kick pairs.
__host__ __device__ inline int step_record_size(int N, int npk, bool kick) {
  return (kick ? 2 * op_size(N) : 0) + 2 * npk * PREC + op_size(N);
}

constexpr int PROD_BS = 32;     // orbit producer: threads per warp-sized unit of work
constexpr int PROD_MAX_WARPS = 4;  // orbit producer: up to 4 independent warps per block
constexpr int CONS_BS = 128;    // Jacobian consumer: four warps per block
constexpr int TRANSIT_BS = 32;  // transit searches: one warp per block
constexpr int OPS_BS = 128;     // operator kernels

// Doubles per transit of the adjoint record: the row u^T = w^T S(dt0) of
// the transit time and gdot (7N + 1); TransitParameters add the rows of
// v_sky and b_sky^2, v_sky and d v_sky / dt (21N + 3).
__host__ __device__ inline int trec_size(int N, int tbv) { return tbv ? 21 * N + 3 : 7 * N + 1; }

// Captured Kepler-pair parameters (producer -> operator kernel): x0[3], v0[3]
// and the 22 values jac_delxv_gamma! returns (ahl21.jl:888-889).
constexpr int PCAP = 28;
// Position snapshots per step: [0] at the correctors, [1] at the first and
// [2] at the second kick (kick groups only); 3N doubles each.
__host__ __device__ inline int snap_count(bool kick) { return kick ? 3 : 1; }


struct GroupArgs {
  int N, S, nsys, grad, K, R, npk;
  int spw;   // orbit producer: systems per warp (lanes >= spw idle)
  int team;  // orbit producer: 1 = a team of lanes per system (orbit_team_kernel), 0 = one lane
  // transit searches of this chunk in the team form (with team != 0): set by
  // the host per chunk when few systems of the group are still running, so
  // that the searches are latency-bound; a full group keeps one lane per
  // search, which uses every lane of every warp
  int search_team;
  // orbit producer in the wide team form (two lanes per pair solve,
  // orbit_team_kernel<N, 2>) for this chunk: set by the host for latency-bound
  // chunks (few systems running) of groups without kick pairs
  int wide;
  // Block layout of the orbit producer: pwarps independent warps per block
  // (0 or 1: one) and prod_smem bytes of dynamic shared memory per block (at
  // least what the team form needs).  A large allocation keeps the
  // shared-memory-hungry consumer blocks, and the operator / search blocks
  // that ask for guard_smem bytes, off the SMs that run producer blocks.
  int pwarps, prod_smem, guard_smem;
  unsigned long long kick;
  // per-system state, structure of arrays: element e of system s at [e * S + s]
  double *x, *v, *xe, *ve, *m, *dqdt, *gsave;
  long long* count;  // [N][S]
  double *t0, *h, *hI;
  long long* nsteps;
  // first chunk of each slot, in steps (null: every system starts at chunk 0);
  // the request server admits systems into running groups this way
  const long long* kbase;
  // length of each system's last step (null: h); the plain integration
  // drivers end on a fractional step (Integrator.jl:187-194)
  const double* hlast;
  int notransit;  // 1: no transit detection (the plain integration drivers)
  int tbv;        // 1: TransitParameters outputs (t, v_sky, b_sky^2 per transit)
  // CartesianOutput recording (null: off): the state at the start of every
  // step of the chunk, x and v as [slot][step][x (3N), v (3N)], jac_step as
  // [slot][step][7N x 7N column-major]
  double* trajxv;
  double* trajJ;
  int *ntt, *ti, *sysidx;
  unsigned int* status;
  // packed outputs in the caller's layout, indexed by global system
  double* tt;
  const long long* off_tt;
  double* dtdq0;
  const long long* off_dq;
  // records
  double* steprec;  // [K][R][S]
  double* trec;     // [K][N-1][7N+1][S]
  int* tflag;       // [K][N-1][S]
  // consumer state: non-mass rows of jac_step / jac_error, [S][6N][7N]
  double *Jint, *Eint;
  // transit searches queued by the orbit producer for the transit kernel
  double* task_f;   // [task_cap][12N + 2]: x, v, xerror, verror, first dt0, t
  int* task_i;      // [task_cap][3]: system, slot kk*(N-1)+o, transit index
  int* task_count;  // tasks queued in this chunk
  int task_cap;
  double* tscratch;  // [R][tgrid]: operator records of a search's final partial step
  int tgrid;         // threads of the transit kernel
  // producer captures for the operator kernels
  double* pcap;   // [K][2 npk][28][S]: Kepler-pair parameters
  double* xsnap;  // [K][snaps][3N][S]: positions at the correctors (and kicks)
};

// Length of step istep of the system in slot s (nst steps in all).
__device__ __forceinline__ double step_length(const GroupArgs& g, int s, long long istep, long long nst, double h) {
  return (g.hlast && istep == nst - 1) ? g.hlast[s] : h;
}

// Index of the first step of chunk `chunk` for the system in slot s (negative
// while the slot's system is admitted for a later chunk: the request server
// writes a slot's settings while the previous chunk's kernels may still run).
__device__ __forceinline__ long long chunk_first_step(const GroupArgs& g, int chunk, int s) {
  return (long long)chunk * g.K - (g.kbase ? g.kbase[s] : 0);
}

template <int N> int launch_orbit(const GroupArgs& g, int chunk, cudaStream_t st);
template <int N> int launch_jac(const GroupArgs& g, int chunk, cudaStream_t st);
template <int N> int launch_seed(const GroupArgs& g, cudaStream_t st);
template <int N> int launch_transit(const GroupArgs& g, int chunk, cudaStream_t st);
template <int N> int launch_operators(const GroupArgs& g, int chunk, cudaStream_t st);

}  // namespace nbg
