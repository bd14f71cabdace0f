// nbg_inst.cu -- instantiates the kernels of nbg_kernels_impl.cuh for one
// body count, NBG_N, given on the nvcc command line (-DNBG_N=2 ... -DNBG_N=10).
#include "nbg_kernels_impl.cuh"

#ifndef NBG_N
#error "compile with -DNBG_N=<bodies>"
#endif

namespace nbg {
template int launch_orbit<NBG_N>(const GroupArgs&, int, cudaStream_t);
template int launch_jac<NBG_N>(const GroupArgs&, int, cudaStream_t);
template int launch_seed<NBG_N>(const GroupArgs&, cudaStream_t);
template int launch_transit<NBG_N>(const GroupArgs&, int, cudaStream_t);
template int launch_operators<NBG_N>(const GroupArgs&, int, cudaStream_t);
}  // namespace nbg
