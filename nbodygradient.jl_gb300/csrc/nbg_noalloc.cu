// nbg_noalloc.cu -- the fixed device scratch area behind
// nbg_batch_integrate_transits_noalloc.
//
// That entry point serves callers that cannot let the library allocate device
// memory while it runs: a sampler or pipeline that reserves the GPU's memory
// for itself up front and hands the library only its own buffers, and loops
// that must not pay the device-wide synchronisation and host latency of
// cudaMalloc / cudaFree when a larger batch arrives.  All of its working
// memory (the SoA system state, the operator records, the transit queue, the
// Jacobian columns) is carved out of the one array below, whose size is fixed
// when the library is built (NBG_NOALLOC_SCRATCH_BYTES in nbg.h).
//
// When the array's device memory is reserved depends on CUDA's module
// loading.  With lazy loading (the default since CUDA 12.2) the module that
// holds the array is loaded on a device -- and its 64 MiB reserved there --
// the first time the array's address is asked for on that device, i.e. by
// the first call of the entry point; a caller that then holds the rest of
// the GPU's memory must make that first call before taking it, or the lookup
// fails with an out-of-memory error (reported as NBG_ECUDA).  With
// CUDA_MODULE_LOADING=EAGER every context that loads the library reserves the
// array when it is created, whether or not it ever calls the entry point.
#include <cuda_runtime.h>

#include "../../include/nbg.h"

static __device__ __align__(256) unsigned char g_noalloc_scratch[NBG_NOALLOC_SCRATCH_BYTES];

// Device address of the scratch array on the current device, which must be
// `device`.  Looked up with cudaGetSymbolAddress on every call (cheap once the
// module is loaded), so that an address never outlives the CUDA context it
// belongs to: a cache keyed by device would hand out a stale pointer after the
// host process resets the device and a new primary context is created.
__attribute__((visibility("hidden"))) cudaError_t nbg_noalloc_scratch(int device, unsigned char** out) {
  *out = nullptr;
  int cur = -1;
  cudaError_t e = cudaGetDevice(&cur);
  if (e != cudaSuccess) return e;
  if (cur != device) return cudaErrorInvalidDevice;
  void* p = nullptr;
  e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return e;
  *out = (unsigned char*)p;
  return cudaSuccess;
}
