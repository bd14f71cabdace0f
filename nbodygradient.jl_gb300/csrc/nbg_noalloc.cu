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
// The array lives in this translation unit alone, so its device memory is
// reserved only once something asks for its address, not by the other
// entry points.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/nbg.h"

static __device__ __align__(256) unsigned char g_noalloc_scratch[NBG_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};
}  // namespace

// Device address of the scratch array on `device`, which must be the current
// device.  Resolved with cudaGetSymbolAddress on the first request for each
// device and cached; later requests only read the cache.
__attribute__((visibility("hidden"))) cudaError_t nbg_noalloc_scratch(int device, unsigned char** out) {
  *out = nullptr;
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[device] = (unsigned char*)p;
  }
  *out = g_scratch_ptr[device];
  return cudaSuccess;
}
