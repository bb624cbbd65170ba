// tempo_noalloc.cu -- fixed device scratch for tempo_run_dev_f32_noalloc_c.
//
// Some hosts must not allocate device memory inside their time step: a model that
// sizes its device memory pool once at start-up and leaves no headroom, or one that
// must not let a physics call synchronise the whole device (cudaFree does, cudaMalloc
// may).  tempo_run_dev_f32_c grows its context's scratch with cudaMalloc on demand;
// for these hosts the same step takes its scratch from the file-scope device array
// below instead, whose kNoAllocScratchBytes are reserved when this module is loaded on
// a device.  The array's address is looked up once per device, with that device
// current, and handed to the kernels as a plain pointer.
#include <cuda_runtime.h>

#include <mutex>

#include "tempo_internal.h"

namespace tg {

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
void* g_noalloc_addr[kMaxDevices] = {};
std::mutex g_noalloc_mu;

}  // namespace

cudaError_t noalloc_scratch(int device, void** ptr) {
  *ptr = nullptr;
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[device]) {
    int cur = -1;
    cudaError_t e = cudaGetDevice(&cur);
    if (e != cudaSuccess) return e;
    if (cur != device && (e = cudaSetDevice(device)) != cudaSuccess) return e;
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (cur != device) {
      const cudaError_t e2 = cudaSetDevice(cur);
      if (e == cudaSuccess) e = e2;
    }
    if (e != cudaSuccess) return e;
    g_noalloc_addr[device] = p;
  }
  *ptr = g_noalloc_addr[device];
  return cudaSuccess;
}

}  // namespace tg
