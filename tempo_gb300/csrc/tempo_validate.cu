// tempo_validate.cu -- the input scan of tempo_set_validation on device arrays: one
// grid-stride pass over the tile's points, every listed field read once (HBM-bound),
// the first bad (point, field) kept with one atomicMin.
#include <cuda_runtime.h>

#include "tempo_internal.h"

namespace tg {

namespace {

template <class S>
__global__ void __launch_bounds__(256) tempo_validate_kernel(const __grid_constant__ ValidateFields<S> v,
                                                             unsigned long long* first) {
  const long n = (long)v.ti * v.nz * v.tj;
  for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
    const long i = q % v.ti, k = (q / v.ti) % v.nz, j = q / ((long)v.ti * v.nz);
    const long e = (v.i0 + i) + (v.k0 + k) * v.NI + (v.j0 + j) * v.NI * v.NK;
    for (int f = 0; f < v.nf; f++) {
      const S* p = v.p[f];
      if (!p) continue;
      const double x = (double)p[e];
      if (!isfinite(x) || (v.positive[f] && !(x > 0.0)))
        atomicMin(first, (unsigned long long)q * kValidateFields + (unsigned long long)f);
    }
  }
}

}  // namespace

template <class S>
cudaError_t launch_validate(const ValidateFields<S>& v, unsigned long long* first, cudaStream_t s) {
  const long n = (long)v.ti * v.nz * v.tj;
  if (n <= 0) return cudaSuccess;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long want = (n + 255) / 256;
  const int grid = (int)(want < (long)sms * 8 ? want : (long)sms * 8);
  tempo_validate_kernel<S><<<grid, 256, 0, s>>>(v, first);
  return cudaGetLastError();
}

template cudaError_t launch_validate<float>(const ValidateFields<float>&, unsigned long long*, cudaStream_t);
template cudaError_t launch_validate<double>(const ValidateFields<double>&, unsigned long long*, cudaStream_t);

}  // namespace tg
