// tempo_step_f32.cu -- mixed-precision instantiations of the column step: FP32 bulk
// process rates with the FP64 thermodynamic and sedimentation islands, on FP32 or
// FP64 storage.
#include "tempo_internal.h"
#include "tempo_step.cuh"

namespace tg {

template <class S>
static cudaError_t launch_mixed(const StepArgs<S>& a, const Tables<float>& t, const TempoConsts<float>& c32,
                                const TempoConsts<double>& c64, cudaStream_t s) {
  const int block = 128;
  const unsigned grid = (unsigned)((a.ncol + block - 1) / block);
  if (grid == 0) return cudaSuccess;
  tempo_column_kernel<float, S><<<grid, block, 0, s>>>(a, t, c32, c64);
  return cudaGetLastError();
}

cudaError_t launch_step_mixed_f32(const StepArgs<float>& a, const Tables<float>& t,
                                  const TempoConsts<float>& c32, const TempoConsts<double>& c64,
                                  cudaStream_t s) {
  return launch_mixed(a, t, c32, c64, s);
}
cudaError_t launch_step_mixed_f64(const StepArgs<double>& a, const Tables<float>& t,
                                  const TempoConsts<float>& c32, const TempoConsts<double>& c64,
                                  cudaStream_t s) {
  return launch_mixed(a, t, c32, c64, s);
}

}  // namespace tg
