// tempo_step_f64.cu -- FP64 drop-in instantiation of the column step.
// Built with -fmad=false: the reference's gfortran -O0 build on x86-64 fuses no
// multiply-adds, so neither may this path.
#include "tempo_internal.h"
#include "tempo_step.cuh"

namespace tg {

cudaError_t launch_step_f64(const StepArgs<double>& a, const Tables<double>& t,
                            const TempoConsts<double>& c64, cudaStream_t s) {
  const int block = 128;
  const unsigned grid = (unsigned)((a.ncol + block - 1) / block);
  if (grid == 0) return cudaSuccess;
  tempo_column_kernel<double, double><<<grid, block, 0, s>>>(a, t, c64, c64);
  return cudaGetLastError();
}

}  // namespace tg
