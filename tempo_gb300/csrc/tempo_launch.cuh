// tempo_launch.cuh -- enqueues the four kernels of one column step on a stream.
#pragma once

#include "tempo_internal.h"
#include "tempo_step.cuh"

namespace tg {

// ev (optional, kStepLaunches + 1 events): recorded before each kernel and after the
// last, for per-kernel durations measured on the launching stream
template <class R, class S>
cudaError_t launch_step(const StepArgs<S>& a, const Tables<R>& T, const TempoConsts<R>& c,
                        const IslandConsts<Isl<R>>& ci, cudaStream_t s, const cudaEvent_t* ev) {
  constexpr int B = 128;
  const unsigned long long ncol = (unsigned long long)a.ncol;
  const unsigned long long npts = ncol * (unsigned long long)a.nz;
  if (ncol == 0) return cudaSuccess;
  const unsigned gcol = (unsigned)((ncol + B - 1) / B);
  const unsigned gpts = (unsigned)((npts + B - 1) / B);
  // points/final size their grids for every column; threads past the active count
  // (read on the device after prep) return at once
  if (ev) cudaEventRecord(ev[0], s);
  tempo_prep_kernel<R, S><<<gcol, B, 0, s>>>(a, c, ci);
  if (ev) cudaEventRecord(ev[1], s);
  tempo_points_kernel<R, S><<<gpts, B, 0, s>>>(a, T, c, ci);
  if (ev) cudaEventRecord(ev[2], s);
  tempo_sedim_kernel<R, S><<<gcol, B, 0, s>>>(a);
  if (ev) cudaEventRecord(ev[3], s);
  tempo_final_kernel<R, S><<<gpts, B, 0, s>>>(a, c, ci);
  if (ev) cudaEventRecord(ev[4], s);
  return cudaGetLastError();
}

}  // namespace tg
