// tempo_launch.cuh -- enqueues the four kernels of one column step on a stream.
#pragma once

#include "tempo_internal.h"
#include "tempo_step.cuh"

namespace tg {

constexpr int kBlock = 128;

inline unsigned points_grid(long ncol, int nz) {
  const unsigned long long npts = (unsigned long long)ncol * (unsigned long long)nz;
  return (unsigned)((npts + kBlock - 1) / kBlock);
}

// points kernel, variant V; its grid covers every column's levels and threads past the
// active count (read on the device after prep) return at once
template <class R, class S, int V>
cudaError_t launch_points(const StepArgs<S>& a, const Tables<R>& T, const TempoConsts<R>& c,
                          const IslandConsts<Isl<R>>& ci, cudaStream_t s) {
  tempo_points_kernel<R, S, V><<<points_grid(a.ncol, a.nz), kBlock, 0, s>>>(a, T, c, ci);
  return cudaGetLastError();
}

// ev (optional, kStepLaunches + 1 events): recorded before each kernel and after the
// last, for per-kernel durations measured on the launching stream.  points() launches
// the points kernel (the variant is the caller's choice).
template <class R, class S, class Points>
cudaError_t launch_step(const StepArgs<S>& a, const TempoConsts<R>& c, const IslandConsts<Isl<R>>& ci,
                        cudaStream_t s, const cudaEvent_t* ev, Points&& points) {
  const unsigned long long ncol = (unsigned long long)a.ncol;
  if (ncol == 0) return cudaSuccess;
  const unsigned gcol = (unsigned)((ncol + kBlock - 1) / kBlock);
  const unsigned gpts = points_grid(a.ncol, a.nz);
  if (ev) cudaEventRecordWithFlags(ev[0], s, cudaEventRecordExternal);
  tempo_prep_kernel<R, S><<<gcol, kBlock, 0, s>>>(a, c, ci);
  if (ev) cudaEventRecordWithFlags(ev[1], s, cudaEventRecordExternal);
  cudaError_t e = points();
  if (e != cudaSuccess) return e;
  if (ev) cudaEventRecordWithFlags(ev[2], s, cudaEventRecordExternal);
  tempo_sedim_kernel<R, S><<<gcol, kBlock, 0, s>>>(a);
  if (ev) cudaEventRecordWithFlags(ev[3], s, cudaEventRecordExternal);
  tempo_final_kernel<R, S><<<gpts, kBlock, 0, s>>>(a, c, ci);
  if (ev) cudaEventRecordWithFlags(ev[4], s, cudaEventRecordExternal);
  return cudaGetLastError();
}

}  // namespace tg
