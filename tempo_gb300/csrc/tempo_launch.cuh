// tempo_launch.cuh -- enqueues the four kernels of one column step on a stream.
#pragma once

#include "tempo_internal.h"
#include "tempo_step.cuh"

namespace tg {

constexpr int kBlock = 128;

// Timing event on stream s: a plain record, or, while s is being captured into a CUDA
// graph, an external event-record node (so that the event is recorded at each replay).
inline void record_event(cudaEvent_t ev, cudaStream_t s) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s, &st);
  if (st == cudaStreamCaptureStatusActive)
    cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal);
  else
    cudaEventRecord(ev, s);
}

inline unsigned points_grid(long ncol, int nz) {
  const unsigned long long npts = (unsigned long long)ncol * (unsigned long long)nz;
  return (unsigned)((npts + kBlock - 1) / kBlock);
}

// points kernel, variant V; its grid covers every column's levels and threads past the
// active count (read on the device after prep) return at once
template <class R, class S, int V>
cudaError_t launch_points(const StepArgs<S>& a, const Tables<Cst<R>>& T, const TempoConsts<Cst<R>>& c,
                          const IslandConsts<Isl<R>>& ci, cudaStream_t s) {
  tempo_points_kernel<R, S, V><<<points_grid(a.ncol, a.nz), kBlock, 0, s>>>(a, T, c, ci);
  return cudaGetLastError();
}

// ev (optional, kStepLaunches + 1 events): recorded before each kernel and after the
// last, for per-kernel durations measured on the launching stream.  points() launches
// the points kernel (the variant is the caller's choice).
template <class R, class S, class Points>
cudaError_t launch_step(const StepArgs<S>& a, const TempoConsts<Cst<R>>& c, const IslandConsts<Isl<R>>& ci,
                        cudaStream_t s, const cudaEvent_t* ev, Points&& points) {
  const unsigned long long ncol = (unsigned long long)a.ncol;
  if (ncol == 0) return cudaSuccess;
  const unsigned gcol = (unsigned)((ncol + kBlock - 1) / kBlock);
  const unsigned gpts = points_grid(a.ncol, a.nz);
  if (ev) record_event(ev[0], s);
  tempo_prep_kernel<R, S><<<gcol, kBlock, 0, s>>>(a, c, ci);
  if (ev) record_event(ev[1], s);
  cudaError_t e = points();
  if (e != cudaSuccess) return e;
  if (ev) record_event(ev[2], s);
  if (a.flags & F_SEMI)
    tempo_sedim_semi_kernel<R, S><<<gcol, kBlock, 0, s>>>(a, c, ci);
  else
    tempo_sedim_kernel<R, S><<<gcol, kBlock, 0, s>>>(a);
  if (ev) record_event(ev[3], s);
  tempo_final_kernel<R, S><<<gpts, kBlock, 0, s>>>(a, c, ci);
  if (ev) record_event(ev[4], s);
  return cudaGetLastError();
}

}  // namespace tg
