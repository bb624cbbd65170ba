// tempo_launch.cuh -- enqueues the four kernels of one column step on a stream.
#pragma once

#include <algorithm>

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

inline unsigned points_grid(long ncol, int nz, int block = kBlock) {
  const unsigned long long npts = (unsigned long long)ncol * (unsigned long long)nz;
  return (unsigned)((npts + block - 1) / block);
}

// points kernel, variant V; its grid covers every column's levels and threads past the
// active count (read on the device after prep) return at once
template <class R, class S, int V>
cudaError_t launch_points(const StepArgs<S>& a, const Tables<Cst<R>>& T, const TempoConsts<Cst<R>>& c,
                          const IslandConsts<Isl<R>>& ci, cudaStream_t s) {
  constexpr int block = points_block(V);
  unsigned grid = points_grid(a.ncol, a.nz, block);
  if constexpr (points_persistent(V)) {
    // one resident block per SM (or fewer blocks than that when the points are few)
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tempo_points_kernel<R, S, V>, block, 0);
    if (e != cudaSuccess) return e;
    grid = std::min<unsigned>(grid, (unsigned)(std::max(per_sm, 1) * sms));
  }
  tempo_points_kernel<R, S, V><<<grid, block, 0, s>>>(a, T, c, ci);
  return cudaGetLastError();
}

// the explicit sedimentation kernel, variant sv (tempo_step.cuh: sedim_group,
// sedim_split, sedim_blocked)
template <class R, class S, int V = 0>
void launch_sedim(const StepArgs<S>& a, int sv, unsigned gcol, cudaStream_t s) {
  if constexpr (V + 1 < kSedimVariants)
    if (sv != V) return launch_sedim<R, S, V + 1>(a, sv, gcol, s);
  tempo_sedim_kernel<R, S, sedim_group(V), sedim_split(V), sedim_blocked(V)>
      <<<dim3(gcol, sedim_split(V) ? 2 : 1), kBlock, 0, s>>>(a);
}

// regime order of phase A's points into a.ord (nothing when a.ord is NULL); the grid
// covers every column's levels, windows past the active points return at once
template <class S>
cudaError_t launch_regime_order(const StepArgs<S>& a, cudaStream_t s) {
  if (!a.ord || a.ncol == 0) return cudaSuccess;
  constexpr unsigned long long per = kRegimeWindow;
  const unsigned greg = (unsigned)(((unsigned long long)a.ncol * (unsigned long long)a.nz + per - 1) / per);
  tempo_regime_order_kernel<S><<<greg, kRegimeBlock, 0, s>>>(a);
  return cudaGetLastError();
}

// ev (optional, kStepPhases + 1 events): recorded before prep, before the regime
// kernels (an empty interval when a.ord is NULL), before the points, sedimentation and
// final kernels and after the last, for per-kernel durations measured on the launching
// stream.  points() launches the points kernel (the variant is the caller's choice).
// With a.ord the regime kernels order phase A's points first.
// sedimentation variant sv (sedim_group) for the explicit path
template <class R, class S, class Points>
cudaError_t launch_step(const StepArgs<S>& a, const TempoConsts<Cst<R>>& c, const IslandConsts<Isl<R>>& ci,
                        cudaStream_t s, const cudaEvent_t* ev, Points&& points, int sv = 0) {
  const unsigned long long ncol = (unsigned long long)a.ncol;
  if (ncol == 0) return cudaSuccess;
  const unsigned gcol = (unsigned)((ncol + kBlock - 1) / kBlock);
  const unsigned gpts = points_grid(a.ncol, a.nz);
  if (ev) record_event(ev[0], s);
  tempo_prep_kernel<R, S><<<gcol, kBlock, 0, s>>>(a, c, ci);
  if (ev) record_event(ev[1], s);
  cudaError_t e = launch_regime_order(a, s);
  if (e != cudaSuccess) return e;
  if (ev) record_event(ev[2], s);
  e = points();
  if (e != cudaSuccess) return e;
  if (ev) record_event(ev[3], s);
  if (a.flags & F_SEMI)
    tempo_sedim_semi_kernel<R, S><<<gcol, kBlock, 0, s>>>(a, c, ci);
  else
    launch_sedim<R, S>(a, sv, gcol, s);
  if (ev) record_event(ev[4], s);
  tempo_final_kernel<R, S><<<gpts, kBlock, 0, s>>>(a, c, ci);
  if (ev) record_event(ev[5], s);
  return cudaGetLastError();
}

}  // namespace tg
