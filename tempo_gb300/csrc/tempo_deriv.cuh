// tempo_deriv.cuh -- launch layer of the tangent-linear and adjoint steps (element type
// T: double for the FP64 derivatives, float for the FP32 ones).
//
// Tangent-linear: the four step kernels instantiated with R = S = Dual<T, 1> on packed
// (value, tangent) copies of the state.  Adjoint: that same step with zero tangents
// recomputes the forward trajectory (snapshots after phase A and before
// sedimentation), then the adjoint kernels of tempo_adjoint.cuh run in reverse order:
// final (phase C), sedimentation, points (phase A), early-exit columns.
#pragma once

#include "tempo_adjoint.cuh"
#include "tempo_launch.cuh"

namespace tg {

template <class T>
__global__ void k_pack_dual(Dual<T, 1>* dst, const T* v, const T* d, long n) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  dst[i].v = v ? v[i] : T(0);
  dst[i].d[0] = d ? d[i] : T(0);
}
template <class T>
__global__ void k_unpack_dual(T* v, T* d, const Dual<T, 1>* src, long n) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (v) v[i] = src[i].v;
  if (d) d[i] = src[i].d[0];
}
// colflag[c] = 1 for the active columns of the last prep
__global__ void k_colflag(uint8_t* flag, const int* act, const unsigned* nact, long ncol);

inline unsigned grid_of(long n, int b = 256) { return (unsigned)((n + b - 1) / b); }

template <class T>
cudaError_t pack_dual(Dual<T, 1>* dst, const T* v, const T* d, long n, cudaStream_t s) {
  if (n > 0) k_pack_dual<T><<<grid_of(n), 256, 0, s>>>(dst, v, d, n);
  return cudaGetLastError();
}
template <class T>
cudaError_t unpack_dual(T* v, T* d, const Dual<T, 1>* src, long n, cudaStream_t s) {
  if (n > 0) k_unpack_dual<T><<<grid_of(n), 256, 0, s>>>(v, d, src, n);
  return cudaGetLastError();
}

// step on packed dual state: part 0 = all four kernels, 1 = prep + points, 2 = sedim
// only, 3 = final only (with a.ord, phase A's points in regime order)
template <class T>
cudaError_t tl_step(const StepArgs<Dual<T, 1>>& a, const Tables<T>& t, const TempoConsts<T>& c,
                    const IslandConsts<Dual<T, 1>>& ci, cudaStream_t s, int part) {
  using D1 = Dual<T, 1>;
  const long ncol = a.ncol;
  if (ncol == 0) return cudaSuccess;
  const unsigned gcol = (unsigned)((ncol + kBlock - 1) / kBlock);
  const unsigned gpts = points_grid(a.ncol, a.nz);
  if (part == 0 || part == 1) {
    tempo_prep_kernel<D1, D1><<<gcol, kBlock, 0, s>>>(a, c, ci);
    if (cudaError_t e = launch_regime_order(a, s)) return e;
    tempo_points_kernel<D1, D1, 0><<<gpts, kBlock, 0, s>>>(a, t, c, ci);
  }
  if (part == 0 || part == 2) tempo_sedim_kernel<D1, D1><<<gcol, kBlock, 0, s>>>(a);
  if (part == 0 || part == 3) tempo_final_kernel<D1, D1><<<gpts, kBlock, 0, s>>>(a, c, ci);
  return cudaGetLastError();
}

template <class T>
cudaError_t adjoint_final(const StepArgs<T>& a, const TempoConsts<T>& c,
                          const IslandConsts<Dual<T, C_N>>& ci, const AdjArgs<T>& j, cudaStream_t s) {
  tempo_final_adjoint_kernel<T><<<points_grid(a.ncol, a.nz), kBlock, 0, s>>>(a, c, ci, j);
  return cudaGetLastError();
}
template <class T>
cudaError_t adjoint_sedim(const StepArgs<T>& a, const AdjArgs<T>& j, T* work, const SedWork& W,
                          cudaStream_t s) {
  tempo_sedim_adjoint_kernel<T><<<(unsigned)((a.ncol + kBlock - 1) / kBlock), kBlock, 0, s>>>(a, j, work, W);
  return cudaGetLastError();
}
template <class T, int N>
cudaError_t adjoint_points(const StepArgs<T>& a, const Tables<T>& t, const TempoConsts<T>& c,
                           const IslandConsts<Dual<T, N>>& ci, const AdjArgs<T>& j, cudaStream_t s) {
  tempo_points_adjoint_kernel<T, N><<<points_grid(a.ncol, a.nz), kBlock, 0, s>>>(a, t, c, ci, j);
  return cudaGetLastError();
}
template <class T>
cudaError_t adjoint_early(const StepArgs<T>& a, const TempoConsts<T>& c,
                          const IslandConsts<Dual<T, IN_N>>& ci, const AdjArgs<T>& j, cudaStream_t s) {
  tempo_early_adjoint_kernel<T><<<points_grid(a.ncol, a.nz), kBlock, 0, s>>>(a, c, ci, j);
  return cudaGetLastError();
}

}  // namespace tg
