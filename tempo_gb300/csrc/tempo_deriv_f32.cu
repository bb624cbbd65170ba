// tempo_deriv_f32.cu -- tangent-linear and adjoint launches on float.
// Derivatives of the all-FP32 step (FP32 bulk and FP32 islands).
#include "tempo_deriv.cuh"

namespace tg {

using T_ = float;
template <> cudaError_t DerivOps<T_>::pack(Dual<T_, 1>* dst, const T_* v, const T_* d, long n, cudaStream_t s) {
  return pack_dual<T_>(dst, v, d, n, s);
}
template <> cudaError_t DerivOps<T_>::unpack(T_* v, T_* d, const Dual<T_, 1>* src, long n, cudaStream_t s) {
  return unpack_dual<T_>(v, d, src, n, s);
}
template <> cudaError_t DerivOps<T_>::tl_step(const StepArgs<Dual<T_, 1>>& a, const Tables<T_>& t,
                                              const TempoConsts<T_>& c, const IslandConsts<Dual<T_, 1>>& ci,
                                              cudaStream_t s, int part) {
  return tg::tl_step<T_>(a, t, c, ci, s, part);
}
template <> cudaError_t DerivOps<T_>::colflag(uint8_t* flag, const int* act, const unsigned* nact, long ncol,
                                              cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(flag, 0, (size_t)ncol, s);
  if (e != cudaSuccess) return e;
  if (ncol > 0) k_colflag<<<grid_of(ncol), 256, 0, s>>>(flag, act, nact, ncol);
  return cudaGetLastError();
}
template <> cudaError_t DerivOps<T_>::adj_final(const StepArgs<T_>& a, const TempoConsts<T_>& c,
                                                const IslandConsts<Dual<T_, C_N>>& ci, const AdjArgs<T_>& j,
                                                cudaStream_t s) {
  return adjoint_final<T_>(a, c, ci, j, s);
}
template <> cudaError_t DerivOps<T_>::adj_sedim(const StepArgs<T_>& a, const AdjArgs<T_>& j, T_* work,
                                                const SedWork& W, cudaStream_t s) {
  return adjoint_sedim<T_>(a, j, work, W, s);
}
template <> cudaError_t DerivOps<T_>::adj_points(const StepArgs<T_>& a, const Tables<T_>& t,
                                                 const TempoConsts<T_>& c, const IslandConsts<Dual<T_, IN_N>>& ci,
                                                 const AdjArgs<T_>& j, cudaStream_t s) {
  return adjoint_points<T_, IN_N>(a, t, c, ci, j, s);
}
template <> cudaError_t DerivOps<T_>::adj_points_nohail(const StepArgs<T_>& a, const Tables<T_>& t,
                                                        const TempoConsts<T_>& c,
                                                        const IslandConsts<Dual<T_, IN_NG>>& ci,
                                                        const AdjArgs<T_>& j, cudaStream_t s) {
  return adjoint_points<T_, IN_NG>(a, t, c, ci, j, s);
}
template <> cudaError_t DerivOps<T_>::adj_early(const StepArgs<T_>& a, const TempoConsts<T_>& c,
                                                const IslandConsts<Dual<T_, IN_N>>& ci, const AdjArgs<T_>& j,
                                                cudaStream_t s) {
  return adjoint_early<T_>(a, c, ci, j, s);
}

}  // namespace tg
