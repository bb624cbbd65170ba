// tempo_points_f32.cu -- the points-kernel variants of the mixed form on FP32 storage.
// Compiled twice (TEMPO_VARIANT_SET 0: variants 0-3, 1: variants 4-7) so that the
// build compiles them in parallel.
#include "tempo_launch.cuh"

#ifndef TEMPO_VARIANT_SET
#error "TEMPO_VARIANT_SET must be 0 or 1"
#endif

namespace tg {

#if TEMPO_VARIANT_SET == 0
cudaError_t launch_points_mixed_f32_lo(int v, const StepArgs<float>& a, const Tables<float>& t,
                                       const TempoConsts<float>& c, const IslandConsts<df>& ci,
                                       cudaStream_t s) {
  switch (v) {
    case 0: return launch_points<float, float, 0>(a, t, c, ci, s);
    case 1: return launch_points<float, float, 1>(a, t, c, ci, s);
    case 2: return launch_points<float, float, 2>(a, t, c, ci, s);
    case 3: return launch_points<float, float, 3>(a, t, c, ci, s);
    default: return cudaErrorInvalidValue;
  }
}
#else
cudaError_t launch_points_mixed_f32_hi(int v, const StepArgs<float>& a, const Tables<float>& t,
                                       const TempoConsts<float>& c, const IslandConsts<df>& ci,
                                       cudaStream_t s) {
  switch (v) {
    case 4: return launch_points<float, float, 4>(a, t, c, ci, s);
    case 5: return launch_points<float, float, 5>(a, t, c, ci, s);
    case 6: return launch_points<float, float, 6>(a, t, c, ci, s);
    case 7: return launch_points<float, float, 7>(a, t, c, ci, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_points_mixed_f32(int v, const StepArgs<float>& a, const Tables<float>& t,
                                    const TempoConsts<float>& c, const IslandConsts<df>& ci,
                                    cudaStream_t s) {
  if (v < 0 || v >= kPointsVariants) return cudaErrorInvalidValue;
  return v < 4 ? launch_points_mixed_f32_lo(v, a, t, c, ci, s)
               : launch_points_mixed_f32_hi(v, a, t, c, ci, s);
}
#endif

}  // namespace tg
