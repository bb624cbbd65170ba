// tempo_step_f32.cu -- mixed-precision instantiations of the column step: FP32 bulk
// process rates with double-float thermodynamic and sedimentation islands, on FP32 or
// FP64 storage.  The points-kernel variants on FP32 storage live in tempo_points_f32.cu.
#include "tempo_launch.cuh"

namespace tg {

cudaError_t launch_step_mixed_f32(const StepArgs<float>& a, const Tables<float>& t,
                                  const TempoConsts<float>& c32, const IslandConsts<df>& idf,
                                  cudaStream_t s, const cudaEvent_t* ev, int variant, int sedim_variant) {
  return launch_step<float, float>(a, c32, idf, s, ev, [&] {
    return launch_points_mixed_f32(variant, a, t, c32, idf, s);
  }, sedim_variant);
}
cudaError_t launch_step_mixed_f64(const StepArgs<double>& a, const Tables<float>& t,
                                  const TempoConsts<float>& c32, const IslandConsts<df>& idf,
                                  cudaStream_t s, const cudaEvent_t* ev, int sedim_variant) {
  return launch_step<float, double>(a, c32, idf, s, ev, [&] {
    return launch_points<float, double, 0>(a, t, c32, idf, s);
  }, sedim_variant);
}

}  // namespace tg
