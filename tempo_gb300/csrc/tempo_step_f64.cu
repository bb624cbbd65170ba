// tempo_step_f64.cu -- FP64 drop-in instantiation of the column step.
// Built with -fmad=false: the reference's gfortran -O0 build on x86-64 fuses no
// multiply-adds, so neither may this path.
#include "tempo_launch.cuh"

namespace tg {

cudaError_t launch_step_f64(const StepArgs<double>& a, const Tables<double>& t,
                            const TempoConsts<double>& c64, const IslandConsts<double>& i64,
                            cudaStream_t s, const cudaEvent_t* ev, int sedim_variant) {
  return launch_step<double, double>(a, c64, i64, s, ev, [&] {
    return launch_points<double, double, 0>(a, t, c64, i64, s);
  }, sedim_variant);
}

}  // namespace tg
