// tempo_internal.h -- interfaces between the translation units of libtempo_gb300.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "tempo_consts.h"
#include "tempo_dfloat.cuh"
#include "tempo_dual.cuh"
#include "tempo_types.h"

namespace tg {

template <class R> struct Tables;
template <class S> struct StepArgs;
template <class S> struct BatchArgs;
template <class I> struct IslandConsts;

// tempo_step_f64.cu (FP64 drop-in, compiled without FMA contraction)
cudaError_t launch_step_f64(const StepArgs<double>& a, const Tables<double>& t,
                            const TempoConsts<double>& c64, const IslandConsts<double>& i64,
                            cudaStream_t s, const cudaEvent_t* ev, int sedim_variant);

// tempo_step_f32.cu (mixed precision: FP32 bulk, double-float islands); sedim_variant
// in [0, kSedimCandidates) (tempo_step.cuh: sedim_group, sedim_split)
cudaError_t launch_step_mixed_f32(const StepArgs<float>& a, const Tables<float>& t,
                                  const TempoConsts<float>& c32, const IslandConsts<df>& idf,
                                  cudaStream_t s, const cudaEvent_t* ev, int points_variant,
                                  int sedim_variant);
cudaError_t launch_step_mixed_f64(const StepArgs<double>& a, const Tables<float>& t,
                                  const TempoConsts<float>& c32, const IslandConsts<df>& idf,
                                  cudaStream_t s, const cudaEvent_t* ev, int sedim_variant);
// tempo_points_f32.cu: points kernel of the mixed form on FP32 storage, variant v in
// [0, kPointsVariants) (tempo_step.cuh describes the variants)
cudaError_t launch_points_mixed_f32(int v, const StepArgs<float>& a, const Tables<float>& t,
                                    const TempoConsts<float>& c, const IslandConsts<df>& ci,
                                    cudaStream_t s);
cudaError_t launch_points_mixed_f32_lo(int v, const StepArgs<float>& a, const Tables<float>& t,
                                       const TempoConsts<float>& c, const IslandConsts<df>& ci,
                                       cudaStream_t s);
cudaError_t launch_points_mixed_f32_hi(int v, const StepArgs<float>& a, const Tables<float>& t,
                                       const TempoConsts<float>& c, const IslandConsts<df>& ci,
                                       cudaStream_t s);
// tempo_deriv_f64.cu / tempo_deriv_f32.cu: tangent-linear and adjoint launches of the
// step on element type T (tempo_deriv.cuh)
template <class T>
struct DerivOps {
  static cudaError_t pack(Dual<T, 1>* dst, const T* v, const T* d, long n, cudaStream_t s);
  static cudaError_t unpack(T* v, T* d, const Dual<T, 1>* src, long n, cudaStream_t s);
  static cudaError_t tl_step(const StepArgs<Dual<T, 1>>& a, const Tables<T>& t, const TempoConsts<T>& c,
                             const IslandConsts<Dual<T, 1>>& ci, cudaStream_t s, int part);
  static cudaError_t colflag(uint8_t* flag, const int* act, const unsigned* nact, long ncol,
                             cudaStream_t s);
  static cudaError_t adj_final(const StepArgs<T>& a, const TempoConsts<T>& c,
                               const IslandConsts<Dual<T, C_N>>& ci, const AdjArgs<T>& j, cudaStream_t s);
  static cudaError_t adj_sedim(const StepArgs<T>& a, const AdjArgs<T>& j, T* work, const SedWork& W,
                               cudaStream_t s);
  static cudaError_t adj_points(const StepArgs<T>& a, const Tables<T>& t, const TempoConsts<T>& c,
                                const IslandConsts<Dual<T, IN_N>>& ci, const AdjArgs<T>& j, cudaStream_t s);
  // the same without hail-aware graupel: IN_NG directions (ng and qb are no inputs)
  static cudaError_t adj_points_nohail(const StepArgs<T>& a, const Tables<T>& t, const TempoConsts<T>& c,
                                       const IslandConsts<Dual<T, IN_NG>>& ci, const AdjArgs<T>& j,
                                       cudaStream_t s);
  static cudaError_t adj_early(const StepArgs<T>& a, const TempoConsts<T>& c,
                               const IslandConsts<Dual<T, IN_N>>& ci, const AdjArgs<T>& j, cudaStream_t s);
};

// tempo_batch.cu: the mixed step over a multi-domain batch (FP32 storage), one launch
// sequence for every domain
cudaError_t launch_batch_mixed_f32(const BatchArgs<float>& b, const Tables<float>& t,
                                   const TempoConsts<float>& c32, const IslandConsts<df>& idf,
                                   cudaStream_t s, const cudaEvent_t* ev, int sedim_variant);

// tempo_noalloc.cu: the fixed scratch of tempo_run_dev_f32_noalloc_c (bytes, and its
// address on `device`, looked up on the first call for that device)
constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;
cudaError_t noalloc_scratch(int device, void** ptr);

// tempo_validate.cu: the input scan of tempo_set_validation.  Field f of the tile is
// bad where it is not finite or, with positive[f], not > 0; the scan keeps the least
// (tile point q = i + ti * (k + nz * j)) * kValidateFields + f over all bad values
// in *first (which the caller sets to ~0 first).
constexpr int kValidateFields = 20;
template <class S>
struct ValidateFields {
  const S* p[kValidateFields];
  int positive[kValidateFields];
  int nf;
  long NI, NK;
  int i0, k0, j0, ti, tj, nz;
};
template <class S>
cudaError_t launch_validate(const ValidateFields<S>& v, unsigned long long* first, cudaStream_t s);

// tempo_melt.cu: melting-layer reflectivity pass after phase C (F_MELT), FP64
template <class S>
cudaError_t launch_melt_refl(const StepArgs<S>& a, const TempoConsts<double>& c, const RadarConsts& rc,
                             cudaStream_t s);

// number of points-kernel variants of the mixed form on FP32 storage, and of the
// autotuner's candidates (each variant in level-major and in regime order)
constexpr int kPointsVariants = 8;
constexpr int kPointsCandidates = 2 * kPointsVariants;
// number of sedimentation-kernel variants (tempo_step.cuh: sedim_group, sedim_split,
// sedim_blocked)
constexpr int kSedimCandidates = 12;
// kernels launched per step (prep, points, sedim, final), and one more when phase A's
// points run in regime order
constexpr int kStepLaunches = 4;
constexpr int kOrderLaunches = 1;
// timed intervals of a step: prep, regime order, points, sedim, final
constexpr int kStepPhases = 5;

// tempo_tables.cu (FP64 table construction on the GPU)
struct DevTables64 {
  double *t_efrw, *t_efsw, *tpc_wev, *tnc_wev, *tps_iaus, *tni_iaus, *tpi_ide;
  double *qg, *qs, *qrfz, *qcfz;  // AoS layouts described in tempo_level.cuh
  float* tnccn;
  double* edges;  // [kEdgesCount] bin edges of the log-based indices (make_index_edges)
};
// small init tables: compute_efrw/efsw, compute_drop_evap, qi_aut_qs
// (tc: the constant set; the small tables use only its hail-independent members)
cudaError_t build_small_tables(const DevTables64& t, const TempoBins& bins,
                               const TempoConsts<double>& tc, cudaStream_t s);
// the three large tables (tables.F90:493-805) with hail-aware graupel constants
cudaError_t build_big_tables(const DevTables64& t, const TempoBins& bins,
                             const TempoConsts<double>& hail_consts, double* work,
                             size_t work_bytes, cudaStream_t s);
size_t big_tables_work_bytes();
// element-wise double -> float copy
cudaError_t narrow_copy(float* dst, const double* src, long n, cudaStream_t s);
// AoS <-> Fortran-order SoA conversion for one array of a family
cudaError_t aos_scatter(double* aos, const double* soa, long n, int nfam, int which, cudaStream_t s);
cudaError_t aos_gather(double* soa, const double* aos, long n, int nfam, int which, cudaStream_t s);
// nwfa(i,kts,j) += nwfa2d(i,j)*dt
cudaError_t launch_surface_emissions(double* nwfa, const double* nwfa2d, long ni, long nk, long nj,
                                     int kts_off, double dt, cudaStream_t s);

}  // namespace tg
