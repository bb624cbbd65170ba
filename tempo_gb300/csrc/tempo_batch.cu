// tempo_batch.cu -- the mixed-form column step over a batch of independent domains as
// one sequence of launches: prep over every domain's columns, a plan of the active work,
// the regime order and the persistent points kernel over every domain's points, the
// sedimentation over every active column and the final kernel over every point.  Each
// work item finds its domain by a binary search over the batch's prefix counts and runs
// the same per-point / per-column code as the single-tile step with its domain's step
// arguments (levels, dt, arrays, scratch), so a domain's results equal those of its own
// tempo_run_dev_f32_c call.  Small domains no longer leave the GPU idle between launches.
#include "tempo_launch.cuh"

namespace tg {

namespace {

// the domain of batch item x: the last d in [0, nd) with start[d] <= x (empty domains,
// whose start equals the next one's, are skipped)
template <class T>
__device__ __forceinline__ int domain_of(const T* start, int nd, long x) {
  int lo = 0, hi = nd - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((long)__ldg(start + mid) <= x)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

template <class R, class S>
__global__ void __launch_bounds__(128) tempo_prep_batch_kernel(const __grid_constant__ BatchArgs<S> b,
                                                                const __grid_constant__ TempoConsts<Cst<R>> cst,
                                                                const __grid_constant__ IslandConsts<Isl<R>> ci) {
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = g < b.ncol;
  const int d = valid ? domain_of(b.col_start, b.nd, g) : 0;
  prep_column<R, S>(b.dom[d], cst, ci, valid ? g - b.col_start[d] : 0, valid, d);
}

// prefix counts of the active slots and points of the domains; resets the work queue
template <class S>
__global__ void tempo_batch_plan_kernel(const __grid_constant__ BatchArgs<S> b) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  unsigned ns = 0, np = 0;
  for (int d = 0; d < b.nd; d++) {
    b.slot_start[d] = ns;
    b.pt_start[d] = np;
    const unsigned n = *b.dom[d].nact;
    ns += n;
    np += n * (unsigned)b.dom[d].nz;
  }
  b.slot_start[b.nd] = ns;
  b.pt_start[b.nd] = np;
  *b.queue = 0;
}

// (domain, level, slot) of batch point q
struct BatchPoint {
  int d, k;
  long s;
};
template <class S>
__device__ __forceinline__ BatchPoint batch_point(const BatchArgs<S>& b, long q) {
  BatchPoint r;
  r.d = domain_of(b.pt_start, b.nd, q);
  const long nact = (long)b.slot_start[r.d + 1] - (long)b.slot_start[r.d];
  const long p = q - (long)b.pt_start[r.d];
  r.k = (int)(p / nact);
  r.s = p - (long)r.k * nact;
  return r;
}

template <class S>
__global__ void __launch_bounds__(kRegimeBlock) tempo_regime_order_batch_kernel(const __grid_constant__ BatchArgs<S> b) {
  const long npts = (long)b.pt_start[b.nd];
  const long q0 = (long)blockIdx.x * kRegimeWindow;
  if (q0 >= npts) return;
  regime_order_window(q0, npts, [&](long q) {
    const BatchPoint bp = batch_point(b, q);
    const StepArgs<S>& a = b.dom[bp.d];
    return point_regime(a, col_geom(a, a.act[bp.s]).base + (long)bp.k * a.NI);
  }, b.ord);
}

// persistent points kernel (variant V of the single-tile kernel): blocks take chunks of
// points of the whole batch from the work queue
template <class R, class S, int V>
__global__ void __launch_bounds__(points_block(V), points_min_blocks(V)) tempo_points_batch_kernel(
    const __grid_constant__ BatchArgs<S> b, const __grid_constant__ Tables<Cst<R>> T,
    const __grid_constant__ TempoConsts<Cst<R>> cst, const __grid_constant__ IslandConsts<Isl<R>> ci) {
  const long npts = (long)b.pt_start[b.nd];
  __shared__ unsigned chunk;
  for (;;) {
    if (threadIdx.x == 0) chunk = atomicAdd(b.queue, (unsigned)blockDim.x);
    __syncthreads();
    const long q0 = (long)chunk;
    __syncthreads();
    if (q0 >= npts) return;
    const bool go = q0 + (long)blockDim.x <= npts;  // a full chunk takes the barriers
    const long q = q0 + threadIdx.x;
    if (q < npts) {
      long p = b.ord ? (long)b.ord[q] : q;
      if (p >= npts) p = npts - 1;  // never for an order built by the order kernel
      const BatchPoint bp = batch_point(b, p);
      const StepArgs<S>& a = b.dom[bp.d];
      points_point<R, S, V>(a, T, cst, ci, bp.k, bp.s, FwdIO<S>{a}, go);
    }
  }
}

template <class R, class S, int G, bool SPLIT, bool BLOCK>
__global__ void __launch_bounds__(128, sedim_min_blocks<R>()) tempo_sedim_batch_kernel(const __grid_constant__ BatchArgs<S> b) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)b.slot_start[b.nd]) return;
  const int d = domain_of(b.slot_start, b.nd, t);
  sedim_column<R, S, false, G, BLOCK>(b.dom[d], nullptr, nullptr, t - (long)b.slot_start[d],
                               SPLIT ? (int)blockIdx.y : -1);
}

template <class R, class S>
__global__ void __launch_bounds__(128, final_min_blocks<R>()) tempo_final_batch_kernel(
    const __grid_constant__ BatchArgs<S> b, const __grid_constant__ TempoConsts<Cst<R>> cst,
    const __grid_constant__ IslandConsts<Isl<R>> ci) {
  const long npts = (long)b.pt_start[b.nd];
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= npts) return;
  const long p = b.ord ? (long)b.ord[q] : q;
  if (p >= npts) return;
  const BatchPoint bp = batch_point(b, p);
  final_point<R, S>(b.dom[bp.d], cst, ci, bp.k, bp.s, FwdIO<S>{b.dom[bp.d]});
}

template <class R, class S, int V = 0>
void launch_sedim_batch(const BatchArgs<S>& b, int sv, unsigned gcol, cudaStream_t s) {
  if constexpr (V + 1 < kSedimVariants)
    if (sv != V) return launch_sedim_batch<R, S, V + 1>(b, sv, gcol, s);
  tempo_sedim_batch_kernel<R, S, sedim_group(V), sedim_split(V), sedim_blocked(V)>
      <<<dim3(gcol, sedim_split(V) ? 2 : 1), kBlock, 0, s>>>(b);
}

}  // namespace

cudaError_t launch_batch_mixed_f32(const BatchArgs<float>& b, const Tables<float>& T,
                                   const TempoConsts<float>& c, const IslandConsts<df>& ci,
                                   cudaStream_t s, const cudaEvent_t* ev, int sedim_variant) {
  if (b.ncol == 0) return cudaSuccess;
  constexpr int V = 7;  // the persistent lockstep variant of the points kernel
  const unsigned gcol = (unsigned)((b.ncol + kBlock - 1) / kBlock);
  if (ev) record_event(ev[0], s);
  tempo_prep_batch_kernel<float, float><<<gcol, kBlock, 0, s>>>(b, c, ci);
  tempo_batch_plan_kernel<float><<<1, 32, 0, s>>>(b);
  if (ev) record_event(ev[1], s);
  if (b.ord) {
    const unsigned greg = (unsigned)((b.npts_max + kRegimeWindow - 1) / kRegimeWindow);
    tempo_regime_order_batch_kernel<float><<<greg, kRegimeBlock, 0, s>>>(b);
  }
  if (ev) record_event(ev[2], s);
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tempo_points_batch_kernel<float, float, V>,
                                                      points_block(V), 0);
  if (e != cudaSuccess) return e;
  const unsigned gpts = (unsigned)((b.npts_max + points_block(V) - 1) / points_block(V));
  const unsigned gp = std::min<unsigned>(gpts, (unsigned)(std::max(per_sm, 1) * sms));
  tempo_points_batch_kernel<float, float, V><<<gp, points_block(V), 0, s>>>(b, T, c, ci);
  if (ev) record_event(ev[3], s);
  launch_sedim_batch<float, float>(b, sedim_variant, gcol, s);
  if (ev) record_event(ev[4], s);
  const unsigned gfin = (unsigned)((b.npts_max + kBlock - 1) / kBlock);
  tempo_final_batch_kernel<float, float><<<gfin, kBlock, 0, s>>>(b, c, ci);
  if (ev) record_event(ev[5], s);
  return cudaGetLastError();
}

}  // namespace tg
