// tempo_step.cuh -- the TEMPO column step (tempo_run -> tempo_main) as four sm_103a
// kernels.
//
//   prep    one thread per column.  The early-exit test of tempo_main (main:417-418:
//           no hydrometeor and no ice supersaturation anywhere in the column) and the
//           first-step graupel test; early-exit columns are finished here (initial
//           checks only).  Active columns are compacted into slots with one
//           warp-aggregated atomic, so later kernels touch no dry column.
//   points  one thread per (level, active slot): phase A of tempo_main (main:321-588),
//           pointwise physics -- initial checks, process rates, limiter, tendency
//           sums, provisional update, saturation adjustment, rain evaporation -- and
//           each species' fall-speed candidate.
//   sedim   one thread per active slot: phase B (main:593-727), the vertically
//           coupled part -- fall-speed fill from above, CFL substep counts, and the
//           explicit upwind sedimentation sweeps with their precipitation sums.
//   final   one thread per (level, active slot): phase C (main:731-863) -- instant
//           freeze/melt, final update and checks, diagnostics -- and, on the lowest
//           level, the column diagnostics.
//
// Host arrays keep the host model's (ims:ime, kms:kme, jms:jme) layout, i fastest.
// Threads of a warp take consecutive active slots at one level; slots follow column
// order within each warp of prep, so field accesses stay coalesced.  Scratch is
// [field][level][slot], slot fastest.  Template parameters: R the bulk arithmetic
// (double: FP64 drop-in; float: mixed form with double-float islands), S the storage.
#pragma once

#include <type_traits>

#include "tempo_rates.cuh"

namespace tg {

template <class I, class S> __device__ __forceinline__ I ldi(const S* p) { return I(*p); }

// Forward I/O policy: a point reads the step's arrays and stores its outputs where the
// step keeps them.  The derivative kernels substitute policies that seed input
// directions and contract outputs with their adjoints.
template <class S>
struct FwdIO {
  const StepArgs<S>& a;
  template <class R, class X> __device__ __forceinline__ R in(const X& v, int) const { return R(v); }
  template <class V> __device__ __forceinline__ void arr(int id, long e, const V& v) const {
    S* p = id == A_T ? a.t : id == A_QV ? a.qv : id == A_QC ? a.qc : id == A_NC ? a.nc
         : id == A_QR ? a.qr : id == A_NR ? a.nr : id == A_QI ? a.qi : id == A_NI ? a.ni
         : id == A_QS ? a.qs : id == A_QG ? a.qg : id == A_NG ? a.ng : id == A_QB ? a.qb
         : id == A_NWFA ? a.nwfa : a.nifa;
    p[e] = S(v);
  }
  template <class V> __device__ __forceinline__ void th(long e, const V& v) const { a.th[e] = S(v); }
  // scratch read of element type E as type O (seeded direction id in derivative policies)
  template <class O, class E> __device__ __forceinline__ O sdin(long idx, int) const {
    return O(reinterpret_cast<const E*>(a.sd)[idx]);
  }
  template <class E> __device__ __forceinline__ E scin(long idx) const {
    return reinterpret_cast<const E*>(a.sc)[idx];
  }
  template <class X> __device__ __forceinline__ void sd(X* base, long idx, const X& v) const { base[idx] = v; }
  // the sedimenting fields and their tendencies: scratch planes (island-type slots) that
  // hold values of the bulk type R, in the first sizeof(R) / sizeof(I) of each plane
  template <class I, class R> __device__ __forceinline__ void sx(long fsd, int f, long o, const R& v) const {
    reinterpret_cast<R*>(reinterpret_cast<I*>(a.sd) + (long)f * fsd)[o] = v;
  }
  template <class R, class I> __device__ __forceinline__ R sxin(long fsd, int f, long o, int) const {
    return reinterpret_cast<const R*>(reinterpret_cast<const I*>(a.sd) + (long)f * fsd)[o];
  }
  template <class X> __device__ __forceinline__ void sr(X* base, long idx, const X& v) const { base[idx] = v; }
  __device__ __forceinline__ void pmask(long o, uint8_t m) const { a.pmask[o] = m; }
  template <class V> __device__ __forceinline__ void diag3(S* p, long e3, const V& v) const {
    if (p) p[e3] = S(v);
  }
  template <class V> __device__ __forceinline__ void diag2(S* p, long t2, const V& v) const {
    if (p) p[t2] = S(v);
  }
  static constexpr bool forward = true;
};

// a barrier of the block when B (the lockstep variants of the points kernel) and go
// (the same for every thread of the block)
template <bool B>
__device__ __forceinline__ void block_sync(bool go) {
  if constexpr (B)
    if (go) __syncthreads();
}

// the time step in the bulk type, its reciprocal, and the time step in the island type
// (host-computed, so that no kernel of the mixed form converts or divides in FP64)
template <class R, class S> __device__ __forceinline__ R step_dt(const StepArgs<S>& a) {
  if constexpr (std::is_same<Cst<R>, double>::value) return R(a.dt); else return R(a.dt_hi);
}
template <class R, class S> __device__ __forceinline__ R step_odt(const StepArgs<S>& a) {
  if constexpr (std::is_same<Cst<R>, double>::value) return R(a.odt); else return R(a.odt_f);
}
template <class R, class S> __device__ __forceinline__ Isl<R> step_dti(const StepArgs<S>& a) {
  if constexpr (std::is_same<Isl<R>, df>::value) return df(a.dt_hi, a.dt_lo);
  else if constexpr (std::is_same<Cst<R>, double>::value) return Isl<R>(a.dt);
  else return Isl<R>(a.dt_hi);
}

// geometry of column c of the tile
struct ColGeom {
  long base;   // memory offset of (its+ii, kts, jts+jj)
  long tile2;  // offset in 2-D tile diagnostics
  int ii, jj;
};
template <class S>
__device__ __forceinline__ ColGeom col_geom(const StepArgs<S>& a, long c) {
  ColGeom g;
  g.ii = (int)(c % a.ti);
  g.jj = (int)(c / a.ti);
  g.base = (long)(a.i0 + g.ii) + (long)a.k0 * a.NI + (long)(a.j0 + g.jj) * a.NI * a.NK;
  g.tile2 = (long)g.ii + (long)g.jj * a.ti;
  return g;
}
template <class S>
__device__ __forceinline__ long tile3_of(const StepArgs<S>& a, const ColGeom& g, int k) {
  return (long)g.ii + (long)k * a.ti + (long)g.jj * a.ti * a.nz;
}

// ncsave: single-moment cloud number when nc is absent (main:364-380)
template <class R, class S>
__device__ __forceinline__ R ncsave_of(const StepArgs<S>& a, const ColGeom& g) {
  if (a.flags & F_NC) return R(nt_c_l);
  if (a.flags & F_LAND)
    return (a.land[(long)(a.i0 + g.ii) + (long)(a.j0 + g.jj) * a.NI] != 1) ? R(nt_c_o) : R(nt_c_l);
  return R(a.nc_single);
}

template <class R, class S, class IO>
__device__ __forceinline__ void load_level(const StepArgs<S>& a, long e, Lev<R>& L, const IO& io) {
  using I = Isl<R>;
  const uint32_t f = a.flags;
  L.t1d = (f & F_USE_T) ? io.template in<I>(a.t[e], IN_T)
                        : io.template in<I>(a.th[e], IN_T) * ldi<I>(a.pii + e);
  L.qv1d = io.template in<I>(a.qv[e], IN_QV);
  L.pres = R(a.p[e]);
  L.qc1d = io.template in<R>(a.qc[e], IN_QC);
  L.qr1d = io.template in<R>(a.qr[e], IN_QR);
  L.qi1d = io.template in<R>(a.qi[e], IN_QI);
  L.qs1d = io.template in<R>(a.qs[e], IN_QS);
  L.qg1d = io.template in<R>(a.qg[e], IN_QG);
  L.ni1d = io.template in<R>(a.ni[e], IN_NI);
  L.nr1d = io.template in<R>(a.nr[e], IN_NR);
  L.nc1d = (f & F_NC) ? io.template in<R>(a.nc[e], IN_NC) : R(0);
  L.ng1d = (f & F_HAIL) ? io.template in<R>(a.ng[e], IN_NG) : R(0);
  L.qb1d = (f & F_HAIL) ? io.template in<R>(a.qb[e], IN_QB) : R(0);
  L.temp = L.t1d;
  L.qv = Max(I(min_qv), L.qv1d);
  L.rho = rho_of(*L.ci, I(L.pres), L.temp, L.qv);
  L.qvs_t0 = calc_rslf(I(L.pres), I(t0));
  L.tten = L.qvten = I(0.0);
  L.qcten = L.ncten = L.qiten = L.niten = L.qrten = L.nrten = L.qsten = L.qgten = L.ngten =
      L.qbten = L.nwfaten = L.nifaten = R(0);
  L.smob = L.smoc = L.smo0 = L.smo1 = L.smo2 = L.smoe = L.smof = L.smog = L.smoz = R(0);
  L.vtboost = R(1);
}

// initial checks (main:347-396)
// cloud number (kg^-1) of the ML path (ml:104-176): input scaler, two dense layers with
// ReLU, the exponent clamped to [-6, log10(2e9)], the reference's bias correction and
// 10**x; weights from the host (kMlNet values)
template <class R>
__device__ R ml_cloud_number(const double* net, R qc, R qr, R qi, R qs, R pres, R temp, R w) {
  const double *mean = net, *var = net + 7, *w00 = net + 14, *b00 = net + 182, *w01 = net + 206,
               *b01 = net + 230;
  const R in[7] = {qc, qr, qi, qs, pres, temp, w};
  R x[7];
TG_UNROLL
  for (int j = 0; j < 7; j++) x[j] = (in[j] - R(mean[j])) / Sqrt(R(var[j]));
  R acc1 = R(0.0);
  for (int i = 0; i < 24; i++) {
    R acc = R(0.0);
TG_UNROLL
    for (int j = 0; j < 7; j++) acc = acc + R(w00[j * 24 + i]) * x[j];
    acc = Max(acc + R(b00[i]), R(0.0));
    acc1 = acc1 + R(w01[i]) * acc;
  }
  const R out = Max(acc1 + R(b01[0]), R(0.0));
  const R pe = Min(R(9.3010299957), Max(R(-6.0), out));
  R corr = R(1.0);
  if (pe >= R(0.0) && pe < R(3.0)) {
    const R p2 = pe * pe, p4 = p2 * p2;  // integer powers by binary powering
    corr = R(-0.2704) * (pe * p4) + R(1.838) * p4 - R(5.127) * (pe * p2) + R(8.547) * p2 -
           R(8.439) * pe + R(4.297);
  }
  return corr * Pow10(pe);
}

// The initial checks of the level (main:346-396).  With F_MLNC the single-moment cloud
// number comes from the network (main:364-371) and is returned in ncsave.
template <class R>
__device__ __forceinline__ void initial_checks(Lev<R>& L, uint32_t f, R& ncsave, bool do_ginit, R dt,
                                               R odt, const double* mlnet = nullptr, R w = R(0)) {
  using I = Isl<R>;
  TG_TRACE_PASS(L, 0);
  rain_check(L, L.qr1d, L.nr1d, dt, odt);
  ice_check(L, L.qi1d, L.ni1d, dt, odt);
  snow_check(L, L.qs1d, dt, odt);
  if (L.l_qs) snow_moments(L, R(Min(I(-0.1), L.temp - t0)), 1);
  if ((f & F_MLNC) && mlnet) {
    const R xq = L.qc1d <= R(1.e-12) ? R(0.0) : L.qc1d;
    ncsave = ml_cloud_number(mlnet, xq, L.qr1d, L.qi1d, L.qs1d, R(L.pres), R(L.temp), w) * R(L.rho);
  }
  if (!(f & F_NC)) L.nc = ncsave;
  cloud_check(L, L.qc1d, L.nc1d, (f & F_NC) != 0, ncsave, dt, odt);
  if (do_ginit) graupel_init(L);
  graupel_check(L, L.qg1d, L.ng1d, L.qb1d, (f & F_HAIL) != 0, dt, odt);
}

template <class R, class S, class IO>
__device__ __forceinline__ void store_checked(const StepArgs<S>& a, long e, const Lev<R>& L,
                                              const IO& io) {
  io.arr(A_QC, e, L.qc1d);
  io.arr(A_QR, e, L.qr1d);
  io.arr(A_NR, e, L.nr1d);
  io.arr(A_QI, e, L.qi1d);
  io.arr(A_NI, e, L.ni1d);
  io.arr(A_QS, e, L.qs1d);
  io.arr(A_QG, e, L.qg1d);
  if (a.flags & F_NC) io.arr(A_NC, e, L.nc1d);
  if (a.flags & F_HAIL) {
    io.arr(A_NG, e, L.ng1d);
    io.arr(A_QB, e, L.qb1d);
  }
}

// ---------------------------------------------------------------------------------
// prep: early-exit test, early columns, compaction
// ---------------------------------------------------------------------------------
// Prep of column c of a's tile (valid: c < a.ncol).  Every lane of the warp calls it;
// lanes with the same `group` (the domain of a multi-domain batch; 0 for one tile) take
// their slots with one atomic on their tile's counter.
template <class R, class S>
__device__ __forceinline__ void prep_column(const StepArgs<S>& a, const TempoConsts<Cst<R>>& cst,
                                            const IslandConsts<Isl<R>>& ci, long c, bool valid,
                                            int group) {
  using I = Isl<R>;
  const uint32_t f = a.flags;
  const int nz = a.nz;
  const bool hail = f & F_HAIL;
  const R dt = step_dt<R>(a), odt = step_odt<R>(a);
  ColGeom g = {};
  bool early = true, do_ginit = false;
  if (valid) {
    g = col_geom(a, c);
    bool do_micro = false, supersat = false;
    I sqg = I(0.0), sng = I(0.0), sqb = I(0.0);
    for (int k = 0; k < nz; k++) {
      const long e = g.base + (long)k * a.NI;
      I t1 = (f & F_USE_T) ? ldi<I>(a.t + e) : ldi<I>(a.th + e) * ldi<I>(a.pii + e);
      I qv = Max(I(min_qv), ldi<I>(a.qv + e));
      I p = ldi<I>(a.p + e);
      do_micro |= (ldi<I>(a.qc + e) > r1) | (ldi<I>(a.qr + e) > r1) | (ldi<I>(a.qi + e) > r1) |
                  (ldi<I>(a.qs + e) > r1) | (ldi<I>(a.qg + e) > r1);
      I qvsi = (t1 - t0 <= 0.0) ? calc_rsif(p, t1) : calc_rslf(p, t1);
      I ssati = qv / qvsi - 1.0;
      if (Fabs(ssati) < eps) ssati = I(0.0);
      supersat |= ssati > 0.0;
      if (hail && (f & F_FIRST)) {
        sqg = sqg + ldi<I>(a.qg + e);
        sng = sng + ldi<I>(a.ng + e);
        sqb = sqb + ldi<I>(a.qb + e);
      } else if (do_micro || supersat) {
        break;  // the column is active whatever the levels above hold
      }
    }
    do_ginit = hail && (f & F_FIRST) && sqg > r1 && sng < eps && sqb < eps;
    early = !do_micro && !supersat;
  }

  // compaction: one atomic per warp (per group of the warp), slots in lane order
  const bool active = valid && !early;
  const unsigned lanes = __ballot_sync(0xffffffffu, active) & __match_any_sync(0xffffffffu, group);
  const int lane = threadIdx.x & 31;
  unsigned first = 0;
  const int leader = lanes ? __ffs(lanes) - 1 : lane;
  if (lanes && lane == leader) first = atomicAdd(a.nact, (unsigned)__popc(lanes));
  first = __shfl_sync(0xffffffffu, first, leader);
  if (!valid) return;
  if (active) {
    const long s = first + __popc(lanes & ((1u << lane) - 1u));
    a.act[s] = (int)c;
    a.cmask[s] = do_ginit ? CM_GINIT : 0;
    if (a.mhd_col) a.mhd_col[g.tile2] = S(0);
    if (!(f & F_NWFA) || !(f & F_NIFA)) {
      // heights for the aerosol initial profiles (init_*_friendly_aerosols,
      // aerosols:14-73): hgt(1) = 0, and level 1 takes hgt(2)
      Cst<R>* hgt = reinterpret_cast<Cst<R>*>(a.hgt) + pt_base(s, nz);
      I h = I(0.0);
      for (int k = 1; k < nz; k++) {
        h = h + ldi<I>(a.dz + g.base + (long)k * a.NI);
        hgt[(long)k * kSlotTile] = Cst<R>(h);
      }
      hgt[0] = (nz > 1) ? Cst<R>(ldi<I>(a.dz + g.base + a.NI)) : Cst<R>(0.0);
    }
    return;
  }

  // early exit: initial checks only, default diagnostics
  for (int k = 0; k < nz; k++) {
    const long e = g.base + (long)k * a.NI;
    Lev<R> L;
    L.cs = &cst;
    L.ci = &ci;
#ifdef TEMPO_TRACE
    L.tr = a.trace ? a.trace + (c * nz + k) * kTracePoint : nullptr;
#endif
    const FwdIO<S> io{a};
    load_level(a, e, L, io);
    R ncsave = ncsave_of<R>(a, g);
    initial_checks(L, f, ncsave, do_ginit, dt, odt, a.mlnet, R(a.w[e]));
    store_checked(a, e, L, io);
  }
  const long t2 = g.tile2;
  if (a.rain_precip) a.rain_precip[t2] = S(0);
  if (a.ice_precip) a.ice_precip[t2] = S(0);
  if (a.snow_precip) a.snow_precip[t2] = S(0);
  if (a.graupel_precip) a.graupel_precip[t2] = S(0);
  if (a.frozen_fraction) a.frozen_fraction[t2] = S(0);
  if (a.frz_rain) a.frz_rain[t2] = S(0);
  if (a.mhd_sfc) a.mhd_sfc[t2] = S(0);
  if (a.mhd_col) a.mhd_col[t2] = S(0);
  for (int k = 0; k < nz; k++) {
    const long e3 = tile3_of(a, g, k);
    if (a.refl10cm) a.refl10cm[e3] = S(-35.0);
    if (a.re_cloud) a.re_cloud[e3] = S(0);
    if (a.re_ice) a.re_ice[e3] = S(0);
    if (a.re_snow) a.re_snow[e3] = S(0);
    if (a.mvd_r) a.mvd_r[e3] = S(0);
    if (a.mvd_g) a.mvd_g[e3] = S(0);
    if (a.ncmr) a.ncmr[e3] = S(0);
  }
  atomicAdd(a.stats, 1ull);
}

template <class R, class S>
__global__ void __launch_bounds__(128) tempo_prep_kernel(const __grid_constant__ StepArgs<S> a,
                                                          const __grid_constant__ TempoConsts<Cst<R>> cst,
                                                          const __grid_constant__ IslandConsts<Isl<R>> ci) {
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  prep_column<R, S>(a, cst, ci, c, c < a.ncol, 0);
}

// ---------------------------------------------------------------------------------
// regime order of phase A's points
// ---------------------------------------------------------------------------------
// Phase A's work at a point depends on which species are present and on the side of
// 0 C (ice nucleation, deposition and riming below it, melting above).  In level-major
// order a warp's 32 points mix clear air with cloud.  Inside each window of W
// consecutive level-major points, the points are grouped by regime (the regimes with
// more species first), so that a warp's points take the same branches.  Keeping the
// grouping inside a window keeps the writes of phase A to a window's scratch sectors
// close together in time (a global grouping scatters them over the whole step and
// costs partial-sector writes).  The order decides only which thread computes a
// point, never its value.
// windows of 32 768 points (measured at 1 M columns, points kernel variant 7: 36.8 ms
// against 37.5 ms with windows of 16 384, 38.4 ms with 8 192 and 39.6 ms with 4 096;
// the order kernel then takes 0.76 ms)
constexpr int kRegimeBlock = 1024, kRegimeItems = 32;
constexpr int kRegimeWindow = kRegimeBlock * kRegimeItems;  // 32768 points

// bits 1-5: cloud, rain, ice, snow, graupel present (> r1) in the input state; bit 0:
// below 0 C.  Compared in FP32: the regime only groups points.
template <class S>
__device__ __forceinline__ int point_regime(const StepArgs<S>& a, long e) {
  const float t = (a.flags & F_USE_T) ? float(a.t[e]) : float(a.th[e]) * float(a.pii[e]);
  constexpr float q1 = float(r1);
  return (t < float(t0) ? 1 : 0) | (float(a.qc[e]) > q1 ? 2 : 0) | (float(a.qr[e]) > q1 ? 4 : 0) |
         (float(a.qi[e]) > q1 ? 8 : 0) | (float(a.qs[e]) > q1 ? 16 : 0) |
         (float(a.qg[e]) > q1 ? 32 : 0);
}

// one block per window: the regime of each of its points, then their positions in the
// window (regime by regime from regime 63 down; inside a regime, warp w's points after
// those of the warps below w, each warp's in the order of its items and lanes)
// The body of one block: window q0 of npts points, regime_of(q) the regime of point q,
// ord the output.
template <class RegimeOf>
__device__ __forceinline__ void regime_order_window(long q0, long npts, RegimeOf regime_of, unsigned* ord) {
  constexpr int kWarps = kRegimeBlock / 32;
  __shared__ unsigned wcnt[kWarps][kRegimes];  // per warp: count, then offset in the window
  __shared__ unsigned start[kRegimes];         // first position of a regime in the window
  __shared__ unsigned wtot;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < kWarps * kRegimes; i += kRegimeBlock) (&wcnt[0][0])[i] = 0;
  __syncthreads();
  int reg[kRegimeItems];
  unsigned rank[kRegimeItems];
  // the regimes first (independent loads), then the ranks
#pragma unroll
  for (int j = 0; j < kRegimeItems; j++) {
    const long q = q0 + (long)j * kRegimeBlock + threadIdx.x;
    reg[j] = q < npts ? regime_of(q) : -1;
  }
#pragma unroll
  for (int j = 0; j < kRegimeItems; j++) {
    const int r = reg[j];
    const unsigned m = __match_any_sync(0xffffffffu, r);
    const unsigned before = r >= 0 ? wcnt[wid][r] : 0u;
    __syncwarp();
    if (r >= 0 && lane == __ffs(m) - 1) wcnt[wid][r] = before + (unsigned)__popc(m);
    __syncwarp();
    rank[j] = before + (unsigned)__popc(m & ((1u << lane) - 1u));
  }
  __syncthreads();
  // threads 0-63 (two warps), thread t for regime i = 63 - t: per-warp offsets, the
  // regime's count in the window, and the sum of the counts of the regimes above i (a
  // shuffle scan per warp; the second warp adds the first warp's total below)
  if (threadIdx.x < kRegimes) {
    const int t = threadIdx.x, i = kRegimes - 1 - t;
    unsigned tot = 0;
#pragma unroll
    for (int w = 0; w < kWarps; w++) {
      const unsigned n = wcnt[w][i];
      wcnt[w][i] = tot;
      tot += n;
    }
    unsigned inc = tot;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned v = __shfl_up_sync(0xffffffffu, inc, d);
      if (lane >= d) inc += v;
    }
    if (t == 31) wtot = inc;
    start[i] = inc - tot;
  }
  __syncthreads();
  if (threadIdx.x >= 32 && threadIdx.x < kRegimes) start[kRegimes - 1 - threadIdx.x] += wtot;
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kRegimeItems; j++)
    if (reg[j] >= 0) {
      const long pos = q0 + (long)(start[reg[j]] + wcnt[wid][reg[j]] + rank[j]);
      if (pos < npts) ord[pos] = (unsigned)(q0 + (long)j * kRegimeBlock + threadIdx.x);
    }
}

template <class S>
__global__ void __launch_bounds__(kRegimeBlock) tempo_regime_order_kernel(const __grid_constant__ StepArgs<S> a) {
  const long nact = (long)*a.nact, npts = nact * a.nz;
  const long q0 = (long)blockIdx.x * kRegimeWindow;
  if (q0 >= npts) return;
  regime_order_window(q0, npts, [&](long q) {
    const int k = (int)(q / nact);
    const long s = q - (long)k * nact;
    return point_regime(a, col_geom(a, a.act[s]).base + (long)k * a.NI);
  }, a.ord);
}

// One stage of phase A, each followed by thermo_vars in the caller: 0 = process
// rates, limiter, tendency sums, provisional update and checks on temporaries
// (main:420-522); 1 = saturation adjustment (main:530-560); 2 = rain evaporation
// (main:563-588).
// With kSync and go, a block barrier follows each process group of stage 0 (all
// threads of the block call the stage).
template <class R, bool kSync = false>
__device__ __forceinline__ void points_stage(int stage, Lev<R>& L, Tend<R>& td, const Tables<Cst<R>>& T,
                                             const IslandConsts<Isl<R>>& ci, uint32_t f, R w, R dt,
                                             R odt, Isl<R> dti, R ncsave, R ncsave_cond, R nwfa_in,
                                             R nifa_in, bool go = false) {
  using I = Isl<R>;
  const bool has_nc = f & F_NC, has_nwfa = f & F_NWFA, has_nifa = f & F_NIFA, hail = f & F_HAIL;
  if (stage == 0) {
    if (!(f & F_NOMICRO)) {
      warm_rain(L, td, T, odt);
      block_sync<kSync>(go);
      rain_snow_rain_graupel(L, td, T, odt);
      block_sync<kSync>(go);
      ice_nucleation(L, td, T, w, f, dt, odt);
      block_sync<kSync>(go);
      const R t1s = t1_subl_of(L);
      ice_processes(L, td, T, w, t1s, odt);
      block_sync<kSync>(go);
      riming(L, td, T, odt);
      block_sync<kSync>(go);
      melting(L, td, t1s, f, dt, odt);
      if (has_nwfa || has_nifa) aerosol_scavenging(L, td, odt);
      block_sync<kSync>(go);
      L.psd_have = 0;
      L.rain_idx = 0;
    }
    check_over_depletion(L, td, odt);
    sum_tendencies(L, td);

    // provisional update (main:460-468)
    L.temp = L.t1d + L.tten * dti;
    L.qv = Max(I(min_qv), L.qv1d + L.qvten * dti);
    L.rho = rho_of(ci, I(L.pres), L.temp, L.qv);
    {
      R rho = R(L.rho);
      L.nwfaten = L.nwfaten - (td.pna_rca + td.pna_sca + td.pna_gca + td.pni_iha) / rho;
      L.nifaten = L.nifaten - (td.pnd_rcd + td.pnd_scd + td.pnd_gcd) / rho;
    }
    if (has_nwfa) L.nwfa = nwfa_in;
    if (has_nifa) L.nifa = nifa_in;
    aerosol_check(L, f, dt);

    // checks on temporaries (main:475-522)
    TG_TRACE_PASS(L, 1);
    R xq = L.qc1d, xn = L.nc1d, xb;
    cloud_check(L, xq, xn, has_nc, ncsave, dt, odt);
    xq = L.qr1d;
    xn = L.nr1d;
    rain_check(L, xq, xn, dt, odt);
    xq = L.qi1d;
    xn = L.ni1d;
    ice_check(L, xq, xn, dt, odt);
    xq = L.qs1d;
    snow_check(L, xq, dt, odt);
    L.smo0 = L.smo1 = L.smo2 = L.smob = L.smoc = L.smoe = L.smof = L.smog = R(0);
    if (L.l_qs) snow_moments(L, R(Min(I(-0.1), L.temp - t0)), 0);
    xq = L.qg1d;
    xn = L.ng1d;
    xb = L.qb1d;
    graupel_check(L, xq, xn, xb, hail, dt, odt);
  } else if (stage == 1) {
    cloud_condensation(L, td, T, w, f, ncsave_cond, dt, odt);
    L.qvten = L.qvten - I(td.prw_vcd);
    L.qcten = L.qcten + td.prw_vcd;
    L.ncten = L.ncten + td.pnc_wcd;
    L.qcmag = L.qcmag + mag(td.prw_vcd);
    L.ncmag = L.ncmag + mag(td.pnc_wcd);
    TG_TRACE_PASS(L, 2);
    L.nwfaten = L.nwfaten - td.pnc_wcd;
    L.tten = L.tten + I(L.lvap) * L.ocp * td.prw_vcd;
    R xq = L.qc1d, xn = L.nc1d;
    cloud_check(L, xq, xn, has_nc, ncsave, dt, odt);
    L.qv = Max(I(min_qv), L.qv1d + L.qvten * dti);
    L.temp = L.t1d + L.tten * dti;
    L.rho = rho_of(ci, I(L.pres), L.temp, L.qv);
  } else {
    rain_evaporation(L, td, odt);
    L.qrten = L.qrten - td.prv_rev;
    L.qvten = L.qvten + I(td.prv_rev);
    L.nrten = L.nrten - td.pnr_rev;
    L.qrmag = L.qrmag + mag(td.prv_rev);
    L.nrmag = L.nrmag + mag(td.pnr_rev);
    TG_TRACE_PASS(L, 3);
    L.nwfaten = L.nwfaten + td.pnr_rev;
    L.tten = L.tten - I(L.lvap) * L.ocp * td.prv_rev;
    R xq = L.qr1d, xn = L.nr1d;
    rain_check(L, xq, xn, dt, odt);
    L.qv = Max(I(min_qv), L.qv1d + L.qvten * dti);
    L.temp = L.t1d + L.tten * dti;
    L.rho = rho_of(ci, I(L.pres), L.temp, L.qv);
  }
}

// Variants of the points kernel (picked per context by tempo_autotune_c).  Bit 0 = 0:
// blocks of 128 threads, bits 1-2 select the minimum resident blocks per SM asked of
// the register allocator (1, 3, 4 or 5: no cap, 170, 128 or 102 registers per thread).
// Bit 0 = 1 (lockstep): the warps of a block run the stages and the process groups of
// stage 0 between block barriers, so that an SM fetches each part of the kernel's code
// for all of its warps at once (a thread's path through phase A is a long run of code
// executed once, longer than the instruction cache); bits 1-2 select the block (128,
// 256, 512 or 512 threads) and the resident blocks per SM asked (4, 2, 1, 1: 128
// registers per thread).  Variant 7 is persistent: one block per SM takes chunks of
// 512 points from a device work queue (a counter after the active-slot count) until
// the points run out.
__host__ __device__ constexpr int points_block(int v) {
  return (v & 1) ? ((v >> 1) & 3) == 0 ? 128 : ((v >> 1) & 3) == 1 ? 256 : 512 : 128;
}
__host__ __device__ constexpr bool points_persistent(int v) { return v == 7; }
__host__ __device__ constexpr int points_min_blocks(int v) {
  return (v & 1) ? ((v >> 1) & 3) == 0 ? 4 : ((v >> 1) & 3) == 1 ? 2 : 1
                 : ((v >> 1) & 3) == 0 ? 1 : ((v >> 1) & 3) + 2;
}

// mass- and number-weighted fall speeds of rain at a level with rain (rain_fallspeed,
// main:1771-1774)
template <class R>
__device__ __forceinline__ void rain_speeds(const Lev<R>& L, const TempoConsts<Cst<R>>& cc, R& vt, R& vtn) {
  R lamr = R(1.0) / L.ilamr;
  vt = L.rhof * R(av_r) * cc.crg[5] * cc.org3 * PowCre<2>(lamr, cc.cre[2]) *
       PowCre<5, -1>(lamr + R(fv_r), -cc.cre[5]);
  vtn = L.rhof * R(av_r) * cc.crg[6] / cc.crg[11] * PowCre<11>(lamr, cc.cre[11]) *
        PowCre<6, -1>(lamr + R(fv_r), -cc.cre[6]);
}
// the same for graupel (graupel_fallspeed, main:1817-1833), density-dependent with qb
template <class R>
__device__ __forceinline__ void graupel_speeds(const Lev<R>& L, const TempoConsts<Cst<R>>& cc, uint32_t f,
                                               R& vt, R& vtn) {
  R afall, bfall;
  if (f & F_QB) {
    R dens_g = Max(rho_g<R>(1), Min(R(meters3_to_liters) * L.rg / L.rb, rho_g<R>(nrhg)));
    afall = R(a_coeff) * Pow((R(4.0) * dens_g * R(earth_gravity)) / (R(3.0) * R(L.rho)), R(b_coeff));
    afall = afall * Pow(L.visco, R(1.0) - R(2.0) * R(b_coeff));
    bfall = R(3.0) * R(b_coeff) - R(1.0);
  } else {
    afall = R(av_g_old);
    bfall = R(bv_g_old);
  }
  const int ig = L.idx_bg;
  R pb = Pow(L.ilamg, bfall);
  vt = L.rhof * afall * cc.cgg[ig - 1][5] * cc.ogg3 * pb;
  vtn = L.rhof * afall * cc.cgg[ig - 1][6] / cc.cgg[ig - 1][11] * pb;
}

// ---------------------------------------------------------------------------------
// points: phase A at one (level, active slot)
// ---------------------------------------------------------------------------------
// Phase A at point (level k, active slot s); outputs go through the I/O policy.  go:
// the block's barriers of the lockstep variants (V odd) are taken.
template <class R, class S, int V, class IO>
__device__ __forceinline__ void points_point(const StepArgs<S>& a, const Tables<Cst<R>>& T,
                                             const TempoConsts<Cst<R>>& cst,
                                             const IslandConsts<Isl<R>>& ci, int k, long s,
                                             const IO& io, bool go = false) {
  using I = Isl<R>;
  const int nz = a.nz;
  const long c = a.act[s];
  const ColGeom g = col_geom(a, c);
  const long e = g.base + (long)k * a.NI;
  const uint32_t f = a.flags;
  const bool has_nc = f & F_NC, has_nwfa = f & F_NWFA, has_nifa = f & F_NIFA;
  const R dt = step_dt<R>(a), odt = step_odt<R>(a);
  const I dti = step_dti<R>(a);
  R ncsave = ncsave_of<R>(a, g);  // per level with F_MLNC, set by the initial checks
  const bool do_ginit = a.cmask[s] & CM_GINIT;
  const long cs = a.ncol_pad, fsd = (long)nz * cs, o = pt_off(s, k, nz);
  I* sd = reinterpret_cast<I*>(a.sd);
  R* sr = reinterpret_cast<R*>(a.sr);

  Lev<R> L;
  L.cs = &cst;
  L.ci = &ci;
#ifdef TEMPO_TRACE
  L.tr = a.trace ? a.trace + ((long)c * nz + k) * kTracePoint : nullptr;
#endif
  load_level(a, e, L, io);
  const R w = R(a.w[e]);
  R nwfa_in, nifa_in;
  if (has_nwfa && has_nifa) {
    nwfa_in = R(a.nwfa[e]);
    nifa_in = R(a.nifa[e]);
  } else {
    const R hk = R(reinterpret_cast<const Cst<R>*>(a.hgt)[o]);
    nwfa_in = has_nwfa ? R(a.nwfa[e]) : R(naccn1) + R(naccn0) * Exp(-(hk / R(1000.0)) * R(a.niccn3));
    nifa_in = has_nifa ? R(a.nifa[e]) : R(nain1) + R(nain0) * Exp(-(hk / R(1000.0)) * R(a.niin3));
  }
  L.nwfa = nwfa_in;
  L.nifa = nifa_in;
  aerosol_check(L, f, dt);
  initial_checks(L, f, ncsave, do_ginit, dt, odt, a.mlnet, w);
  if constexpr (IO::forward && !IsDual<S>::value)
    if (f & F_MLNC) reinterpret_cast<R*>(a.ncw)[o] = ncsave;  // for phase C
  const R ncsave_cond = has_nc ? R(nt_c_l) : ncsave;
  L.qcten = L.qiten = L.qrten = L.qsten = L.qgten = L.ngten = L.qbten = L.niten = L.nrten =
      L.ncten = R(0);
  clear_mags(L);

  // thermo_vars runs after the initial checks and after each of the three stages
  // that follow (main:412, 524, 557, 585)
  Tend<R> td = {};
  const bool do_cond = !(f & F_NOMICRO) && (f & F_COND);
  const bool do_evap = !(f & F_NOMICRO);
  // Where no later reader needs them, the thermodynamic fields are not recomputed:
  // rain evaporation reads them only where rain exists (it returns at once otherwise),
  // and after the last stage only the fall speeds' rhof and visco are read
  // (thermo_tail).  The values read are the same as with every call made.  The
  // lockstep variants put a block barrier after each stage when go (do_cond and do_evap
  // are the same for every thread).
  constexpr bool kSync = (V & 1) != 0;
  block_sync<kSync>(go);
  thermo(L);
  points_stage<R, kSync>(0, L, td, T, ci, f, w, dt, odt, dti, ncsave, ncsave_cond, nwfa_in, nifa_in, go);
  if (do_cond) {
    thermo<R, false>(L);
    points_stage<R, kSync>(1, L, td, T, ci, f, w, dt, odt, dti, ncsave, ncsave_cond, nwfa_in, nifa_in, go);
    block_sync<kSync>(go);
  }
  if (do_evap) {
    if (L.l_qr)
      thermo<R, false>(L);
    else
      thermo_tail(L);
    points_stage<R, kSync>(2, L, td, T, ci, f, w, dt, odt, dti, ncsave, ncsave_cond, nwfa_in, nifa_in, go);
    block_sync<kSync>(go);
  }
  thermo_tail(L);

  // fall-speed candidates (main:1770-1977), unfilled; < 0 marks "absent"
  const TempoConsts<Cst<R>>& cc = cst;
  R vtr = R(-1), vtnr = R(-1), vtg = R(-1), vtng = R(-1), vsa = R(-1), vsb = R(0);
  R vti = R(-1), vtni = R(-1), vtc = R(0), vtnc = R(0);
  if (L.rr > R(r1)) rain_speeds(L, cc, vtr, vtnr);
  if (L.rg > R(r1)) graupel_speeds(L, cc, f, vtg, vtng);
  if (L.rs > R(r1)) {
    R xds = L.smoc / L.smob;
    R mrat = R(1.0) / xds;
    R ils1 = R(1.0) / (mrat * R(lam0) + R(fv_s));
    R ils2 = R(1.0) / (mrat * R(lam1) + R(fv_s));
    R mrmu = Pow(mrat, R(mu_s));
    R t1_vts = R(kap0) * cc.csg[3] * Pow(ils1, cc.cse[3]);
    R t2_vts = R(kap1) * mrmu * cc.csg[9] * Pow(ils2, cc.cse[9]);
    ils1 = R(1.0) / (mrat * R(lam0));
    ils2 = R(1.0) / (mrat * R(lam1));
    R t3_vts = R(kap0) * cc.csg[0] * Pow(ils1, cc.cse[0]);
    R t4_vts = R(kap1) * mrmu * cc.csg[6] * Pow(ils2, cc.cse[6]);
    R vts = L.rhof * R(av_s) * (t1_vts + t2_vts) / (t3_vts + t4_vts);
    if (td.prr_sml > R(0.0)) {
      // mixed with the rain speed at fill time, with rr after rain sedimentation
      // (snow_fallspeed is called after the rain sweeps updated rr in place, main:699)
      vsa = vts;
      vsb = R(1.0);
    } else {
      vsa = vts * L.vtboost;
      vsb = R(0);
    }
  }
  if (L.ri > R(r1)) {
    R pb = Pow(L.ilami, R(bv_i));
    vti = L.rhof * R(av_i) * cc.cig[2] * cc.oig2 * pb;
    vtni = L.rhof * R(av_i) * cc.cig[5] / cc.cig[6] * pb;
  }
  if (L.rc > R(r1) && w < R(0.1)) {
    int nu_c = get_nuc(L.nc);
    R pb = Pow(L.ilamc, R(bv_c));
    vtc = L.rhof * R(av_c) * cc.ccg[nu_c - 1][4] * cc.ocg2[nu_c - 1] * pb;
    vtnc = L.rhof * R(av_c) * cc.ccg[nu_c - 1][3] * cc.ocg1[nu_c - 1] * pb;
  }
  io.pmask(o, (L.l_qr ? PM_QR : 0) | (L.l_qg ? PM_QG : 0) | (L.l_qs ? PM_QS : 0) |
               (L.l_qi ? PM_QI : 0) | (L.l_qc ? PM_QC : 0));

  io.sd(sd, SD_TTEN * fsd + o, I(L.tten));
  io.sd(sd, SD_QV * fsd + o, I(L.qv));
  io.sd(sd, SD_RHO * fsd + o, I(L.rho));
  io.template sx<I>(fsd, SD_XRR, o, R(L.rr));
  io.template sx<I>(fsd, SD_XNR, o, R(L.nr));
  io.template sx<I>(fsd, SD_XRG, o, R(L.rg));
  io.template sx<I>(fsd, SD_XNG, o, R(L.ng));
  io.template sx<I>(fsd, SD_XRB, o, R(L.rb));
  io.template sx<I>(fsd, SD_XRS, o, R(L.rs));
  io.template sx<I>(fsd, SD_XRI, o, R(L.ri));
  io.template sx<I>(fsd, SD_XNI, o, R(L.ni));
  io.template sx<I>(fsd, SD_XRC, o, R(L.rc));
  io.template sx<I>(fsd, SD_XNC, o, R(L.nc));
  io.template sx<I>(fsd, SD_TQR, o, R(L.qrten));
  io.template sx<I>(fsd, SD_TNR, o, R(L.nrten));
  io.template sx<I>(fsd, SD_TQG, o, R(L.qgten));
  io.template sx<I>(fsd, SD_TNG, o, R(L.ngten));
  io.template sx<I>(fsd, SD_TQB, o, R(L.qbten));
  io.template sx<I>(fsd, SD_TQS, o, R(L.qsten));
  io.template sx<I>(fsd, SD_TQI, o, R(L.qiten));
  io.template sx<I>(fsd, SD_TNI, o, R(L.niten));
  io.template sx<I>(fsd, SD_TQC, o, R(L.qcten));
  io.template sx<I>(fsd, SD_TNC, o, R(L.ncten));
  if constexpr (std::is_same<I, df>::value) {
    // the mixed form's sedimentation multiplies by these instead of dividing per sweep
    const I odz = 1.0 / ldi<I>(a.dz + e);
    io.sd(sd, SD_ODZ * fsd + o, I(odz));
    io.sd(sd, SD_OZR * fsd + o, I(odz / L.rho));
  }
  io.sr(sr, SR_VTR * fsd + o, R(vtr));
  io.sr(sr, SR_VTNR * fsd + o, R(vtnr));
  io.sr(sr, SR_VTG * fsd + o, R(vtg));
  io.sr(sr, SR_VTNG * fsd + o, R(vtng));
  io.sr(sr, SR_VTSA * fsd + o, R(vsa));
  io.sr(sr, SR_VTSB * fsd + o, R(vsb));
  io.sr(sr, SR_VTI * fsd + o, R(vti));
  io.sr(sr, SR_VTNI * fsd + o, R(vtni));
  io.sr(sr, SR_VTC * fsd + o, R(vtc));
  io.sr(sr, SR_VTNC * fsd + o, R(vtnc));

  // outputs final after phase A: checked prognostics, qv, aerosols (main:738-748)
  store_checked(a, e, L, io);
  io.arr(A_QV, e, Max(I(min_qv), (L.qv1d + L.qvten * dti)));
  if (has_nwfa) io.arr(A_NWFA, e, Max(R(nwfa_default), Min(R(aero_max), (nwfa_in + L.nwfaten * dt))));
  if (has_nifa) io.arr(A_NIFA, e, Max(R(nifa_default), Min(R(aero_max), (nifa_in + L.nifaten * dt))));
}

template <class R, class S, int V>
__global__ void __launch_bounds__(points_block(V), points_min_blocks(V)) tempo_points_kernel(const __grid_constant__ StepArgs<S> a,
                                                            const __grid_constant__ Tables<Cst<R>> T,
                                                            const __grid_constant__ TempoConsts<Cst<R>> cst,
                                                            const __grid_constant__ IslandConsts<Isl<R>> ci) {
  const long nact = (long)*a.nact, npts = nact * a.nz;
  if constexpr (points_persistent(V)) {
    // work queue: a.nact[1] (zero before the step) counts the points handed out
    __shared__ unsigned chunk;
    for (;;) {
      if (threadIdx.x == 0) chunk = atomicAdd(a.nact + 1, (unsigned)blockDim.x);
      __syncthreads();
      const long q0 = (long)chunk;
      __syncthreads();
      if (q0 >= npts) return;
      const bool go = q0 + (long)blockDim.x <= npts;  // a full chunk takes the barriers
      const long q = q0 + threadIdx.x;
      if (q < npts) {
        long p = a.ord ? (long)a.ord[q] : q;
        if (p >= npts) p = npts - 1;  // never for an order built by tempo_regime_order_kernel
        const int k = (int)(p / nact);
        points_point<R, S, V>(a, T, cst, ci, k, p - (long)k * nact, FwdIO<S>{a}, go);
      }
    }
  } else {
    const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
    // lockstep variants: a block whose threads all have points takes the barriers; the
    // last, partial block runs without them (its threads past the points return)
    const bool go = (V & 1) && (long)(blockIdx.x + 1) * blockDim.x <= npts;
    if (q >= npts) return;  // (never in a block with go)
    long p = a.ord ? (long)a.ord[q] : q;  // level-major index of the point
    if (p >= npts) {  // never for an order built by tempo_regime_order_kernel
      if (!go) return;
      p = npts - 1;
    }
    const int k = (int)(p / nact);
    points_point<R, S, V>(a, T, cst, ci, k, p - (long)k * nact, FwdIO<S>{a}, go);
  }
}

// ---------------------------------------------------------------------------------
// sedim: phase B for one active column
// ---------------------------------------------------------------------------------
// semilagrangian_sedimentation (main:1562-1749), the scheme of Juang and Hong (2010),
// Mon. Wea. Rev. 138, 1778-1791, on one column: x and ten are level planes of the bulk
// type (stride ls; the substep runs in the island type and stores its results), vt the
// filled speeds (vt(nz + 1) = 0), w the column's work rows (row stride wr, level stride
// wl).  Indices below are the reference's, 1-based.
template <class R, class I, class S>
__device__ void sl_sweep(int nz, R* x, R* ten, const R* vt, long ls, const S* dzp, long NI,
                         const I* rho, I* w, long wr, long wl, int steps, double limit, I* precip,
                         I dt, I odt) {
  auto row = [&](int r, int i) -> I& { return w[(long)r * wr + (long)(i - 1) * wl]; };
  auto ZI = [&](int i) -> I& { return row(0, i); };
  auto WI = [&](int i) -> I& { return row(1, i); };
  auto ZA = [&](int i) -> I& { return row(2, i); };
  auto DZA = [&](int i) -> I& { return row(3, i); };
  auto QA = [&](int i) -> I& { return row(4, i); };
  auto QMI = [&](int i) -> I& { return row(5, i); };
  auto QPI = [&](int i) -> I& { return row(6, i); };
  auto X0 = [&](int i) -> I& { return row(7, i); };
  auto VT = [&](int i) -> I { return i <= nz ? I(vt[(long)(i - 1) * ls]) : I(0.0); };
  auto DZ = [&](int i) -> I { return ldi<I>(dzp + (long)(i - 1) * NI); };
  const I osteps = 1.0 / I(steps), fsteps = I(steps);
  for (int k = 1; k <= nz; k++) X0(k) = I(x[(long)(k - 1) * ls]);
  ZI(1) = I(0.0);
  for (int k = 1; k <= nz; k++) ZI(k + 1) = ZI(k) + DZ(k);
  // 3rd-order interpolation of the interface speeds (:1599-1611)
  const I fa1 = I(9.0 / 16.0), fa2 = I(1.0 / 16.0);
  WI(1) = VT(1);
  WI(2) = 0.5 * (VT(2) + VT(1));
  for (int k = 3; k <= nz - 1; k++) WI(k) = fa1 * (VT(k) + VT(k - 1)) - fa2 * (VT(k + 1) + VT(k - 2));
  WI(nz) = 0.5 * (VT(nz) + VT(nz - 1));
  WI(nz + 1) = VT(nz + 1);
  for (int k = 2; k <= nz; k++)
    if (VT(k) == 0.0) WI(k) = VT(k - 1);
  // limit of the speed's divergence per substep (:1613-1621)
  const I con1 = I(0.05);
  for (int k = nz; k >= 1; k--) {
    const I decfl = (WI(k + 1) - WI(k)) * dt * osteps / DZ(k);
    if (decfl > con1) WI(k) = WI(k + 1) - con1 * DZ(k) * odt * fsteps;
  }
  // departure heights of the interfaces and the deformed cells (:1623-1636)
  for (int k = 1; k <= nz + 1; k++) ZA(k) = ZI(k) - WI(k) * dt * osteps;
  ZA(nz + 2) = ZI(nz + 1);
  for (int k = 1; k <= nz + 1; k++) DZA(k) = ZA(k + 1) - ZA(k);
  for (int k = 1; k <= nz; k++) QA(k) = X0(k) * DZ(k) / DZA(k);
  QA(nz + 1) = I(0.0);
  // interface values with the reference's monotonicity test (:1638-1659)
  for (int k = 2; k <= nz; k++) {
    const I dip = (QA(k + 1) - QA(k)) / (DZA(k + 1) + DZA(k));
    const I dim = (QA(k) - QA(k - 1)) / (DZA(k - 1) + DZA(k));
    if (dip * dim <= 0.0) {
      QMI(k) = QA(k);
      QPI(k) = QA(k);
    } else {
      QPI(k) = QA(k) + 0.5 * (dip + dim) * DZA(k);
      QMI(k) = 2.0 * QA(k) - QPI(k);
      if (QPI(k) > 0.0 || QMI(k) < 0.0) {
        QPI(k) = QA(k);
        QMI(k) = QA(k);
      }
    }
  }
  QPI(1) = QA(1);
  QMI(1) = QA(1);
  QMI(nz + 1) = QA(nz + 1);
  QPI(nz + 1) = QA(nz + 1);
  // remap onto the regular cells (:1661-1723)
  int kb = 1, kt = 1;
  for (int k = 1; k <= nz; k++) {
    kb = max(kb - 1, 1);
    kt = max(kt - 1, 1);
    if (ZI(k) >= ZA(nz + 1)) break;
    for (int kk = kb; kk <= nz; kk++)
      if (ZI(k) <= ZA(kk + 1)) {
        kb = kk;
        break;
      }
    for (int kk = kt; kk <= nz + 2; kk++)
      if (ZI(k + 1) <= ZA(kk)) {
        kt = kk;
        break;
      }
    kt = kt - 1;
    I xr = X0(k);
    if (kt == kb) {
      const I tl = (ZI(k) - ZA(kb)) / DZA(kb);
      const I th = (ZI(k + 1) - ZA(kb)) / DZA(kb);
      const I tl2 = tl * tl, th2 = th * th;
      const I qqd = 0.5 * (QPI(kb) - QMI(kb));
      const I qqh = qqd * th2 + QMI(kb) * th;
      const I qql = qqd * tl2 + QMI(kb) * tl;
      xr = (qqh - qql) / (th - tl);
    } else if (kt > kb) {
      const I tl = (ZI(k) - ZA(kb)) / DZA(kb);
      const I tl2 = tl * tl;
      I qqd = 0.5 * (QPI(kb) - QMI(kb));
      const I qql = qqd * tl2 + QMI(kb) * tl;
      const I dql = QA(kb) - qql;
      I zsum = (1.0 - tl) * DZA(kb);
      I qsum = dql * DZA(kb);
      if (kt - kb > 1)
        for (int m = kb + 1; m <= kt - 1; m++) {
          zsum = zsum + DZA(m);
          qsum = qsum + QA(m) * DZA(m);
        }
      const I th = (ZI(k + 1) - ZA(kt)) / DZA(kt);
      const I th2 = th * th;
      qqd = 0.5 * (QPI(kt) - QMI(kt));
      const I dqh = qqd * th2 + QMI(kt) * th;
      zsum = zsum + th * DZA(kt);
      qsum = qsum + dqh * DZA(kt);
      xr = qsum / zsum;
    }
    const I orho = 1.0 / rho[(long)(k - 1) * ls];
    xr = xr > limit ? xr : I(limit);
    ten[(long)(k - 1) * ls] = R(I(ten[(long)(k - 1) * ls]) + (xr - X0(k)) * orho * odt);
    x[(long)(k - 1) * ls] = R(xr);
  }
  // mass through the surface (:1725-1739)
  for (int k = 1; k <= nz; k++) {
    if (ZA(k) < 0.0 && ZA(k + 1) <= 0.0) {
      if (precip) *precip = *precip + QA(k) * DZA(k);
    } else if (ZA(k) < 0.0 && ZA(k + 1) > 0.0) {
      const I th = (0.0 - ZA(k)) / DZA(k);
      const I th2 = th * th;
      const I qqd = 0.5 * (QPI(k) - QMI(k));
      const I qqh = qqd * th2 + QMI(k) * th;
      if (precip) *precip = *precip + qqh * DZA(k);
      break;
    }
  }
}

// Phase B on the column of active slot s.  SEMI: rain and graupel by the
// semi-Lagrangian scheme (semi_sedi_flag, main:599-613, 640-671), which rechecks the
// species and recomputes their fall speeds after every substep (needs cst and ci).
// Variants of the sedimentation kernel (picked per context by the autotuner): v % 3
// selects the number of levels whose loads a substep's sweep issues together, 1, 2 or
// 3 (more loads in flight per thread against more registers per thread; 4 and 8 were
// measured slower still); (v / 3) % 2 = 1 splits a column's species over two threads
// (rain and snow -- snow's fall speed reads rain's state after rain sedimentation --
// and graupel, ice and cloud), twice the threads for the same serial chains; v < 6
// runs a species' substeps level by level (sweep_all) where the warp's substep counts
// fit its register history, v >= 6 always substep by substep.  In the level-by-level
// walk, v % 3 > 0 issues the next level's loads while a level runs its substeps.
constexpr int kSedimVariants = 12;
__host__ __device__ constexpr int sedim_group(int v) { return v % 3 + 1; }
__host__ __device__ constexpr bool sedim_split(int v) { return (v / 3) % 2 == 1; }
__host__ __device__ constexpr bool sedim_blocked(int v) { return v < 6; }

// Phase B of active slot s; part < 0: every species, 0: rain and snow, 1: graupel, ice
// and cloud (each part writes the precipitation sums and substep counts of its own
// species).
template <class R, class S, bool SEMI, int G = 1, bool BLOCK = true>
__device__ __forceinline__ void sedim_column(const StepArgs<S>& a, const TempoConsts<Cst<R>>* cst,
                                             const IslandConsts<Isl<R>>* ci, long s, int part = -1) {
  using I = Isl<R>;
  const int nz = a.nz;
  const long NI = a.NI;
  const ColGeom g = col_geom(a, a.act[s]);
  const long cs = a.ncol_pad, fsd = (long)nz * cs;
  I* sd = reinterpret_cast<I*>(a.sd) + pt_base(s, nz);
  R* sr = reinterpret_cast<R*>(a.sr) + pt_base(s, nz);
  // this slot's level 0 in the plane of a sedimenting field or its tendency: values of
  // the bulk type R (in the mixed form FP32 in the first half of the plane); the walks
  // below keep them in the island type between the loads and stores
  auto xp = [&](int f) -> R* {
    return reinterpret_cast<R*>(reinterpret_cast<I*>(a.sd) + (long)f * fsd) + pt_base(s, nz);
  };
  const R dt = step_dt<R>(a);
  const I dti = step_dti<R>(a);
  const S* dzp = a.dz + g.base;

  uint8_t any = 0;
  for (int k = 0; k < nz; k++) any |= a.pmask[pt_off(s, k, nz)];
  const bool any_qr = any & PM_QR, any_qg = any & PM_QG, any_qs = any & PM_QS,
             any_qi = any & PM_QI, any_qc = any & PM_QC;

  I prec_r = I(0.0), prec_g = I(0.0), prec_s = I(0.0), prec_i = I(0.0), prec_c = I(0.0);
  const I* rho = sd + SD_RHO * fsd;
  // fills vt (and vtn) from above in place, computes ktop and substeps
  auto fill = [&](int fv, int fvn, bool use_max, bool snow, int& steps, int& ktop) {
    steps = 1;
    ktop = 1;
    R vup = R(0), vnup = R(0);
    for (int k = nz - 1; k >= 0; k--) {
      const long o = (long)k * kSlotTile;
      R v, vn = R(0);
      if (snow) {
        R A = sr[SR_VTSA * fsd + o];
        if (A >= R(0)) {
          if (sr[SR_VTSB * fsd + o] != R(0)) {
            R vrain = any_qr ? sr[SR_VTR * fsd + o] : R(0);
            R rsk = xp(SD_XRS)[o];
            R srr = rsk / (rsk + xp(SD_XRR)[o]);
            v = A * srr + (R(1.0) - srr) * vrain;
          } else {
            v = A;
          }
        } else {
          v = vup;
        }
      } else {
        v = sr[fv * fsd + o];
        vn = sr[fvn * fsd + o];
        if (v < R(0)) {
          v = vup;
          vn = vnup;
        }
        sr[fvn * fsd + o] = vn;
      }
      sr[fv * fsd + o] = v;
      vup = v;
      vnup = vn;
      R vm = use_max ? Max(v, vn) : v;
      if (vm > R(1.e-3)) {
        ktop = max(ktop, k + 1);
        R dz_by_vt = R(dzp[k * NI]) / vm;
        steps = max(steps, Int(dt / dz_by_vt + R(1.0)));
      }
    }
    if (ktop == nz) ktop = nz - 1;
  };
  // one substep of NF fields whose fall speeds sit in the R scratch (sedimentation,
  // main:1516-1559), each field's arithmetic exactly that of a sweep of its own:
  // fluxes from the pre-substep state, level nz first, then ktop..1.  The fields of
  // one species share the levels' factors, loaded once.  The levels below ktop go in
  // groups of G: a group's loads are issued together (no level's update reads
  // another level's updated values), then the group's levels are updated in the
  // serial order and stored.  Field 0 feeds the precipitation sum.
  auto sweep = [&](auto nf, const int* fx, const int* ften, const int* fv, const double* limit,
                   int steps, int ktop, I* precip) {
    constexpr int NF = decltype(nf)::value;
    constexpr bool kMixed = std::is_same<I, df>::value;
    R* x[NF];
    R* ten[NF];
    const R* vt[NF];
    I lim[NF], s_up[NF], s0[NF];
#pragma unroll
    for (int f = 0; f < NF; f++) {
      x[f] = xp(fx[f]);
      ten[f] = xp(ften[f]);
      vt[f] = sr + fv[f] * fsd;
      lim[f] = I(limit[f]);
    }
    const I osteps = 1.0 / I(steps);
    // mixed form: the per-level factors 1/dz and 1/(dz rho) precomputed in the points
    // kernel; FP64: 1/dz and 1/rho formed here, as the reference does
    const I* odz = sd + SD_ODZ * fsd;
    const I* ozr = sd + SD_OZR * fsd;
    const I cx = dti * osteps;
    {
      const int k = nz - 1;
      const long o = (long)k * kSlotTile;
      I fo, fr;
      if constexpr (kMixed) {
        fo = odz[o];
        fr = ozr[o];
      } else {
        fo = 1.0 / ldi<I>(dzp + k * NI);
        fr = 1.0 / rho[o];
      }
#pragma unroll
      for (int f = 0; f < NF; f++) {
        const I xt = I(x[f][o]), tt = I(ten[f][o]);
        const I s_top = I(vt[f][o]) * xt;
        if constexpr (kMixed) {
          ten[f][o] = R(tt - s_top * fr * osteps);
          x[f][o] = R(Max(lim[f], xt - s_top * fo * cx));
        } else {
          ten[f][o] = R(tt - s_top * fo * osteps * fr);
          x[f][o] = R(Max(lim[f], xt - s_top * fo * dti * osteps));
        }
        s_up[f] = (ktop == nz - 1) ? s_top : I(vt[f][ktop * kSlotTile]) * I(x[f][ktop * kSlotTile]);
        s0[f] = (nz == 1) ? s_top : I(vt[f][0]) * I(x[f][0]);
      }
    }
    for (int k = ktop - 1; k >= 0; k -= G) {
      R gv[NF][G];
      I gx[NF][G], gt[NF][G], ga[G], gb[G];
#pragma unroll
      for (int u = 0; u < G; u++)
        if (u <= k) {
          const long o = (long)(k - u) * kSlotTile;
          if constexpr (kMixed) {
            ga[u] = odz[o];
            gb[u] = ozr[o];
          } else {
            ga[u] = ldi<I>(dzp + (long)(k - u) * NI);
            gb[u] = rho[o];
          }
#pragma unroll
          for (int f = 0; f < NF; f++) {
            gv[f][u] = vt[f][o];
            gx[f][u] = I(x[f][o]);
            gt[f][u] = I(ten[f][o]);
          }
        }
#pragma unroll
      for (int u = 0; u < G; u++)
        if (u <= k) {
          I fo, fr;
          if constexpr (kMixed) {
            fo = ga[u];
            fr = gb[u];
          } else {
            fo = 1.0 / ga[u];
            fr = 1.0 / gb[u];
          }
#pragma unroll
          for (int f = 0; f < NF; f++) {
            const I s_k = I(gv[f][u]) * gx[f][u];
            if constexpr (kMixed) {
              const I dflux = s_up[f] - s_k;
              gt[f][u] = gt[f][u] + dflux * fr * osteps;
              gx[f][u] = Max(lim[f], gx[f][u] + dflux * fo * cx);
            } else {
              gt[f][u] = gt[f][u] + (s_up[f] - s_k) * fo * osteps * fr;
              gx[f][u] = Max(lim[f], gx[f][u] + (s_up[f] - s_k) * fo * dti * osteps);
            }
            if (k - u == 0) s0[f] = s_k;
            s_up[f] = s_k;
          }
        }
#pragma unroll
      for (int u = 0; u < G; u++)
        if (u <= k) {
          const long o = (long)(k - u) * kSlotTile;
#pragma unroll
          for (int f = 0; f < NF; f++) {
            ten[f][o] = R(gt[f][u]);
            x[f][o] = R(gx[f][u]);
          }
        }
    }
    if (precip && I(x[0][0]) > low_limit_mass_for_precip) *precip = *precip + s0[0] * dti * osteps;
  };
  // All substeps of NF fields, level by level (temporal blocking).  In the upwind
  // scheme level k's substep n reads only level k's state and the flux of level k + 1
  // at substep n, so the column is walked once, top down: each level runs its substeps
  // in order while hist[f][n] carries the flux of the level above at substep n.  Every
  // level update, and every addition to the precipitation sum, is the arithmetic of
  // the substep-by-substep sweep above in the same order; a level's fields are read
  // and written once for all substeps instead of once per substep.  One call runs
  // nsub <= SM of the steps substeps (hist lives in registers); a column with more
  // substeps is walked in passes, each from the state the previous pass stored.
  auto sweep_all = [&](auto nf, auto smax, const int* fx, const int* ften, const int* fv,
                       const double* limit, int steps, int nsub, int ktop, I* precip) {
    constexpr int NF = decltype(nf)::value;
    constexpr int SM = decltype(smax)::value;
    constexpr bool kMixed = std::is_same<I, df>::value;
    R* x[NF];
    R* ten[NF];
    const R* vt[NF];
    I lim[NF], hist[NF][SM];
#pragma unroll
    for (int f = 0; f < NF; f++) {
      x[f] = xp(fx[f]);
      ten[f] = xp(ften[f]);
      vt[f] = sr + fv[f] * fsd;
      lim[f] = I(limit[f]);
    }
    const I osteps = 1.0 / I(steps);
    const I* odz = sd + SD_ODZ * fsd;
    const I* ozr = sd + SD_OZR * fsd;
    const I cx = dti * osteps;
    {
      const int k = nz - 1;
      const long o = (long)k * kSlotTile;
      I fo, fr;
      if constexpr (kMixed) {
        fo = odz[o];
        fr = ozr[o];
      } else {
        fo = 1.0 / ldi<I>(dzp + k * NI);
        fr = 1.0 / rho[o];
      }
#pragma unroll
      for (int f = 0; f < NF; f++) {
        I xk = I(x[f][o]), tk = I(ten[f][o]);
        const I v = I(vt[f][o]);
#pragma unroll
        for (int n = 0; n < SM; n++)
          if (n < nsub) {
            const I s_top = v * xk;
            if constexpr (kMixed) {
              tk = tk - s_top * fr * osteps;
              xk = Max(lim[f], xk - s_top * fo * cx);
            } else {
              tk = tk - s_top * fo * osteps * fr;
              xk = Max(lim[f], xk - s_top * fo * dti * osteps);
            }
            hist[f][n] = s_top;
            if (k == 0 && f == 0 && precip && xk > low_limit_mass_for_precip)
              *precip = *precip + s_top * dti * osteps;
          }
        ten[f][o] = R(tk);
        x[f][o] = R(xk);
      }
      if (ktop != nz - 1) {  // levels ktop..nz-2 keep their state: a constant flux
#pragma unroll
        for (int f = 0; f < NF; f++) {
          const I s_c = I(vt[f][ktop * kSlotTile]) * I(x[f][ktop * kSlotTile]);
#pragma unroll
          for (int n = 0; n < SM; n++) hist[f][n] = s_c;
        }
      }
    }
    // Levels ktop-1 .. 0.  G >= 2: each level's loads are issued one level ahead (while
    // the level above runs its substeps), so the column walk does not wait a memory
    // round trip per level, at the cost of registers; G = 1: loaded when reached.
    if constexpr (G >= 2) {
      I cx_[NF], ct_[NF], ca = I(0.0), cb = I(0.0);
      R cv_[NF];
      auto load_level = [&](int k, I* xx, I* tt, R* vv, I& a, I& b) {
        const long o = (long)k * kSlotTile;
        if constexpr (kMixed) {
          a = odz[o];
          b = ozr[o];
        } else {
          a = ldi<I>(dzp + (long)k * NI);
          b = rho[o];
        }
#pragma unroll
        for (int f = 0; f < NF; f++) {
          xx[f] = I(x[f][o]);
          tt[f] = I(ten[f][o]);
          vv[f] = vt[f][o];
        }
      };
      if (ktop >= 1) load_level(ktop - 1, cx_, ct_, cv_, ca, cb);
      for (int k = ktop - 1; k >= 0; k--) {
        I nx_[NF], nt_[NF], na = I(0.0), nb = I(0.0);
        R nv_[NF];
        if (k >= 1) load_level(k - 1, nx_, nt_, nv_, na, nb);
        const long o = (long)k * kSlotTile;
        I fo, fr;
        if constexpr (kMixed) {
          fo = ca;
          fr = cb;
        } else {
          fo = 1.0 / ca;
          fr = 1.0 / cb;
        }
#pragma unroll
        for (int f = 0; f < NF; f++) {
          I xk = cx_[f], tk = ct_[f];
          const I v = I(cv_[f]);
#pragma unroll
          for (int n = 0; n < SM; n++)
            if (n < nsub) {
              const I s_k = v * xk;
              if constexpr (kMixed) {
                const I dflux = hist[f][n] - s_k;
                tk = tk + dflux * fr * osteps;
                xk = Max(lim[f], xk + dflux * fo * cx);
              } else {
                tk = tk + (hist[f][n] - s_k) * fo * osteps * fr;
                xk = Max(lim[f], xk + (hist[f][n] - s_k) * fo * dti * osteps);
              }
              hist[f][n] = s_k;
              if (k == 0 && f == 0 && precip && xk > low_limit_mass_for_precip)
                *precip = *precip + s_k * dti * osteps;
            }
          ten[f][o] = R(tk);
          x[f][o] = R(xk);
        }
        if (k >= 1) {
#pragma unroll
          for (int f = 0; f < NF; f++) {
            cx_[f] = nx_[f];
            ct_[f] = nt_[f];
            cv_[f] = nv_[f];
          }
          ca = na;
          cb = nb;
        }
      }
    } else {
      for (int k = ktop - 1; k >= 0; k--) {
        const long o = (long)k * kSlotTile;
        I fo, fr;
        if constexpr (kMixed) {
          fo = odz[o];
          fr = ozr[o];
        } else {
          fo = 1.0 / ldi<I>(dzp + (long)k * NI);
          fr = 1.0 / rho[o];
        }
#pragma unroll
        for (int f = 0; f < NF; f++) {
          I xk = I(x[f][o]), tk = I(ten[f][o]);
          const I v = I(vt[f][o]);
#pragma unroll
          for (int n = 0; n < SM; n++)
            if (n < nsub) {
              const I s_k = v * xk;
              if constexpr (kMixed) {
                const I dflux = hist[f][n] - s_k;
                tk = tk + dflux * fr * osteps;
                xk = Max(lim[f], xk + dflux * fo * cx);
              } else {
                tk = tk + (hist[f][n] - s_k) * fo * osteps * fr;
                xk = Max(lim[f], xk + (hist[f][n] - s_k) * fo * dti * osteps);
              }
              hist[f][n] = s_k;
              if (k == 0 && f == 0 && precip && xk > low_limit_mass_for_precip)
                *precip = *precip + s_k * dti * osteps;
            }
          ten[f][o] = R(tk);
          x[f][o] = R(xk);
        }
      }
    }
    if (ktop == 0 && nz > 1 && precip) {  // level 0 above the fall: its flux, unchanged
      const I s0 = I(vt[0][0]) * I(x[0][0]);
      const bool add = I(x[0][0]) > low_limit_mass_for_precip;
#pragma unroll
      for (int n = 0; n < SM; n++)
        if (n < nsub && add) *precip = *precip + s0 * dti * osteps;
    }
  };
  // the substeps of one species: level by level when the warp's largest count fits the
  // register history, else substep by substep.  The mixed form walks level by level
  // always, in passes of up to 8 substeps: its planes hold FP32 values, so a pass
  // stores FP32 and a substep-by-substep sweep would round the state after every
  // substep where the walk keeps it in the island type.
  auto sweeps = [&](auto nf, const int* fx, const int* ften, const int* fv, const double* limit,
                    int steps, int ktop, I* precip) {
    constexpr bool kMixed = std::is_same<I, df>::value;
    const int wmax = (BLOCK || kMixed) ? __reduce_max_sync(__activemask(), steps) : 1 << 30;
    if (wmax <= 4) {
      sweep_all(nf, std::integral_constant<int, 4>{}, fx, ften, fv, limit, steps, steps, ktop, precip);
    } else if (wmax <= 8) {
      sweep_all(nf, std::integral_constant<int, 8>{}, fx, ften, fv, limit, steps, steps, ktop, precip);
    } else if constexpr (kMixed) {
      for (int n0 = 0; n0 < steps; n0 += 8)
        sweep_all(nf, std::integral_constant<int, 8>{}, fx, ften, fv, limit, steps, min(8, steps - n0),
                  ktop, precip);
    } else {
      for (int n = 0; n < steps; n++) sweep(nf, fx, ften, fv, limit, steps, ktop, precip);
    }
  };
  using One = std::integral_constant<int, 1>;
  using Two = std::integral_constant<int, 2>;
  using Three = std::integral_constant<int, 3>;
  int steps, ktop;
  unsigned sub[5] = {0, 0, 0, 0, 0};
  // semi-Lagrangian path: one sweep on this column's work rows, and the level's state
  // for the species checks (rhof and visco as after the last stage of phase A)
  [[maybe_unused]] auto sl = [&](int fx, int ften, int fv, double limit, int st, I* precip) {
    if constexpr (SEMI) {
      const long cs2 = a.ncol_pad;
      sl_sweep<R, I, S>(nz, xp(fx), xp(ften), sr + fv * fsd, kSlotTile, dzp, NI, rho,
                        reinterpret_cast<I*>(a.slw) + s, (long)(nz + 2) * cs2, cs2, st, limit,
                        precip, dti, I(a.odt));
    }
  };
  [[maybe_unused]] auto level_state = [&](int k, Lev<R>& L) {
    const long o = (long)k * kSlotTile, e = g.base + (long)k * NI;
    L.cs = cst;
    L.ci = ci;
    L.rho = sd[SD_RHO * fsd + o];
    const I t1d = (a.flags & F_USE_T) ? ldi<I>(a.t + e) : ldi<I>(a.th + e) * ldi<I>(a.pii + e);
    L.temp = t1d + sd[SD_TTEN * fsd + o] * dti;
    thermo_tail(L);
  };
  [[maybe_unused]] const R odt_r = step_odt<R>(a);
  const bool p0 = part != 1, p1 = part != 0;
  // decision trace of a test build: substep count j and top level 4 + j of species j
  [[maybe_unused]] auto trace_col = [&](int j, int st, int kt) {
#ifdef TEMPO_TRACE
    if (a.trace) {
      int* tc = a.trace + a.ncol * nz * kTracePoint + (long)a.act[s] * kTraceColumn;
      if (j < 4) tc[j] = st;
      tc[4 + j] = kt;
    }
#endif
  };
  if (any_qr && p0) {
    fill(SR_VTR, SR_VTNR, true, false, steps, ktop);
    trace_col(0, steps, ktop);
    if constexpr (SEMI) {
      steps = max((int)(steps / 10.0) + 1, 1);  // semi_sedi_factor (main:595, 599)
      sub[0] = steps;
      for (int n = 0; n < steps; n++) {
        sl(SD_XRR, SD_TQR, SR_VTR, r1, steps, &prec_r);
        sl(SD_XNR, SD_TNR, SR_VTNR, r2, steps, nullptr);
        // rain_check_and_update from qr1d, then rain_fallspeed without substeps
        // (main:604-613), top down
        R vup = R(0), vnup = R(0);
        for (int k = nz - 1; k >= 0; k--) {
          Lev<R> L;
          level_state(k, L);
          const long o = (long)k * kSlotTile, e = g.base + (long)k * NI;
          const R tq = xp(SD_TQR)[o], tn = xp(SD_TNR)[o];
          L.qrten = tq;
          L.nrten = tn;
          R q = R(a.qr[e]), nn = R(a.nr[e]);
          rain_check(L, q, nn, dt, odt_r);
          xp(SD_XRR)[o] = L.rr;
          xp(SD_XNR)[o] = L.nr;
          if (!(L.qrten == tq)) xp(SD_TQR)[o] = L.qrten;
          if (!(L.nrten == tn)) xp(SD_TNR)[o] = L.nrten;
          R v = vup, vn = vnup;
          if (L.rr > R(r1)) rain_speeds(L, *cst, v, vn);
          sr[SR_VTR * fsd + o] = v;
          sr[SR_VTNR * fsd + o] = vn;
          vup = v;
          vnup = vn;
        }
      }
    } else {
      sub[0] = steps;
      const int fx[2] = {SD_XRR, SD_XNR}, ft[2] = {SD_TQR, SD_TNR}, fv[2] = {SR_VTR, SR_VTNR};
      const double lim[2] = {r1, r2};
      sweeps(Two{}, fx, ft, fv, lim, steps, ktop, &prec_r);
    }
  }
  if (any_qg && p1) {
    fill(SR_VTG, SR_VTNG, false, false, steps, ktop);
    trace_col(1, steps, ktop);
    if constexpr (SEMI) {
      const bool hail = a.flags & F_HAIL;
      steps = max((int)(steps / 10.0) + 1, 1);  // main:636, 640
      sub[1] = steps;
      for (int n = 0; n < steps; n++) {
        sl(SD_XRG, SD_TQG, SR_VTG, r1, steps, &prec_g);
        sl(SD_XNG, SD_TNG, SR_VTNG, r2, steps, nullptr);
        sl(SD_XRB, SD_TQB, SR_VTG, meters3_to_liters * r1 / rho_gd(nrhg), steps, nullptr);
        // graupel_check_and_update from qg1d (ng1d, qb1d), then graupel_fallspeed
        // without substeps (main:651-667), top down
        R vup = R(0), vnup = R(0);
        for (int k = nz - 1; k >= 0; k--) {
          Lev<R> L;
          level_state(k, L);
          const long o = (long)k * kSlotTile, e = g.base + (long)k * NI;
          const R tq = xp(SD_TQG)[o], tn = xp(SD_TNG)[o], tb = xp(SD_TQB)[o];
          L.qgten = tq;
          L.ngten = tn;
          L.qbten = tb;
          R q = R(a.qg[e]), nn = hail ? R(a.ng[e]) : R(0), b = hail ? R(a.qb[e]) : R(0);
          graupel_check(L, q, nn, b, hail, dt, odt_r);
          xp(SD_XRG)[o] = L.rg;
          xp(SD_XNG)[o] = L.ng;
          xp(SD_XRB)[o] = L.rb;
          if (!(L.qgten == tq)) xp(SD_TQG)[o] = L.qgten;
          if (!(L.ngten == tn)) xp(SD_TNG)[o] = L.ngten;
          if (!(L.qbten == tb)) xp(SD_TQB)[o] = L.qbten;
          R v = vup, vn = vnup;
          if (L.rg > R(r1)) graupel_speeds(L, *cst, a.flags, v, vn);
          sr[SR_VTG * fsd + o] = v;
          sr[SR_VTNG * fsd + o] = vn;
          vup = v;
          vnup = vn;
        }
      }
    } else {
      sub[1] = steps;
      const int fx[3] = {SD_XRG, SD_XNG, SD_XRB}, ft[3] = {SD_TQG, SD_TNG, SD_TQB},
                fv[3] = {SR_VTG, SR_VTNG, SR_VTG};
      const double lim[3] = {r1, r2, meters3_to_liters * r1 / rho_gd(nrhg)};
      sweeps(Three{}, fx, ft, fv, lim, steps, ktop, &prec_g);
    }
  }
  if (any_qs && p0) {
    fill(SR_VTSA, SR_VTSA, false, true, steps, ktop);
    trace_col(2, steps, ktop);
    sub[2] = steps;
    const int fx[1] = {SD_XRS}, ft[1] = {SD_TQS}, fv[1] = {SR_VTSA};
    const double lim[1] = {r1};
    sweeps(One{}, fx, ft, fv, lim, steps, ktop, &prec_s);
  }
  if (any_qi && p1) {
    fill(SR_VTI, SR_VTNI, false, false, steps, ktop);
    trace_col(3, steps, ktop);
    sub[3] = steps;
    const int fx[2] = {SD_XRI, SD_XNI}, ft[2] = {SD_TQI, SD_TNI}, fv[2] = {SR_VTI, SR_VTNI};
    const double lim[2] = {r1, r2};
    sweep(Two{}, fx, ft, fv, lim, steps, ktop, &prec_i);
  }
  if (any_qc && p1) {  // cloud_fallspeed (main:1945-1977): settles only below 500 m
    int kt = 1;
    I hgtc = I(0.0);
    for (int k = 1; k <= nz - 1; k++) {
      if (xp(SD_XRC)[(long)(k - 1) * kSlotTile] > r2) kt = k;
      hgtc = hgtc + ldi<I>(dzp + (long)(k - 1) * NI);
      if (hgtc > 500.0) break;
    }
    for (int k = kt; k < nz; k++) {  // vt stays zero above ktop
      sr[SR_VTC * fsd + (long)k * kSlotTile] = R(0);
      sr[SR_VTNC * fsd + (long)k * kSlotTile] = R(0);
    }
    sub[4] = 1;
    trace_col(4, 1, kt);
    const int fx[2] = {SD_XRC, SD_XNC}, ft[2] = {SD_TQC, SD_TNC}, fv[2] = {SR_VTC, SR_VTNC};
    const double lim[2] = {r1, r2};
    sweep(Two{}, fx, ft, fv, lim, 1, kt, &prec_c);
  }
  for (int q = 0; q < 5; q++)
    if (sub[q]) atomicMax(a.stats + 1 + q, (unsigned long long)sub[q]);
  I* sc = reinterpret_cast<I*>(a.sc) + s;
  if (p0) {
    sc[SC_PR * cs] = prec_r;
    sc[SC_PS * cs] = prec_s;
  }
  if (p1) {
    sc[SC_PG * cs] = prec_g;
    sc[SC_PI * cs] = prec_i;
    sc[SC_PC * cs] = prec_c;
  }
}

// phase B, one thread per active column (SPLIT: per active column and part, the part
// in blockIdx.y)
// The mixed form asks for 5 resident blocks (at most 102 registers): 12.9 against
// 13.6 ms unasked and 16.5 ms with 6 blocks at 1 M columns (variant 5).
template <class R>
__host__ __device__ constexpr int sedim_min_blocks() {
  return std::is_same<R, float>::value ? 5 : 1;
}
template <class R, class S, int G = 1, bool SPLIT = false, bool BLOCK = true>
__global__ void __launch_bounds__(128, sedim_min_blocks<R>()) tempo_sedim_kernel(const __grid_constant__ StepArgs<S> a) {
  const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= (long)*a.nact) return;
  sedim_column<R, S, false, G, BLOCK>(a, nullptr, nullptr, s, SPLIT ? (int)blockIdx.y : -1);
}
// phase B with semi-Lagrangian rain and graupel (F_SEMI), one thread per active column
template <class R, class S>
__global__ void __launch_bounds__(128) tempo_sedim_semi_kernel(const __grid_constant__ StepArgs<S> a,
                                                               const __grid_constant__ TempoConsts<Cst<R>> cst,
                                                               const __grid_constant__ IslandConsts<Isl<R>> ci) {
  const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= (long)*a.nact) return;
  sedim_column<R, S, true>(a, &cst, &ci, s);
}

// non-negative value into a running maximum (IEEE order of non-negative floats is the
// integer order of their bit patterns)
__device__ __forceinline__ void atomic_max_nonneg(float* p, float v) {
  atomicMax(reinterpret_cast<int*>(p), __float_as_int(v));
}
__device__ __forceinline__ void atomic_max_nonneg(double* p, double v) {
  atomicMax(reinterpret_cast<unsigned long long*>(p), (unsigned long long)__double_as_longlong(v));
}

// ---------------------------------------------------------------------------------
// final: phase C at one (level, active slot)
// ---------------------------------------------------------------------------------
// Phase C at point (level k, active slot s); outputs go through the I/O policy.
template <class R, class S, class IO>
__device__ __forceinline__ void final_point(const StepArgs<S>& a, const TempoConsts<Cst<R>>& cst,
                                            const IslandConsts<Isl<R>>& ci, int k, long s,
                                            const IO& io) {
  using I = Isl<R>;
  const int nz = a.nz;
  const ColGeom g = col_geom(a, a.act[s]);
  const long e = g.base + (long)k * a.NI;
  const uint32_t f = a.flags;
  const bool has_nc = f & F_NC, hail = f & F_HAIL;
  const R dt = step_dt<R>(a), odt = step_odt<R>(a);
  const I dti = step_dti<R>(a);
  const long cs = a.ncol_pad, fsd = (long)nz * cs, o = pt_off(s, k, nz);
  // the cloud number of phase A's initial checks (per level from the network with F_MLNC)
  const R ncsave = (f & F_MLNC) ? reinterpret_cast<const R*>(a.ncw)[o] : ncsave_of<R>(a, g);

  Lev<R> L;
  L.cs = &cst;
  L.ci = &ci;
#ifdef TEMPO_TRACE
  L.tr = a.trace ? a.trace + ((long)a.act[s] * nz + k) * kTracePoint : nullptr;
#endif
  L.t1d = (f & F_USE_T) ? io.template in<I>(a.t[e], C_T1D)
                        : io.template in<I>(a.th[e], C_T1D) * ldi<I>(a.pii + e);
  L.pres = R(a.p[e]);
  L.tten = io.template sdin<I, I>(SD_TTEN * fsd + o, C_TTEN);
  L.qv = io.template sdin<I, I>(SD_QV * fsd + o, C_QV);
  L.rho = io.template sdin<I, I>(SD_RHO * fsd + o, C_RHO);
  L.temp = L.t1d + L.tten * dti;
  const R ocp = R(1.0) / (R(cp) * (R(1.0) + R(0.887) * R(L.qv)));
  const R lvap = R(lvap0) + (R(2106.0) - R(4218.0)) * R(L.temp - t0);
  L.qc1d = io.template in<R>(a.qc[e], C_QC);
  L.nc1d = has_nc ? io.template in<R>(a.nc[e], C_NC) : R(0);
  L.qr1d = io.template in<R>(a.qr[e], C_QR);
  L.nr1d = io.template in<R>(a.nr[e], C_NR);
  L.qi1d = io.template in<R>(a.qi[e], C_QI);
  L.ni1d = io.template in<R>(a.ni[e], C_NI);
  L.qs1d = io.template in<R>(a.qs[e], C_QS);
  L.qg1d = io.template in<R>(a.qg[e], C_QG);
  L.ng1d = hail ? io.template in<R>(a.ng[e], C_NG) : R(0);
  L.qb1d = hail ? io.template in<R>(a.qb[e], C_QB) : R(0);
  L.qrten = io.template sxin<R, I>(fsd, SD_TQR, o, C_TQR);
  L.nrten = io.template sxin<R, I>(fsd, SD_TNR, o, C_TNR);
  L.qgten = io.template sxin<R, I>(fsd, SD_TQG, o, C_TQG);
  L.ngten = io.template sxin<R, I>(fsd, SD_TNG, o, C_TNG);
  L.qbten = io.template sxin<R, I>(fsd, SD_TQB, o, C_TQB);
  L.qsten = io.template sxin<R, I>(fsd, SD_TQS, o, C_TQS);
  L.qiten = io.template sxin<R, I>(fsd, SD_TQI, o, C_TQI);
  L.niten = io.template sxin<R, I>(fsd, SD_TNI, o, C_TNI);
  L.qcten = io.template sxin<R, I>(fsd, SD_TQC, o, C_TQC);
  L.ncten = io.template sxin<R, I>(fsd, SD_TNC, o, C_TNC);
  L.smob = L.smoc = L.smo2 = L.smoz = R(0);
  if (!(f & F_NOMICRO)) {  // freeze_cloud_melt_ice (main:2124-2165)
    R xri = Max(R(0.0), L.qi1d + L.qiten * dt);
    if ((L.temp > t0) && (xri > R(0.0))) {
      L.qcten = L.qcten + xri * odt;
      L.ncten = L.ncten + L.ni1d * odt;
      L.qiten = L.qiten - xri * odt;
      L.niten = -(L.ni1d * odt);
      L.tten = L.tten - ci.lfus * ocp * xri * odt;
    }
    R xrc = Max(R(0.0), L.qc1d + L.qcten * dt);
    if ((L.temp < hgfrz) && (xrc > R(0.0))) {
      R lfus2 = R(lsub) - lvap;
      R xnc;
      if (has_nc)
        xnc = L.nc1d + L.ncten * dt;
      else
        xnc = ncsave / R(L.rho) + L.ncten * dt;
      L.qiten = L.qiten + xrc * odt;
      L.niten = L.niten + xnc * odt;
      L.qcten = L.qcten - xrc * odt;
      L.ncten = L.ncten - xnc * odt;
      L.tten = L.tten + I(lfus2) * ocp * xrc * odt;
    }
  }
  const I tnew = L.t1d + L.tten * dti;
  if (f & F_USE_T)
    io.arr(A_T, e, tnew);
  else
    io.th(e, tnew / ldi<I>(a.pii + e));
  // final checks (main:750-781)
  TG_TRACE_PASS(L, 4);
  cloud_check(L, L.qc1d, L.nc1d, has_nc, ncsave, dt, odt);
  rain_check(L, L.qr1d, L.nr1d, dt, odt);
  ice_check(L, L.qi1d, L.ni1d, dt, odt);
  snow_check(L, L.qs1d, dt, odt);
  if (L.l_qs) snow_moments(L, R(Min(I(-0.1), L.temp - t0)), 2);
  graupel_check(L, L.qg1d, L.ng1d, L.qb1d, hail, dt, odt);
  store_checked(a, e, L, io);
  // diagnostics (main:796-863)
  const long e3 = tile3_of(a, g, k);
  io.diag3(a.ncmr, e3, L.nc * R(L.rho));
  io.diag3(a.mvd_r, e3, L.mvd_r);
  io.diag3(a.mvd_g, e3, L.mvd_g);
  S mhd = S(0);
  if constexpr (IO::forward && !IsDual<S>::value) {  // a maximum over levels: no derivative
    if (f & F_MHD) {
      mhd = S(max_hail_diam(L));
      if (a.mhd_col && mhd > S(0)) atomic_max_nonneg(a.mhd_col + g.tile2, mhd);
    }
  }
  if (a.refl10cm) io.diag3(a.refl10cm, e3, reflectivity_10cm(L));
  if constexpr (IO::forward && !IsDual<S>::value) {
    if (f & F_MELT) {  // the melting-layer pass needs the column: keep this level's record
      R zr, zs, zg;
      reflectivity_parts(L, zr, zs, zg);
      const long pl = (long)nz * a.ncol_pad, po = pt_off(s, k, nz);
      double* mv = reinterpret_cast<double*>(a.mlw) + po;
      const double vals[kMeltN] = {double(zr), double(zs), double(zg), double(L.rs), double(L.smob),
                                   double(L.smoc), double(L.rr), double(L.rg), double(L.ng),
                                   double(L.ilamg), double(L.idx_bg)};
#pragma unroll
      for (int q = 0; q < kMeltN; q++) mv[q * pl] = vals[q];
      reinterpret_cast<uint8_t*>(reinterpret_cast<double*>(a.mlw) + kMeltN * pl)[po] =
          ((L.temp > t0 && L.l_qr) ? MB_WARMRAIN : 0) | (L.l_qs ? MB_QS : 0) | (L.l_qg ? MB_QG : 0);
    }
  }
  if (f & F_RE) {  // effective_radius (diags:13-56)
    if constexpr (IO::forward && !IsDual<S>::value) {
      if (f & F_BLRE) {
        // main:832-857: the in-cloud boundary-layer water joins the resolved cloud, the
        // network predicts its number, and the cloud check recomputes rc, nc and ilamc
        // for the effective radius (the step's outputs are already stored)
        R xq = L.qc1d;
        const R qbl = R(a.qc_bl[e]), fbl = R(a.qcfrac_bl[e]);
        if (xq <= R(r1) && qbl > R(1.e-9) && fbl > R(0.0)) xq = xq + qbl / fbl;
        if (xq <= R(1.e-12)) xq = R(0.0);
        R xn = ml_cloud_number(a.mlnet, xq, L.qr1d, L.qi1d, L.qs1d, R(L.pres), R(L.temp), R(a.w[e]));
        L.qcten = R(0.0);
        L.ncten = R(0.0);
        cloud_check(L, xq, xn, true, ncsave, dt, odt);
      }
    }
    R rec = R(0), rei = R(0), res = R(0);
    if (L.l_qc) {
      int nu_c = get_nuc(L.nc);
      rec = Max(R(2.51e-6), Min(R(0.5) * (R(3.0) + R(nu_c)) * L.ilamc, R(50.e-6)));
    }
    if (L.l_qi) rei = Max(R(2.51e-6), Min(R(0.5) * (R(3.0) + R(mu_i)) * L.ilami, R(125.e-6)));
    if (L.l_qs) res = Max(R(5.01e-6), Min(R(0.5) * (L.smoc / L.smob), R(999.e-6)));
    io.diag3(a.re_cloud, e3, rec);
    io.diag3(a.re_ice, e3, rei);
    io.diag3(a.re_snow, e3, res);
  } else {
    io.diag3(a.re_cloud, e3, R(0));
    io.diag3(a.re_ice, e3, R(0));
    io.diag3(a.re_snow, e3, R(0));
  }
  if (k != 0) return;
  // column diagnostics on the lowest level (main:785-794; driver:452-484)
  const I prec_r = io.template scin<I>(SC_PR * cs + s), prec_g = io.template scin<I>(SC_PG * cs + s),
          prec_s = io.template scin<I>(SC_PS * cs + s), prec_i = io.template scin<I>(SC_PI * cs + s),
          prec_c = io.template scin<I>(SC_PC * cs + s);
  const I ffrac = (prec_i + prec_s + prec_g) / (prec_i + prec_s + prec_g + prec_r + r1);
  const I frz = ((L.temp - t0) < -0.5) ? prec_r + prec_c : I(0.0);
  const long t2 = g.tile2;
  io.diag2(a.rain_precip, t2, prec_r);
  io.diag2(a.ice_precip, t2, prec_i);
  io.diag2(a.snow_precip, t2, prec_s);
  io.diag2(a.graupel_precip, t2, prec_g);
  io.diag2(a.frozen_fraction, t2, ffrac);
  io.diag2(a.frz_rain, t2, frz);
  io.diag2(a.mhd_sfc, t2, mhd);
}

// The mixed form asks for 8 resident blocks (64 registers and a few spills, against 87
// registers and 5 blocks unasked; the kernel waits on memory and gains from the
// resident warps: 4.6 against 4.8 ms with 6 blocks and 5.8 ms unasked at 1 M columns);
// the FP64 and dual-number forms keep their registers.
template <class R>
__host__ __device__ constexpr int final_min_blocks() {
  return std::is_same<R, float>::value ? 8 : 1;
}
template <class R, class S>
__global__ void __launch_bounds__(128, final_min_blocks<R>()) tempo_final_kernel(const __grid_constant__ StepArgs<S> a,
                                                           const __grid_constant__ TempoConsts<Cst<R>> cst,
                                                           const __grid_constant__ IslandConsts<Isl<R>> ci) {
  const long nact = (long)*a.nact, npts = nact * a.nz;
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= npts) return;
  const long p = a.ord ? (long)a.ord[q] : q;  // level-major index (phase A's point order)
  if (p >= npts) return;
  const int k = (int)(p / nact);
  final_point<R, S>(a, cst, ci, k, p - (long)k * nact, FwdIO<S>{a});
}

}  // namespace tg
