// tempo_adjoint.cuh -- adjoint (reverse-mode) kernels of the column step.
//
// Given the adjoints of the step's outputs (state after the step, surface precipitation,
// 10-cm reflectivity), these kernels return the adjoints of the step's inputs (state
// before the step: T, qv, qc, nc, qr, nr, qi, ni, qs, qg and, hail-aware, ng, qb).
//
//   Pointwise phases (A: points, C: final, and the early-exit columns): the kernel
//   recomputes the point with dual numbers carrying one direction per input of the
//   phase (Dual<T, N>), which yields the point's local Jacobian column by column, and
//   contracts it with the adjoints of the point's outputs as they are produced (the
//   AdjIO policy).  Branches, clips and table bins follow the recomputed values, which
//   equal the forward trajectory's (the value arithmetic is T's).
//   Phase B (sedimentation, coupled in the vertical): a hand-written reverse sweep per
//   column, with the substep counts, top levels and clip decisions of the forward
//   trajectory, and the pre-substep states recomputed from checkpoints taken every 4
//   substeps.
//
// Adjoint storage: per-output adjoint arrays in the state's memory layout (updated in
// place to the input adjoints), and scratch adjoints in the layout of the step's
// scratch, [field][level][slot].
#pragma once

#include "tempo_step.cuh"

namespace tg {


template <class X> __device__ __forceinline__ auto value_of(const X& x) { return x; }
// Fortran MAX of the forward kernels: the first argument wins ties
template <class T> __device__ __forceinline__ T max_t(T a, T b) { return a > b ? a : b; }
template <class T, int N> __device__ __forceinline__ T value_of(const Dual<T, N>& x) { return x.v; }

// Adjoint I/O policy: seeds direction `id` on the inputs it reads and accumulates
// acc[i] += lambda(output) * d output / d input_i on every output.
template <class T, int N>
struct AdjIO {
  const StepArgs<T>& a;
  const AdjArgs<T>& j;
  T* acc;
  static constexpr bool forward = false;

  template <class R> __device__ __forceinline__ R seed(T v, int id) const {
    R r(v);
    if (id < N) r.d[id] = T(1);
    return r;
  }
  template <class R, class X> __device__ __forceinline__ R in(const X& v, int id) const {
    return seed<R>(T(value_of(v)), id);
  }
  template <class O, class E> __device__ __forceinline__ O sdin(long idx, int id) const {
    return seed<O>(j.psd[idx].v, id);
  }
  template <class E> __device__ __forceinline__ E scin(long idx) const { return E(j.psc[idx].v); }
  template <class V> __device__ __forceinline__ void contract(T lam, const V& v) const {
    if (lam == T(0)) return;
#pragma unroll
    for (int i = 0; i < N; i++) acc[i] += lam * v.d[i];
  }
  template <class V> __device__ __forceinline__ void arr(int id, long e, const V& v) const {
    if (j.lam[id]) contract(j.lam[id][e], v);
  }
  template <class V> __device__ __forceinline__ void th(long e, const V& v) const {
    if (j.lam_th) contract(j.lam_th[e], v);
  }
  template <class X> __device__ __forceinline__ void sd(X*, long idx, const X& v) const {
    contract(j.lam_sd[idx], v);
  }
  // the bulk-type planes of the sedimenting fields (R = I in the derivative types)
  template <class I, class R> __device__ __forceinline__ void sx(long fsd, int f, long o, const R& v) const {
    contract(j.lam_sd[(long)f * fsd + o], v);
  }
  template <class O, class I> __device__ __forceinline__ O sxin(long fsd, int f, long o, int id) const {
    return seed<O>(j.psd[(long)f * fsd + o].v, id);
  }
  template <class X> __device__ __forceinline__ void sr(X*, long idx, const X& v) const {
    contract(j.lam_sr[idx], v);
  }
  __device__ __forceinline__ void pmask(long, uint8_t) const {}
  template <class P, class V> __device__ __forceinline__ void diag3(P* p, long e3, const V& v) const {
    if (p && p == a.refl10cm && j.lam_refl) contract(j.lam_refl[e3], v);
  }
  template <class P, class V> __device__ __forceinline__ void diag2(P*, long, const V&) const {}
};

// adjoint slot of input array `id` at memory offset e (theta mode for the temperature)
template <class T>
__device__ __forceinline__ T* lam_slot(const StepArgs<T>& a, const AdjArgs<T>& j, int id, long e) {
  if (id == A_T) return (a.flags & F_USE_T) ? (j.lam[A_T] ? j.lam[A_T] + e : nullptr)
                                            : (j.lam_th ? j.lam_th + e : nullptr);
  return j.lam[id] ? j.lam[id] + e : nullptr;
}
// input id of the pointwise phases -> array id
__device__ __forceinline__ int arr_of_in(int i) {
  constexpr int m[IN_N] = {A_T, A_QV, A_QC, A_NC, A_QR, A_NR, A_QI, A_NI, A_QS, A_QG, A_NG, A_QB};
  return m[i];
}
template <class T>
__device__ __forceinline__ bool input_present(const StepArgs<T>& a, int i) {
  if (i == IN_NC) return a.flags & F_NC;
  if (i == IN_NG || i == IN_QB) return a.flags & F_HAIL;
  return true;
}

// ---------------------------------------------------------------------------------
// phase A adjoint: one thread per (level, active slot), in the trajectory's point
// order; primal arrays = the state before the step
// ---------------------------------------------------------------------------------
// N directions: IN_N, or IN_NG without hail-aware graupel (ng and qb are then no
// inputs, and the directions IN_NG and IN_QB are the last two)
template <class T, int N = IN_N>
__global__ void __launch_bounds__(128) tempo_points_adjoint_kernel(
    const __grid_constant__ StepArgs<T> a, const __grid_constant__ Tables<T> TT,
    const __grid_constant__ TempoConsts<T> cst, const __grid_constant__ IslandConsts<Dual<T, N>> ci,
    const __grid_constant__ AdjArgs<T> j) {
  using R = Dual<T, N>;
  const long nact = (long)*a.nact;
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nact * a.nz) return;
  const long p = a.ord ? (long)a.ord[q] : q;  // level-major index (regime order of the trajectory)
  if (p >= nact * a.nz) return;
  const int k = (int)(p / nact);
  const long s = p - (long)k * nact;
  T acc[N];
#pragma unroll
  for (int i = 0; i < N; i++) acc[i] = T(0);
  const AdjIO<T, N> io{a, j, acc};
  points_point<R, T, 0>(a, TT, cst, ci, k, s, io);
  const ColGeom g = col_geom(a, a.act[s]);
  const long e = g.base + (long)k * a.NI;
  // phase A overwrites every input but the temperature (the final qv included)
  for (int i = 0; i < N; i++) {
    if (!input_present(a, i)) continue;
    T* slot = lam_slot(a, j, arr_of_in(i), e);
    if (!slot) continue;
    *slot = (i == IN_T ? *slot : T(0)) + acc[i];
  }
}

// ---------------------------------------------------------------------------------
// early-exit columns: the initial checks only (main:417-418), pointwise
// ---------------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(128) tempo_early_adjoint_kernel(
    const __grid_constant__ StepArgs<T> a, const __grid_constant__ TempoConsts<T> cst,
    const __grid_constant__ IslandConsts<Dual<T, IN_N>> ci, const __grid_constant__ AdjArgs<T> j) {
  using R = Dual<T, IN_N>;
  const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.ncol * a.nz) return;
  const long c = p % a.ncol;
  const int k = (int)(p / a.ncol);
  if (j.colflag[c]) return;
  const ColGeom g = col_geom(a, c);
  const long e = g.base + (long)k * a.NI;
  T acc[IN_N];
#pragma unroll
  for (int i = 0; i < IN_N; i++) acc[i] = T(0);
  const AdjIO<T, IN_N> io{a, j, acc};
  // the first-step graupel initialisation test of the column (as in prep)
  bool do_ginit = false;
  if ((a.flags & F_HAIL) && (a.flags & F_FIRST)) {
    T sqg = T(0), sng = T(0), sqb = T(0);
    for (int kk = 0; kk < a.nz; kk++) {
      const long ek = g.base + (long)kk * a.NI;
      sqg = sqg + a.qg[ek];
      sng = sng + a.ng[ek];
      sqb = sqb + a.qb[ek];
    }
    do_ginit = sqg > r1 && sng < eps && sqb < eps;
  }
  Lev<R> L;
  L.cs = &cst;
  L.ci = &ci;
  load_level(a, e, L, io);
  R ncsave = ncsave_of<R>(a, g);
  initial_checks(L, a.flags, ncsave, do_ginit, step_dt<R>(a), step_odt<R>(a));
  store_checked(a, e, L, io);
  // the checks overwrite the hydrometeor inputs; temperature and qv pass through
  for (int i = 0; i < IN_N; i++) {
    if (!input_present(a, i)) continue;
    T* slot = lam_slot(a, j, arr_of_in(i), e);
    if (!slot) continue;
    *slot = ((i == IN_T || i == IN_QV) ? *slot : T(0)) + acc[i];
  }
}

// ---------------------------------------------------------------------------------
// phase C adjoint: one thread per (level, active slot); primal arrays = the state after
// phase A, primal scratch = after sedimentation
// ---------------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(128) tempo_final_adjoint_kernel(
    const __grid_constant__ StepArgs<T> a, const __grid_constant__ TempoConsts<T> cst,
    const __grid_constant__ IslandConsts<Dual<T, C_N>> ci, const __grid_constant__ AdjArgs<T> j) {
  using R = Dual<T, C_N>;
  const long nact = (long)*a.nact;
  const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nact * a.nz) return;
  const int k = (int)(p / nact);
  const long s = p - (long)k * nact;
  T acc[C_N];
#pragma unroll
  for (int i = 0; i < C_N; i++) acc[i] = T(0);
  const AdjIO<T, C_N> io{a, j, acc};
  final_point<R, T>(a, cst, ci, k, s, io);
  const ColGeom g = col_geom(a, a.act[s]);
  const long e = g.base + (long)k * a.NI;
  const long cs = a.ncol_pad, fsd = (long)a.nz * cs, o = pt_off(s, k, a.nz);
  // state inputs: all overwritten by phase C (temperature and the checked species)
  constexpr int carr[14] = {A_T, -1, -1, -1, A_QC, A_NC, A_QR, A_NR, A_QI, A_NI, A_QS, A_QG, A_NG, A_QB};
  for (int i = 0; i < 14; i++) {
    if (carr[i] < 0) continue;
    if (carr[i] == A_NC && !(a.flags & F_NC)) continue;
    if ((carr[i] == A_NG || carr[i] == A_QB) && !(a.flags & F_HAIL)) continue;
    T* slot = lam_slot(a, j, carr[i], e);
    if (slot) *slot = acc[i];
  }
  // scratch inputs: accumulate (sedimentation adds to the density's adjoint later)
  j.lam_sd[SD_TTEN * fsd + o] += acc[C_TTEN];
  j.lam_sd[SD_QV * fsd + o] += acc[C_QV];
  j.lam_sd[SD_RHO * fsd + o] += acc[C_RHO];
  constexpr int tf[10] = {SD_TQR, SD_TNR, SD_TQG, SD_TNG, SD_TQB, SD_TQS, SD_TQI, SD_TNI, SD_TQC, SD_TNC};
#pragma unroll
  for (int i = 0; i < 10; i++) j.lam_sd[tf[i] * fsd + o] += acc[C_TQR + i];
}

// ---------------------------------------------------------------------------------
// phase B adjoint: one thread per active slot
// ---------------------------------------------------------------------------------
// the ten sedimenting fields, in SD order from SD_XRR, and their fall-speed fields
__device__ __forceinline__ int sed_vt(int f) {
  constexpr int m[10] = {SR_VTR, SR_VTNR, SR_VTG, SR_VTNG, SR_VTG, SR_VTSA, SR_VTI, SR_VTNI, SR_VTC, SR_VTNC};
  return m[f];
}

template <class T>
__global__ void __launch_bounds__(128) tempo_sedim_adjoint_kernel(
    const __grid_constant__ StepArgs<T> a, const __grid_constant__ AdjArgs<T> j, T* wbase,
    const __grid_constant__ SedWork W) {
  const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= (long)*a.nact) return;
  const int nz = a.nz;
  const long cs = a.ncol_pad, fsd = (long)nz * cs;
  const ColGeom g = col_geom(a, a.act[s]);
  const T* dzp = a.dz + g.base;
  const long NI = a.NI;
  const T dt = T(a.dt);
  T* w = wbase + s;
  auto WR = [&](long row) -> T& { return w[row * cs]; };
  auto rho = [&](int k) { return j.psd[SD_RHO * fsd + pt_off(s, k, nz)].v; };
  auto cand = [&](int f, int k) { return j.psr[(long)f * fsd + pt_off(s, k, nz)].v; };
  auto lsd = [&](int f, int k) -> T& { return j.lam_sd[(long)f * fsd + pt_off(s, k, nz)]; };
  auto lsr = [&](int f, int k) -> T& { return j.lam_sr[(long)f * fsd + pt_off(s, k, nz)]; };

  uint8_t any = 0;
  for (int k = 0; k < nz; k++) any |= a.pmask[pt_off(s, k, nz)];
  const bool any_qr = any & PM_QR, any_qg = any & PM_QG, any_qs = any & PM_QS,
             any_qi = any & PM_QI, any_qc = any & PM_QC;
  for (int f = 0; f < 10; f++)
    for (int k = 0; k < nz; k++) WR(W.xw(f, k, nz)) = j.psd[(long)(SD_XRR + f) * fsd + pt_off(s, k, nz)].v;

  // fill (forward): filled speeds into VF rows; steps and ktop as in the forward kernel
  auto fill = [&](int fv, int fvn, bool use_max, int& steps, int& ktop) {
    steps = 1;
    ktop = 1;
    T vup = T(0), vnup = T(0);
    for (int k = nz - 1; k >= 0; k--) {
      T v = cand(fv, k), vn = (fvn >= 0) ? cand(fvn, k) : T(0);
      if (v < T(0)) {
        v = vup;
        vn = vnup;
      }
      WR(W.vf(fv, k, nz)) = v;
      if (fvn >= 0) WR(W.vf(fvn, k, nz)) = vn;
      vup = v;
      vnup = vn;
      T vm = use_max ? (v > vn ? v : vn) : v;
      if (vm > T(1.e-3)) {
        ktop = max(ktop, k + 1);
        T dz_by_vt = T(dzp[k * NI]) / vm;
        steps = max(steps, (int)(dt / dz_by_vt + T(1.0)));
      }
    }
    if (ktop == nz) ktop = nz - 1;
  };
  auto fill_snow = [&](int& steps, int& ktop) {
    steps = 1;
    ktop = 1;
    T vup = T(0);
    for (int k = nz - 1; k >= 0; k--) {
      T A = cand(SR_VTSA, k), v;
      if (A >= T(0)) {
        if (cand(SR_VTSB, k) != T(0)) {
          T vrain = any_qr ? WR(W.vf(SR_VTR, k, nz)) : T(0);
          T rsk = WR(W.xw(SD_XRS - SD_XRR, k, nz));
          T srr = rsk / (rsk + WR(W.xw(0, k, nz)));
          v = A * srr + (T(1.0) - srr) * vrain;
        } else {
          v = A;
        }
      } else {
        v = vup;
      }
      WR(W.vf(SR_VTSA, k, nz)) = v;
      vup = v;
      if (v > T(1.e-3)) {
        ktop = max(ktop, k + 1);
        T dz_by_vt = T(dzp[k * NI]) / v;
        steps = max(steps, (int)(dt / dz_by_vt + T(1.0)));
      }
    }
    if (ktop == nz) ktop = nz - 1;
  };
  // one forward substep of field f (state rows at `row(k)`), fluxes from the pre-state
  auto sweep_fwd = [&](auto row, int vtf, T lim, int steps, int ktop) {
    const T osteps = T(1.0) / T(steps);
    int k = nz - 1;
    T s_top = WR(W.vf(vtf, k, nz)) * WR(row(k));
    T odz = T(1.0) / T(dzp[k * NI]);
    WR(row(k)) = max_t(lim, WR(row(k)) - s_top * odz * dt * osteps);
    T s_up = (ktop == nz - 1) ? s_top : WR(W.vf(vtf, ktop, nz)) * WR(row(ktop));
    for (k = ktop - 1; k >= 0; k--) {
      T s_k = WR(W.vf(vtf, k, nz)) * WR(row(k));
      odz = T(1.0) / T(dzp[k * NI]);
      WR(row(k)) = max_t(lim, WR(row(k)) + (s_up - s_k) * odz * dt * osteps);
      s_up = s_k;
    }
  };
  // reverse of one substep: pre-state in rows `pre(k)`, adjoints of the field in the
  // scratch adjoint of field f, fall speed vtf, tendency field tf, precipitation adjoint
  auto sweep_rev = [&](auto pre, int f, int vtf, int tf, T lim, int steps, int ktop, T lamP) {
    const T osteps = T(1.0) / T(steps);
    for (int k = 0; k < nz; k++) WR(W.ls(k, nz)) = T(0);
    const int top = nz - 1;
    auto xs = [&](int k) { return WR(pre(k)); };
    auto vv = [&](int k) { return WR(W.vf(vtf, k, nz)); };
    auto cx = [&](int k) { return (T(1.0) / T(dzp[k * NI])) * dt * osteps; };
    auto ct = [&](int k) { return (T(1.0) / T(dzp[k * NI])) * osteps * (T(1.0) / rho(k)); };
    const T s_top = vv(top) * xs(top);
    const T s_head = (ktop == nz - 1) ? s_top : vv(ktop) * xs(ktop);
    // precipitation: s0 * dt / steps when the post-substep x(0) exceeds the limit
    {
      const T s_up0 = (ktop - 1 == 0) ? s_head : vv(1) * xs(1);
      const T x0new = max_t(lim, xs(0) + (s_up0 - vv(0) * xs(0)) * cx(0));
      if (lamP != T(0) && x0new > T(low_limit_mass_for_precip))
        WR(W.ls(0, nz)) += lamP * dt * osteps;
    }
    T lam_head = T(0);
    for (int k = 0; k <= ktop - 1; k++) {
      // the level's factors once (the stores below may alias the loads for the compiler)
      const T cxk = cx(k), ctk = ct(k), rk = rho(k);
      const T s_k = vv(k) * xs(k);
      const T s_upk = (k == ktop - 1) ? s_head : vv(k + 1) * xs(k + 1);
      const T dflux = s_upk - s_k;
      const T xnew = xs(k) + dflux * cxk;
      const T gx = (lim > xnew) ? T(0) : lsd(f, k);
      const T lt = lsd(tf, k);
      const T gd = gx * cxk + lt * ctk;
      if (k == ktop - 1)
        lam_head += gd;
      else
        WR(W.ls(k + 1, nz)) += gd;
      WR(W.ls(k, nz)) -= gd;
      lsd(SD_RHO, k) += lt * dflux * (-ctk / rk);
      lsd(f, k) = gx;
    }
    {  // top level
      const T cxt = cx(top), ctt = ct(top), rt = rho(top);
      const T xnew = xs(top) - s_top * cxt;
      const T gx = (lim > xnew) ? T(0) : lsd(f, top);
      const T lt = lsd(tf, top);
      WR(W.ls(top, nz)) += -gx * cxt - lt * ctt;
      lsd(SD_RHO, top) += lt * s_top * ctt / rt;
      lsd(f, top) = gx;
    }
    if (ktop == nz - 1)
      WR(W.ls(top, nz)) += lam_head;
    else
      WR(W.ls(ktop, nz)) += lam_head;
    for (int k = 0; k < nz; k++) {
      const T l = WR(W.ls(k, nz));
      if (l == T(0)) continue;
      lsr(vtf, k) += l * xs(k);
      lsd(f, k) += l * vv(k);
    }
  };


  // ---- forward recompute, species by species, with checkpoints every 4 substeps ----
  const double glim = meters3_to_liters * r1 / rho_gd(nrhg);
  const int fr[2] = {0, 1}, fg[3] = {2, 3, 4}, fs[1] = {5}, fi[2] = {6, 7}, fc[2] = {8, 9};
  const T lr[2] = {T(r1), T(r2)}, lg[3] = {T(r1), T(r2), T(glim)}, ls1[1] = {T(r1)};
  int st_r = 0, kt_r = 0, st_g = 0, kt_g = 0, st_s = 0, kt_s = 0, st_i = 0, kt_i = 0, kt_c = 1;
  auto species_fwd = [&](int nf, const int* fl, const T* lim, int steps, int ktop, int nsweeps) {
    for (int n = 0; n < nsweeps; n++) {
      if (n % 4 == 0)
        for (int q = 0; q < nf; q++)
          for (int k = 0; k < nz; k++) WR(W.ck(fl[q], n / 4, k, nz)) = WR(W.xw(fl[q], k, nz));
      for (int q = 0; q < nf; q++)
        sweep_fwd([&](int k) { return W.xw(fl[q], k, nz); }, sed_vt(fl[q]), lim[q], steps, ktop);
    }
  };
  if (any_qr) {
    fill(SR_VTR, SR_VTNR, true, st_r, kt_r);
    species_fwd(2, fr, lr, st_r, kt_r, st_r);
  }
  if (any_qg) {
    fill(SR_VTG, SR_VTNG, false, st_g, kt_g);
    species_fwd(3, fg, lg, st_g, kt_g, st_g);
  }
  if (any_qs) {
    fill_snow(st_s, kt_s);
    species_fwd(1, fs, ls1, st_s, kt_s, st_s);
  }
  if (any_qi) {  // one substep with the substep count's weight (main:712-715)
    fill(SR_VTI, SR_VTNI, false, st_i, kt_i);
    species_fwd(2, fi, lr, st_i, kt_i, 1);
  }
  if (any_qc) {  // settles below 500 m only (main:1945-1977)
    T hgtc = T(0);
    for (int k = 1; k <= nz - 1; k++) {
      if (WR(W.xw(8, k - 1, nz)) > T(r2)) kt_c = k;
      hgtc = hgtc + T(dzp[(long)(k - 1) * NI]);
      if (hgtc > T(500.0)) break;
    }
    for (int k = 0; k < nz; k++) {
      WR(W.vf(SR_VTC, k, nz)) = (k < kt_c) ? cand(SR_VTC, k) : T(0);
      WR(W.vf(SR_VTNC, k, nz)) = (k < kt_c) ? cand(SR_VTNC, k) : T(0);
    }
    species_fwd(2, fc, lr, 1, kt_c, 1);
  }

  // ---- reverse ----
  auto species_rev = [&](int nf, const int* fl, const T* lim, int steps, int ktop, int nsweeps,
                         T lamP) {
    const int nb = (nsweeps + 3) / 4;
    for (int b = nb - 1; b >= 0; b--) {
      const int n0 = 4 * b, n1 = min(nsweeps, n0 + 4);
      for (int q = 0; q < nf; q++)
        for (int k = 0; k < nz; k++) WR(W.bb(q, 0, k, nz)) = WR(W.ck(fl[q], b, k, nz));
      for (int n = n0 + 1; n < n1; n++)
        for (int q = 0; q < nf; q++) {
          for (int k = 0; k < nz; k++) WR(W.bb(q, n - n0, k, nz)) = WR(W.bb(q, n - n0 - 1, k, nz));
          sweep_fwd([&](int k) { return W.bb(q, n - n0, k, nz); }, sed_vt(fl[q]), lim[q], steps, ktop);
        }
      for (int n = n1 - 1; n >= n0; n--)
        for (int q = 0; q < nf; q++)
          sweep_rev([&](int k) { return W.bb(q, n - n0, k, nz); }, SD_XRR + fl[q], sed_vt(fl[q]),
                    SD_TQR + fl[q], lim[q], steps, ktop, q == 0 ? lamP : T(0));
    }
  };
  // fill adjoint: the adjoint of a filled speed goes to its candidate, or, where the
  // level had none, to the filled speed above
  auto fill_rev = [&](int fv, int fvn) {
    for (int k = 0; k < nz; k++) {
      if (cand(fv, k) >= T(0)) continue;
      if (k + 1 < nz) {
        lsr(fv, k + 1) += lsr(fv, k);
        if (fvn >= 0) lsr(fvn, k + 1) += lsr(fvn, k);
      }
      lsr(fv, k) = T(0);
      if (fvn >= 0) lsr(fvn, k) = T(0);
    }
  };
  auto lamp = [&](int q) { return j.lam_precip[q] ? j.lam_precip[q][g.tile2] : T(0); };
  if (any_qc) {
    species_rev(2, fc, lr, 1, kt_c, 1, T(0));
    for (int k = kt_c; k < nz; k++) {
      lsr(SR_VTC, k) = T(0);
      lsr(SR_VTNC, k) = T(0);
    }
  }
  if (any_qi) {
    species_rev(2, fi, lr, st_i, kt_i, 1, lamp(1));
    fill_rev(SR_VTI, SR_VTNI);
  }
  if (any_qs) {
    species_rev(1, fs, ls1, st_s, kt_s, st_s, lamp(2));
    for (int k = 0; k < nz; k++) {
      const T A = cand(SR_VTSA, k);
      if (A >= T(0)) {
        if (cand(SR_VTSB, k) != T(0)) {  // v = A srr + (1 - srr) vrain, srr = rs / (rs + rr)
          const T l = lsr(SR_VTSA, k);
          const T vrain = any_qr ? WR(W.vf(SR_VTR, k, nz)) : T(0);
          const T rsk = j.psd[(long)SD_XRS * fsd + pt_off(s, k, nz)].v;
          const T rrk = WR(W.xw(0, k, nz));  // rain after its sedimentation
          const T srr = rsk / (rsk + rrk);
          lsr(SR_VTSA, k) = l * srr;
          const T lsrr = l * (A - vrain);
          if (any_qr) lsr(SR_VTR, k) += l * (T(1.0) - srr);
          const T den = (rsk + rrk) * (rsk + rrk);
          lsd(SD_XRS, k) += lsrr * rrk / den;
          lsd(SD_XRR, k) += -lsrr * rsk / den;
        }
      } else {
        if (k + 1 < nz) lsr(SR_VTSA, k + 1) += lsr(SR_VTSA, k);
        lsr(SR_VTSA, k) = T(0);
      }
    }
  }
  if (any_qg) {
    species_rev(3, fg, lg, st_g, kt_g, st_g, lamp(3));
    fill_rev(SR_VTG, SR_VTNG);
  }
  if (any_qr) {
    species_rev(2, fr, lr, st_r, kt_r, st_r, lamp(0));
    fill_rev(SR_VTR, SR_VTNR);
  }
}

}  // namespace tg
