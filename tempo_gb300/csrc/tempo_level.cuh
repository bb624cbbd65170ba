// tempo_level.cuh -- per-level microphysics of the TEMPO column step for sm_103a.
//
// Every routine of src/module_mp_tempo_main.F90 that is pointwise in k is written here
// as a device function on one level's scalar state (struct Lev).  The column kernel
// (tempo_step.cuh) sequences them and does the vertically coupled parts.
//
// Template parameter R is the bulk arithmetic type: double for the FP64 drop-in
// (every operation in the reference's order, compiled without FMA contraction) and
// float for the mixed form.  The thermodynamic island -- temperature, vapour,
// density, saturation mixing ratios, (super)saturations and the saturation
// adjustment -- has the island type Isl<R>: double in the FP64 drop-in, double-float
// (tempo_dfloat.cuh, ~48 bits on the FP32 pipes) in the mixed form.  Differences of
// nearly equal quantities (qv - qvs) decide condensation and must not lose digits.
#pragma once

#include <cstdint>
#include <type_traits>

#include "tempo_consts.h"
#include "tempo_dfloat.cuh"
#include "tempo_dual.cuh"
#include "tempo_powers.h"
#include "tempo_types.h"

namespace tg {

using D = double;

// island type of a bulk type
template <class R> struct IslandOf { using type = double; };
template <> struct IslandOf<float> { using type = df; };
// the tangent-linear / adjoint instantiations carry their own type as island
template <class T, int N> struct IslandOf<Dual<T, N>> { using type = Dual<T, N>; };
template <class R> using Isl = typename IslandOf<R>::type;
// scalar type of the constant sets and lookup tables of a bulk type
template <class R> struct ConstOf { using type = R; };
template <class T, int N> struct ConstOf<Dual<T, N>> { using type = T; };
template <class R> using Cst = typename ConstOf<R>::type;

// ---------------------------------------------------------------------------------
// math wrappers: accurate library functions for the chosen type (no fast-math)
// ---------------------------------------------------------------------------------
__device__ __forceinline__ double Pow(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float Pow(float x, float y) { return powf(x, y); }
// Powers with the reference's mass exponents (bm_r = bm_i = bm_g = 3, a parameter of
// the scheme): the size-distribution checks raise slopes to bm and form slopes as
// (...)**(1/bm), and (...)**(1/(bm_g+1)) for the graupel intercept -- about 10 of the
// 22 powers per level-point of a stretched-grid step.  The FP64 drop-in keeps the
// reference's real-exponent pow (x**bm_r is pow(x, 3.0) there); the mixed form forms
// them from products, cube and square roots, within a few rounding errors at a fraction
// of powf's code and time.  The exponent argument is the reference's constant (checked against
// the parameter at compile time for the cube; the roots take the context's 1/bm).
static_assert(bm_r == 3.0 && bm_i == 3.0 && bm_g == 3.0, "mass exponents of the scheme");
__device__ __forceinline__ double PowBm(double x) { return pow(x, 3.0); }
__device__ __forceinline__ float PowBm(float x) { return x * x * x; }
__device__ __forceinline__ double PowObm(double x, double obm) { return pow(x, obm); }
__device__ __forceinline__ float PowObm(float x, float) { return cbrtf(x); }
__device__ __forceinline__ double PowOge1(double x, double oge1) { return pow(x, oge1); }
__device__ __forceinline__ float PowOge1(float x, float) { return sqrtf(sqrtf(x)); }
// x**(S kCre[K]) and x**(S kCge[K]) (S = +1 or -1, tempo_powers.h): y is the same
// exponent as the context holds it, which the FP64 drop-in passes to pow as the
// reference does; the mixed form multiplies
template <int K, int S = 1> __device__ __forceinline__ double PowCre(double x, double y) { return pow(x, y); }
template <int K, int S = 1> __device__ __forceinline__ float PowCre(float x, float) {
  return pow_twice<FixedExp<kCre, K, S>::tw>(x);
}
template <int K, int S = 1> __device__ __forceinline__ double PowCge(double x, double y) { return pow(x, y); }
template <int K, int S = 1> __device__ __forceinline__ float PowCge(float x, float) {
  return pow_twice<FixedExp<kCge, K, S>::tw>(x);
}
// x**y where |y log2 x| is below 1 (the diffusivity's (T/t0)**1.94 with T/t0 within
// [0.7, 1.2]): the mixed form uses the hardware base-2 logarithm and exponential, whose
// error there is a few ulp; the FP64 drop-in keeps pow
__device__ __forceinline__ double PowNear1(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float PowNear1(float x, float y) { return __powf(x, y); }
__device__ __forceinline__ double Exp(double x) { return exp(x); }
__device__ __forceinline__ float Exp(float x) { return expf(x); }
__device__ __forceinline__ double Log(double x) { return log(x); }
__device__ __forceinline__ float Log(float x) { return logf(x); }
__device__ __forceinline__ double Log10(double x) { return log10(x); }
__device__ __forceinline__ float Log10(float x) { return log10f(x); }
__device__ __forceinline__ double Sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float Sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double Cos(double x) { return cos(x); }
__device__ __forceinline__ float Cos(float x) { return cosf(x); }
__device__ __forceinline__ double Fabs(double x) { return fabs(x); }
__device__ __forceinline__ float Fabs(float x) { return fabsf(x); }
__device__ __forceinline__ double Copysign(double a, double b) { return copysign(a, b); }
__device__ __forceinline__ float Copysign(float a, float b) { return copysignf(a, b); }
// 10**x: the FP64 drop-in keeps the reference's pow(10, x); the mixed form calls the
// library's exp10f (its documented error bound is below powf's)
__device__ __forceinline__ double Pow10(double x) { return pow(10.0, x); }
__device__ __forceinline__ float Pow10(float x) { return exp10f(x); }

// the same functions on dual numbers: values through the scalar functions above (so
// the value part matches the plain kernels), derivatives by the chain rule
template <class T, int N>
__device__ __forceinline__ Dual<T, N> Pow(const Dual<T, N>& a, const Dual<T, N>& b) {
  const T r = Pow(a.v, b.v);
  const T dfa = (a.v == T(0)) ? T(0) : b.v * r / a.v;
  const T dfb = (a.v > T(0)) ? r * Log(a.v) : T(0);
  Dual<T, N> o;
  o.v = r;
#pragma unroll
  for (int i = 0; i < N; i++) o.d[i] = dfa * a.d[i] + dfb * b.d[i];
  return o;
}
template <class T, int N, class U, class = typename std::enable_if<std::is_arithmetic<U>::value>::type>
__device__ __forceinline__ Dual<T, N> Pow(const Dual<T, N>& a, U b) {
  const T r = Pow(a.v, T(b));
  return dual_chain(a, r, (a.v == T(0)) ? T(0) : T(b) * r / a.v);
}
template <class T, int N, class U, class = typename std::enable_if<std::is_arithmetic<U>::value>::type>
__device__ __forceinline__ Dual<T, N> Pow(U a, const Dual<T, N>& b) {
  const T r = Pow(T(a), b.v);
  return dual_chain(b, r, (T(a) > T(0)) ? r * Log(T(a)) : T(0));
}
template <class T, int N>
__device__ __forceinline__ Dual<T, N> PowNear1(const Dual<T, N>& a, const Dual<T, N>& b) {
  return Pow(a, b);
}
template <class T, int N> __device__ __forceinline__ Dual<T, N> PowBm(const Dual<T, N>& a) {
  return Pow(a, 3.0);
}
template <class T, int N>
__device__ __forceinline__ Dual<T, N> PowObm(const Dual<T, N>& a, const Dual<T, N>& obm) {
  return Pow(a, obm);
}
template <class T, int N, class U, class = typename std::enable_if<std::is_arithmetic<U>::value>::type>
__device__ __forceinline__ Dual<T, N> PowObm(const Dual<T, N>& a, U obm) {
  return Pow(a, obm);
}
template <class T, int N, class U, class = typename std::enable_if<std::is_arithmetic<U>::value>::type>
__device__ __forceinline__ Dual<T, N> PowOge1(const Dual<T, N>& a, U oge1) {
  return Pow(a, oge1);
}
template <int K, int S = 1, class T, int N, class U,
          class = typename std::enable_if<std::is_arithmetic<U>::value>::type>
__device__ __forceinline__ Dual<T, N> PowCre(const Dual<T, N>& a, U y) {
  return Pow(a, y);
}
template <int K, int S = 1, class T, int N, class U,
          class = typename std::enable_if<std::is_arithmetic<U>::value>::type>
__device__ __forceinline__ Dual<T, N> PowCge(const Dual<T, N>& a, U y) {
  return Pow(a, y);
}
template <class T, int N> __device__ __forceinline__ Dual<T, N> Pow10(const Dual<T, N>& b) {
  return Pow(T(10.0), b);
}
template <class T, int N> __device__ __forceinline__ Dual<T, N> Exp(const Dual<T, N>& a) {
  const T r = Exp(a.v);
  return dual_chain(a, r, r);
}
template <class T, int N> __device__ __forceinline__ Dual<T, N> Log(const Dual<T, N>& a) {
  return dual_chain(a, Log(a.v), T(1) / a.v);
}
template <class T, int N> __device__ __forceinline__ Dual<T, N> Log10(const Dual<T, N>& a) {
  return dual_chain(a, Log10(a.v), T(0.43429448190325182765) / a.v);
}
template <class T, int N> __device__ __forceinline__ Dual<T, N> Sqrt(const Dual<T, N>& a) {
  const T r = Sqrt(a.v);
  return dual_chain(a, r, r > T(0) ? T(0.5) / r : T(0));
}
template <class T, int N> __device__ __forceinline__ Dual<T, N> Cos(const Dual<T, N>& a) {
  return dual_chain(a, Cos(a.v), -sin(a.v));
}
template <class T, int N> __device__ __forceinline__ Dual<T, N> Fabs(const Dual<T, N>& a) {
  return a.v < T(0) ? -a : a;
}
template <class T, int N>
__device__ __forceinline__ Dual<T, N> Copysign(const Dual<T, N>& a, const Dual<T, N>& b) {
  const T r = Copysign(a.v, b.v);
  return (r == a.v) ? a : -a;
}

// Fortran MAX/MIN on reals (first argument wins ties; no NaN special-casing)
template <class T> __device__ __forceinline__ T Max(T a, T b) { return a > b ? a : b; }
template <class T> __device__ __forceinline__ T Min(T a, T b) { return a < b ? a : b; }
template <class T> __device__ __forceinline__ T Max3(T a, T b, T c) { return Max(Max(a, b), c); }
template <class T> __device__ __forceinline__ T Min3(T a, T b, T c) { return Min(Min(a, b), c); }
// NINT: round half away from zero; INT: truncate toward zero
template <class T> __device__ __forceinline__ int Nint(T x) { return (int)round(x); }
template <class T> __device__ __forceinline__ int Int(T x) { return (int)x; }
template <class T, int N> __device__ __forceinline__ int Nint(const Dual<T, N>& x) { return Nint(x.v); }
template <class T, int N> __device__ __forceinline__ int Int(const Dual<T, N>& x) { return Int(x.v); }
// real ** integer: binary powering with a reciprocal for negative exponents
template <class T> __device__ __forceinline__ T Ipow(T x, int m) { return ipow_binary(x, m); }

// ---------------------------------------------------------------------------------
// constants and tables
// ---------------------------------------------------------------------------------
// The constant sets travel with each launch as __grid_constant__ kernel parameters
// (constant bank, no per-process global state); every level carries pointers to them.

template <class T> __device__ __forceinline__ T ld(const T* p) { return __ldg(p); }

// ---------------------------------------------------------------------------------
// per-level state
// ---------------------------------------------------------------------------------
template <class R>
struct Lev {
  using I = Isl<R>;
  const TempoConsts<Cst<R>>* cs;  // constant set of the bulk type
  const IslandConsts<I>* ci;  // constants of the thermodynamic island
  // prognostic "1d" values (after the initial checks) and hydrometeor state
  R qc1d, nc1d, qr1d, nr1d, qi1d, ni1d, qs1d, qg1d, ng1d, qb1d;
  bool l_qc, l_qr, l_qi, l_qs, l_qg;
  int idx_bg;
  R rc, nc, rr, nr, ri, ni, rs, rg, ng, rb, nwfa, nifa;
  R ilamc, ilami, ilamr, ilamg, mvd_c, mvd_r, mvd_g;
  R smob, smoc, smo0, smo1, smo2, smoe, smof, smog, smoz;
  // rain table indices of the process rates (get_rain_table_index, main:2526-2555),
  // which three rate routines use with the same rain state: formed at the first use
  // (0 = not yet)
  mutable int rain_idx = 0, rain_idx1 = 0;
  // size-distribution powers that several rate routines form from the same rain and
  // graupel state (graupel intercept and the 9th collection power, rain intercept and
  // the 9th collection power): formed at the first use (bits of psd_have); the rate
  // stage drops them and the rain indices when it ends, before the state changes
  mutable R psd_n0g, psd_pg9, psd_n0r, psd_pf9;
  mutable int psd_have = 0;
  // thermodynamic island
  I t1d, qv1d, temp, qv, rho, qvs, qvsi, delqvs, ssatw, ssati, tten, qvten;
  I qvs_t0;  // calc_rslf(p, t0): pressure is fixed through the step, so once per level
  R pres;
  R rhof, rhof2, diffu, visco, vsc2, tcond, lvap, ocp, lvt2;
  R qcten, ncten, qiten, niten, qrten, nrten, qsten, qgten, ngten, qbten, nwfaten, nifaten;
  // magnitudes of the terms summed into each tendency (sums of absolute values; used by
  // the mixed form only, see updated())
  Cst<R> qcmag = 0, ncmag = 0, qimag = 0, nimag = 0, qrmag = 0, nrmag = 0, qsmag = 0, qgmag = 0,
         ngmag = 0, qbmag = 0;
  R vtboost;
#ifdef TEMPO_TRACE
  int* tr = nullptr;  // this point's decision-trace record (TraceSlot), NULL = off
  int tpass = 0;      // pass of the check routines (TR_CHECK + tpass)
#endif
};

// decision trace of a test build: OR bits into a slot of the level's record
#ifdef TEMPO_TRACE
#define TG_TRACE(L, slot, bits)                    \
  do {                                             \
    if ((L).tr) (L).tr[(slot)] |= (int)(bits);     \
  } while (0)
#define TG_TRACE_PASS(L, p) ((L).tpass = (p))
// index v of a table read must lie in [lo, hi]: outside, the site's bit goes to the
// point's TR_RANGE slot and v is clamped, so the read stays inside the table
#define TG_RANGE(L, site, v, lo, hi)                 \
  do {                                               \
    if ((v) < (lo) || (v) > (hi)) {                  \
      if ((L).tr) (L).tr[TR_RANGE] |= (int)(site);   \
      (v) = (v) < (lo) ? (lo) : (hi);                \
    }                                                \
  } while (0)
#else
#define TG_TRACE(L, slot, bits) \
  do {                          \
  } while (0)
#define TG_TRACE_PASS(L, p) ((void)0)
#define TG_RANGE(L, site, v, lo, hi) ((void)0)
#endif

// process rates (ty_tend, main:47-64)
template <class R>
struct Tend {
  R prr_wau, pnr_wau, pnc_wau, prr_rcw, pnc_rcw, pnr_rcr;
  R prs_scw, pnc_scw, png_scw, pbg_scw, prg_gcw, pnc_gcw, pbg_gcw, pri_ihm, pni_ihm, prs_ihm,
      prg_ihm, prg_scw;
  R prr_rcs, pnr_rcs, prg_rcs, png_rcs, prs_rcs, pbg_rcs;
  R prr_rcg, pnr_rcg, prg_rcg, png_rcg, pbg_rcg;
  R pri_inu, pni_inu, pri_iha, pni_iha;
  R pri_wfz, pni_wfz;
  R prg_rfz, png_rfz, pnr_rfz, pri_rfz, pni_rfz, pbg_rfz;
  R prs_sde, pri_ide, pni_ide, prs_ide, prg_gde, png_gde;
  R pni_iau, prs_iau;
  R prr_sml, prr_gml, pbg_sml, pbg_gml, pnr_sml, pnr_gml;
  R prr_rci, pnr_rci, pri_rci, pni_rci, prg_rci, png_rci, pbg_rci;
  R pni_sci, prs_sci;
  R prw_vcd, pnc_wcd, prv_rev, pnr_rev;
  R pna_rca, pna_sca, pna_gca, pnd_rcd, pnd_scd, pnd_gcd;
};

__device__ __forceinline__ D rho_gd(int m) {  // rho_g (params:143-144), 1-based
  return m == 1 ? 50. : m == 2 ? 100. : m == 3 ? 200. : m == 4 ? 300. : m == 5 ? 400.
         : m == 6 ? 500. : m == 7 ? 600. : m == 8 ? 700. : 800.;
}
template <class R> __device__ __forceinline__ R rho_g(int m) { return R(rho_gd(m)); }

// ---------------------------------------------------------------------------------
// utils.F90
// ---------------------------------------------------------------------------------
// One Horner step c + x s in the island type (the double-float form has its own,
// tempo_dfloat.cuh), and the nested polynomial c0 + x (c1 + x (c2 + ...)) in the
// reference's order.
template <class I> __device__ __forceinline__ I horner_step(I x, I s, double c) { return c + x * s; }
template <class I> __device__ __forceinline__ I horner(I, double c) { return I(c); }
template <class I, class... Cs>
__device__ __forceinline__ I horner(I x, double c, Cs... cs) {
  return horner_step(x, horner(x, cs...), c);
}

// calc_rslf / calc_rsif (utils:285-331) in the island type
template <class I> __device__ __forceinline__ I calc_rslf(I p, I t) {
  I x = Max(I(-80.0), t - 273.16);
  I esl = horner(x, .611583699E03, .444606896E02, .143177157e01, .264224321e-1, .299291081e-3,
                 .203154182e-5, .702620698e-8, .379534310e-11, -.321582393e-13);
  esl = Min(esl, p * 0.15);
  return .622 * esl / (p - esl);
}
template <class I> __device__ __forceinline__ I calc_rsif(I p, I t) {
  I x = Max(I(-80.0), t - 273.16);
  I esi = horner(x, .609868993e03, .499320233e02, .184672631e01, .402737184e-1, .565392987e-3,
                 .521693933e-5, .307839583e-7, .105785160e-9, .161444444e-12);
  esi = Min(esi, p * 0.15);
  return .622 * esi / Max(I(1.e-4), (p - esi));
}

template <class R> __device__ __forceinline__ int get_nuc(R nc) {  // utils:334-346
  if ((R(nu_c_scale) / nc) >= R(12.5)) return 15;
  int v = Nint(R(nu_c_scale) / nc) + 2;
  return v < 15 ? v : 15;
}

template <class C, class R, class XT>
__device__ __forceinline__ R poly_a(const C* s, R tc, XT Xin) {
  const R X = R(Xin);  // utils:190-199
  return s[0] + s[1] * tc + s[2] * X + s[3] * tc * X + s[4] * tc * tc + s[5] * X * X +
         s[6] * tc * tc * X + s[7] * tc * X * X + s[8] * tc * tc * tc + s[9] * X * X * X;
}

// snow_moments (utils:148-282).  which: 0 = smob/smoc/smo2, 1 = + ns/smo0/smo1/smoe/
// smof/smog (initial), 2 = + smoz (final).
template <class R>
__device__ void snow_moments(Lev<R>& L, R tc, int which) {
  const TempoConsts<Cst<R>>& c = *L.cs;
  R loga_, a_, b_, smo2_;
  L.smob = L.rs * c.oams;
  loga_ = poly_a(c.sa, tc, R(bm_s));
  a_ = Pow10(loga_);
  b_ = poly_a(c.sb, tc, R(bm_s));
  smo2_ = Pow(L.smob / a_, R(1.0) / b_);
  L.smo2 = smo2_;
  loga_ = poly_a(c.sa, tc, c.cse[0]);
  a_ = Pow10(loga_);
  b_ = poly_a(c.sb, tc, c.cse[0]);
  L.smoc = a_ * Pow(smo2_, b_);
  if (which == 1) {
    const auto* sa = c.sa;
    const auto* sb = c.sb;
    loga_ = sa[0] + sa[1] * tc + sa[4] * tc * tc + sa[8] * tc * tc * tc;
    a_ = Pow10(loga_);
    b_ = sb[0] + sb[1] * tc + sb[4] * tc * tc + sb[8] * tc * tc * tc;
    L.smo0 = a_ * Pow(smo2_, b_);
    loga_ = sa[0] + sa[1] * tc + sa[2] + sa[3] * tc + sa[4] * tc * tc + sa[5] + sa[6] * tc * tc +
            sa[7] * tc + sa[8] * tc * tc * tc + sa[9];
    a_ = Pow10(loga_);
    b_ = sb[0] + sb[1] * tc + sb[2] + sb[3] * tc + sb[4] * tc * tc + sb[5] + sb[6] * tc * tc +
         sb[7] * tc + sb[8] * tc * tc * tc + sb[9];
    L.smo1 = a_ * Pow(smo2_, b_);
    loga_ = poly_a(sa, tc, c.cse[12]);
    a_ = Pow10(loga_);
    b_ = poly_a(sb, tc, c.cse[12]);
    L.smoe = a_ * Pow(smo2_, b_);
    loga_ = poly_a(sa, tc, c.cse[15]);
    a_ = Pow10(loga_);
    b_ = poly_a(sb, tc, c.cse[15]);
    L.smof = a_ * Pow(smo2_, b_);
    loga_ = poly_a(sa, tc, c.cse[16]);
    a_ = Pow10(loga_);
    b_ = poly_a(sb, tc, c.cse[16]);
    L.smog = a_ * Pow(smo2_, b_);
  } else if (which == 2) {
    loga_ = poly_a(c.sa, tc, c.cse[2]);
    a_ = Pow10(loga_);
    b_ = poly_a(c.sb, tc, c.cse[2]);
    L.smoz = a_ * Pow(smo2_, b_);
  }
}

// ---------------------------------------------------------------------------------
// check_and_update routines (main:867-1260), one level
// ---------------------------------------------------------------------------------
// A value updated by its tendency, q + ten * dt, as the existence and clipping tests of
// the check routines see it.  Where a step uses a species up completely -- a sink capped
// at q / dt, or scaled by the over-depletion limiter to exactly what is there, or a
// source used up by a sink in the same step -- the sum cancels: FP64 leaves about 1e-16
// of the terms, far below the existence thresholds (r1 for masses, r2 or the minimum
// number for numbers), and takes the species as gone.  FP32 leaves a few 1e-8 of the
// terms, which can pass them.  So in the mixed form a sum within kCancelUlps rounding
// units of its terms counts as cancelled (zero), and the decision is the one FP64 takes;
// a value so close to zero is at the rounding level of the terms either way.  The terms'
// scale is the larger of |q| + |ten dt| and |q| + mag dt, mag being the sum of the
// magnitudes of the rates summed into ten.  The FP64 drop-in keeps the reference's sum.
constexpr float kCancelUlps = 32.0f;
template <class T> __device__ __forceinline__ T mag(T x) { return Fabs(x); }
template <class T, int N> __device__ __forceinline__ T mag(const Dual<T, N>& x) { return Fabs(x.v); }
template <class R>
__device__ __forceinline__ R updated(R q, R ten, R dt, Cst<R> tmag = Cst<R>(0)) {
  const R tdt = ten * dt;
  const R v = q + tdt;
  if constexpr (std::is_same<Cst<R>, float>::value) {
    const float scale = mag(q) + Max(mag(tdt), tmag * mag(dt));
    if (mag(v) <= kCancelUlps * 5.9604645e-8f * scale) return R(0.0f);
  }
  return v;
}

// The size clamps of the check routines (cloud, rain, ice and graupel diameters).  A later
// pass re-checks a state that an earlier pass clamped: the diameter then comes out at the
// clamp to within rounding, and the limit is taken again or not by the last bits (FP64
// takes it again; both branches give the same state to rounding).  In the mixed form a
// diameter within kTieUlps rounding units of its clamp counts as at the clamp, so that it
// takes the limit as FP64 does.  The FP64 drop-in keeps the reference's comparisons.
constexpr float kTieUlps = 16.0f;
template <class R> __device__ __forceinline__ bool over_clamp(R x, R bound) {
  if constexpr (std::is_same<Cst<R>, float>::value)
    return x > bound * R(1.0f - kTieUlps * 5.9604645e-8f);
  else
    return x > bound;
}
template <class R> __device__ __forceinline__ bool under_clamp(R x, R bound) {
  if constexpr (std::is_same<Cst<R>, float>::value)
    return x < bound * R(1.0f + kTieUlps * 5.9604645e-8f);
  else
    return x < bound;
}

// the magnitudes of a level's tendencies start at zero (no rate summed yet)
template <class R> __device__ __forceinline__ void clear_mags(Lev<R>& L) {
  L.qcmag = L.ncmag = L.qimag = L.nimag = L.qrmag = L.nrmag = L.qsmag = L.qgmag = L.ngmag =
      L.qbmag = Cst<R>(0);
}
template <class R>
__device__ __forceinline__ void aerosol_check(Lev<R>& L, uint32_t f, R dt) {  // main:867-888
  R rho = R(L.rho);
  if (f & F_NWFA) L.nwfa = (L.nwfa + L.nwfaten * dt) * rho;  // nwfa holds nwfa1d on entry
  if (f & F_NIFA) L.nifa = (L.nifa + L.nifaten * dt) * rho;
  L.nwfa = Max(R(nwfa_default) * rho, Min(R(aero_max) * rho, L.nwfa));
  L.nifa = Max(R(nifa_default) * rho, Min(R(aero_max) * rho, L.nifa));
}

// cloud_check_and_update (main:891-973) on (q, n) = (qc1d, nc1d) or temporaries
template <class R>
__device__ void cloud_check(Lev<R>& L, R& q, R& n, bool has_nc, R ncsave, R dt, R odt) {
  const TempoConsts<Cst<R>>& c = *L.cs;
  R rho = R(L.rho);
  bool hit_limit = false;
  int nu_c;
  R lamc, xdc;
  const R qn = updated(q, L.qcten, dt, L.qcmag);
  if (qn > R(r1)) {
    L.l_qc = true;
    L.rc = qn * rho;
    q = qn;
    if (has_nc) {
      L.nc = Max(R(nt_c_min), updated(n, L.ncten, dt, L.ncmag) * rho);
      if (L.nc <= R(nt_c_min)) {
        hit_limit = true;
        L.nc = R(nt_c_min);
      }
      if (L.nc > R(nt_c_max)) {
        hit_limit = true;
        L.nc = R(nt_c_max);
      }
      nu_c = get_nuc(L.nc);
      lamc = PowObm(L.nc * c.am_r * c.ccg[nu_c - 1][1] * c.ocg1[nu_c - 1] / L.rc, c.obmr);
      xdc = (R(bm_r) + R(nu_c) + R(1.0)) / lamc;
      if (under_clamp(xdc, R(d0c))) {
        lamc = c.cce[nu_c - 1][1] / R(d0c);
        hit_limit = true;
      } else if (over_clamp(xdc, R(d0r) * R(2.0))) {
        lamc = c.cce[nu_c - 1][1] / (R(d0r) * R(2.0));
        hit_limit = true;
      }
      L.nc = c.ccg[nu_c - 1][0] * c.ocg2[nu_c - 1] * L.rc / c.am_r * PowBm(lamc);
      if (hit_limit) L.ncten = (L.nc / rho - n) * odt;
      n = Max(R(nt_c_min) / rho,
              Min(c.ccg[nu_c - 1][0] * c.ocg2[nu_c - 1] * q / c.am_r * PowBm(lamc),
                  R(nt_c_max) / rho));
    } else {
      L.nc = ncsave;
    }
    nu_c = get_nuc(L.nc);
    lamc = PowObm(L.nc * c.am_r * c.ccg[nu_c - 1][1] * c.ocg1[nu_c - 1] / L.rc, c.obmr);
    L.ilamc = R(1.0) / lamc;
    L.mvd_c = Max(Min((R(3.0) + R(nu_c) + R(0.672)) * L.ilamc, R(d0r)), R(d0c));
    TG_TRACE(L, TR_CHECK + L.tpass, TB_QC | (hit_limit ? TB_QC_HIT : 0) | (nu_c << 16));
  } else {
    L.l_qc = false;
    L.rc = R(r1);
    L.nc = R(nt_c_min);
    L.mvd_c = R(d0c);
    L.ilamc = R(0.0);
    L.qcten = -q * odt;
    q = R(0.0);
    if (has_nc) {
      L.ncten = -n * odt;
      n = R(0.0);
    }
  }
}

// rain_check_and_update (main:976-1042)
template <class R>
__device__ void rain_check(Lev<R>& L, R& q, R& n, R dt, R odt) {
  const TempoConsts<Cst<R>>& c = *L.cs;
  R rho = R(L.rho);
  bool hit_limit = false;
  R lamr;
  const R qn = updated(q, L.qrten, dt, L.qrmag);
  if (qn > R(r1)) {
    L.l_qr = true;
    L.rr = qn * rho;
    q = qn;
    L.nr = Max(R(r2), updated(n, L.nrten, dt, L.nrmag) * rho);
    if (L.nr <= R(r2)) {
      hit_limit = true;
      L.mvd_r = R(1.0e-3);
      lamr = (R(3.0) + R(mu_r) + R(0.672)) / L.mvd_r;
      L.nr = c.crg[1] * c.org3 * L.rr * PowBm(lamr) / c.am_r;
    }
    lamr = PowObm(c.am_r * c.crg[2] * c.org2 * L.nr / L.rr, c.obmr);
    L.mvd_r = (R(3.0) + R(mu_r) + R(0.672)) / lamr;
    if (over_clamp(L.mvd_r, R(d0r_max))) {
      hit_limit = true;
      L.mvd_r = R(d0r_max);
      lamr = (R(3.0) + R(mu_r) + R(0.672)) / L.mvd_r;
      L.nr = c.crg[1] * c.org3 * L.rr * PowBm(lamr) / c.am_r;
    } else if (under_clamp(L.mvd_r, R(d0r) * R(0.75))) {
      hit_limit = true;
      L.mvd_r = R(d0r) * R(0.75);
      lamr = (R(3.0) + R(mu_r) + R(0.672)) / L.mvd_r;
      L.nr = c.crg[1] * c.org3 * L.rr * PowBm(lamr) / c.am_r;
    }
    if (hit_limit) L.nrten = (L.nr / rho - n) * odt;
    n = c.crg[1] * c.org3 * q * PowBm(lamr) / c.am_r;
    L.ilamr = R(1.0) / lamr;
    TG_TRACE(L, TR_CHECK + L.tpass, TB_QR | (hit_limit ? TB_QR_HIT : 0));
  } else {
    L.l_qr = false;
    L.rr = R(r1);
    L.nr = R(r2);
    L.mvd_r = R(d0r);
    L.ilamr = R(0.0);
    L.qrten = -q * odt;
    L.nrten = -n * odt;
    q = R(0.0);
    n = R(0.0);
  }
}

// ice_check_and_update (main:1045-1107)
template <class R>
__device__ void ice_check(Lev<R>& L, R& q, R& n, R dt, R odt) {
  const TempoConsts<Cst<R>>& c = *L.cs;
  R rho = R(L.rho);
  bool hit_limit = false;
  R lami, xdi;
  const R qn = updated(q, L.qiten, dt, L.qimag);
  if (qn > R(r1)) {
    L.l_qi = true;
    L.ri = qn * rho;
    q = qn;
    L.ni = Max(R(r2), updated(n, L.niten, dt, L.nimag) * rho);
    if (L.ni <= R(r2)) {
      hit_limit = true;
      lami = c.cie[1] / R(5.e-6);
      L.ni = Min(R(max_ni), c.cig[0] * c.oig2 * L.ri / c.am_i * PowBm(lami));
    }
    lami = PowObm(c.am_i * c.cig[1] * c.oig1 * L.ni / L.ri, c.obmi);
    xdi = (R(bm_i) + R(mu_i) + R(1.0)) / lami;
    if (under_clamp(xdi, R(5.e-6))) {
      hit_limit = true;
      lami = c.cie[1] / R(5.e-6);
      L.ni = Min(R(max_ni), c.cig[0] * c.oig2 * L.ri / c.am_i * PowBm(lami));
    } else if (over_clamp(xdi, R(d0s))) {
      hit_limit = true;
      lami = c.cie[1] / R(d0s);
      L.ni = c.cig[0] * c.oig2 * L.ri / c.am_i * PowBm(lami);
    }
    if (hit_limit) L.niten = (L.ni / rho - n) * odt;
    n = Max(R(r2) / rho, Min(c.cig[0] * c.oig2 * q / c.am_i * PowBm(lami), R(max_ni) / rho));
    L.ilami = R(1.0) / lami;
    TG_TRACE(L, TR_CHECK + L.tpass, TB_QI | (hit_limit ? TB_QI_HIT : 0));
  } else {
    L.l_qi = false;
    L.ri = R(r1);
    L.ni = R(r2);
    L.ilami = R(0.0);
    L.qiten = -q * odt;
    L.niten = -n * odt;
    q = R(0.0);
    n = R(0.0);
  }
}

// snow_check_and_update (main:1110-1134)
template <class R>
__device__ __forceinline__ void snow_check(Lev<R>& L, R& q, R dt, R odt) {
  R rho = R(L.rho);
  const R qn = updated(q, L.qsten, dt, L.qsmag);
  if (qn > R(r1)) {
    L.l_qs = true;
    L.rs = qn * rho;
    q = qn;
    TG_TRACE(L, TR_CHECK + L.tpass, TB_QS);
  } else {
    L.l_qs = false;
    L.rs = R(r1);
    L.qsten = -q * odt;
    q = R(0.0);
  }
}

// Graupel density class nint(10 rg / rb) + 1 in [1, nrhg] (main:1171, 1200).  Where rb
// sits at its low-density clamp rg * 1000 / rho_g(1) the ratio is rho_g(1) / 100 = 0.5
// exactly, a rounding tie of nint.  The FP64 drop-in evaluates the ratio as the
// reference does (the tie then resolves by the last bit of rg); the mixed form, whose
// FP32 rg carries no such bit, takes the exact ratio's class, nint(0.5) + 1 = 2.
template <class R>
__device__ __forceinline__ int density_class(R ratio, R rb, R rb_lowdens_clamp) {
  if constexpr (sizeof(R) == sizeof(float)) {
    if (!(rb < rb_lowdens_clamp)) return 2;
  }
  return max(1, min(Nint(ratio) + 1, nrhg));
}

// graupel_check_and_update (main:1137-1231)
template <class R>
__device__ void graupel_check(Lev<R>& L, R& q, R& n, R& b, bool hail, R dt, R odt) {
  const TempoConsts<Cst<R>>& c = *L.cs;
  R rho = R(L.rho);
  bool hit_limit = false;
  R lamg;
  const R qn = updated(q, L.qgten, dt, L.qgmag);
  if (qn > R(r1)) {
    L.l_qg = true;
    L.rg = qn * rho;
    q = qn;
    if (hail) {
      L.ng = Max(R(r2), updated(n, L.ngten, dt, L.ngmag) * rho);
      const R rb_hi = L.rg * R(meters3_to_liters) / rho_g<R>(1);
      L.rb = Min(Max(L.rg * R(meters3_to_liters) / rho_g<R>(nrhg), updated(b, L.qbten, dt, L.qbmag) * rho), rb_hi);
      L.idx_bg = density_class(R(10.0) * L.rg / L.rb, L.rb, rb_hi);
      const int ig = L.idx_bg;
      if (L.ng <= R(r2)) {
        hit_limit = true;
        L.mvd_g = R(1.5e-3);
        lamg = (R(3.0) + R(mu_g) + R(0.672)) / L.mvd_g;
        L.ng = c.cgg[0][1] * c.ogg3 * L.rg * PowBm(lamg) / c.am_g[ig - 1];
      }
      lamg = PowObm(c.am_g[ig - 1] * c.cgg[0][2] * c.ogg2 * L.ng / L.rg, c.obmg);
      L.mvd_g = (R(3.0) + R(mu_g) + R(0.672)) / lamg;
      if (over_clamp(L.mvd_g, R(25.4e-3))) {
        hit_limit = true;
        L.mvd_g = R(25.4e-3);
        lamg = (R(3.0) + R(mu_g) + R(0.672)) / L.mvd_g;
        L.ng = c.cgg[0][1] * c.ogg3 * L.rg * PowBm(lamg) / c.am_g[ig - 1];
      } else if (under_clamp(L.mvd_g, R(d0r))) {
        hit_limit = true;
        L.mvd_g = R(d0r);
        lamg = (R(3.0) + R(mu_g) + R(0.672)) / L.mvd_g;
        L.ng = c.cgg[0][1] * c.ogg3 * L.rg * PowBm(lamg) / c.am_g[ig - 1];
      }
      if (hit_limit) L.ngten = (L.ng / rho - n) * odt;
      n = c.cgg[0][1] * c.ogg3 * q * PowBm(lamg) / c.am_g[ig - 1];
      const R b_hi = R(meters3_to_liters) * q / rho_g<R>(1);
      b = Min(Max(q * R(meters3_to_liters) / rho_g<R>(nrhg), updated(b, L.qbten, dt, L.qbmag)), b_hi);
      L.idx_bg = density_class(R(10.0) * q / b, b, b_hi);
    } else {
      L.idx_bg = idx_bg1;
      R ygra1 = Log10(Max(R(1.e-9), L.rg));
      R zans1 = R(3.4) + R(2.0 / 7.0) * (ygra1 + R(8.0));
      R n0_exp = Max(R(gonv_min), Min(Pow10(zans1), R(gonv_max)));
      R lam_exp = PowOge1(n0_exp * c.am_g[idx_bg1 - 1] * c.cgg[0][0] / L.rg, c.oge1);
      lamg = lam_exp * c.graupel_lam_k;
      L.ng = c.cgg[0][1] * c.ogg3 * L.rg * PowBm(lamg) / c.am_g[idx_bg1 - 1];
      L.rb = R(meters3_to_liters) * L.rg / rho_g<R>(idx_bg1);
    }
    L.ilamg = R(1.0) / lamg;
    L.mvd_g = (R(3.0) + R(mu_g) + R(0.672)) * L.ilamg;
    TG_TRACE(L, TR_CHECK + L.tpass, TB_QG | (hit_limit ? TB_QG_HIT : 0) | (L.idx_bg << 12));
  } else {
    L.l_qg = false;
    L.rg = R(r1);
    L.ng = R(r2);
    L.mvd_g = R(d0g);
    L.ilamg = R(0.0);
    L.idx_bg = idx_bg1;
    L.rb = R(meters3_to_liters) * R(r1) / rho_g<R>(idx_bg1);
    L.qgten = -q * odt;
    q = R(0.0);
    if (hail) {
      L.ngten = -n * odt;
      L.qbten = -b * odt;
      n = R(0.0);
      b = R(0.0);
    }
  }
}

// graupel_init (main:1234-1260) for one level
template <class R>
__device__ __forceinline__ void graupel_init(Lev<R>& L) {
  const TempoConsts<Cst<R>>& c = *L.cs;
  if (L.qg1d > R(r1)) {
    R rho = R(L.rho);
    R rg = L.qg1d * rho;
    R rb = rg * R(meters3_to_liters) / rho_g<R>(idx_bg1);
    int idx = max(1, min(Nint(R(10.0) * rg / rb) + 1, nrhg));
    R mvd_g = R(5.e-3);
    R lamg = (R(3.0) + R(mu_g) + R(0.672)) / mvd_g;
    R ng = c.cgg[0][1] * c.ogg3 * rg * PowBm(lamg) / c.am_g[idx - 1];
    L.ng1d = ng / rho;
    L.qb1d = rb / rho;
  }
}

// thermo_vars (main:1263-1310) for one level.  kIce = false leaves out the ice
// saturation (qvsi, ssati) and delqvs: their readers -- nucleation, ice processes,
// melting and the over-depletion limiter -- all run in the first stage of phase A, so
// the calls before saturation adjustment and rain evaporation need them not (the
// fields keep the first stage's values, which nothing reads again).
template <class R, bool kIce = true>
__device__ void thermo(Lev<R>& L) {
  using I = Isl<R>;
  I otemp = 1.0 / L.temp;
  I tempc = L.temp - t0;
  L.rhof = R(Sqrt(L.ci->rho_not / L.rho));
  L.rhof2 = Sqrt(L.rhof);
  L.qvs = calc_rslf(I(L.pres), L.temp);
  I satw = L.qv / L.qvs;
  L.ssatw = satw - 1.0;
  if (Fabs(L.ssatw) < eps) L.ssatw = I(0.0);
  if constexpr (kIce) {
    L.delqvs = Max(I(0.0), L.qvs_t0 - L.qv);
    if (tempc <= 0.0)
      L.qvsi = calc_rsif(I(L.pres), L.temp);
    else
      L.qvsi = L.qvs;
    I sati = L.qv / L.qvsi;
    L.ssati = sati - 1.0;
    if (Fabs(L.ssati) < eps) L.ssati = I(0.0);
  }
  R rtc = R(tempc);
  L.diffu = R(2.11e-5) * PowNear1(R(L.temp / t0), R(1.94)) * (R(101325.0) / L.pres);
  if (tempc >= 0.0)
    L.visco = (R(1.718) + R(0.0049) * rtc) * R(1.0e-5);
  else
    L.visco = (R(1.718) + R(0.0049) * rtc - R(1.2e-5) * rtc * rtc) * R(1.0e-5);
  // multiplicative factors: the bulk type suffices (they scale, never cancel)
  R ocp = R(1.0) / (R(cp) * (R(1.0) + R(0.887) * R(L.qv)));
  L.ocp = ocp;
  L.vsc2 = Sqrt(R(L.rho) / L.visco);
  R lvap = R(lvap0) + (R(2106.0) - R(4218.0)) * rtc;
  L.lvap = lvap;
  L.tcond = (R(5.69) + R(0.0168) * rtc) * R(1.0e-5) * R(418.936);
  L.lvt2 = lvap * lvap * ocp * R(L.ci->orv) * R(otemp) * R(otemp);
}

// The part of thermo_vars that the fall speeds read after the last stage of phase A
// (rhof; visco for the density-dependent graupel speed), computed exactly as thermo
// does; the other fields of the last thermo_vars call have no reader.
template <class R>
__device__ __forceinline__ void thermo_tail(Lev<R>& L) {
  using I = Isl<R>;
  I tempc = L.temp - t0;
  L.rhof = R(Sqrt(L.ci->rho_not / L.rho));
  R rtc = R(tempc);
  if (tempc >= 0.0)
    L.visco = (R(1.718) + R(0.0049) * rtc) * R(1.0e-5);
  else
    L.visco = (R(1.718) + R(0.0049) * rtc - R(1.2e-5) * rtc * rtc) * R(1.0e-5);
}

template <class I>
__device__ __forceinline__ I rho_of(const IslandConsts<I>& ci, I pres, I temp, I qv) {  // main:325
  return ci.roverrv * pres / (rdry * temp * (qv + ci.roverrv));
}

}  // namespace tg
