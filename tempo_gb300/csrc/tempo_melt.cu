// tempo_melt.cu -- melting-layer 10-cm reflectivity (refl10cm_from_melting_flag,
// src/module_mp_tempo_diags.F90:59-395), a pass after phase C.
//
// The reference replaces the snow and graupel contributions to Ze by those of melting
// particles on the levels below the melting level of the column (find_melting_level),
// so the pass needs the whole column: phase C leaves, per point, the three dry
// contributions and the state the melting formulas read (the record of MeltVal), and one
// thread per active column finds the melting level and rewrites refl10cm where it
// applies.  The melting formulas (Maxwell-Garnett mixing of ice, water and air and the
// Rayleigh backscatter over 50 radar bins) run in FP64 in both precision forms; they
// touch only the levels below a melting level.
#include "tempo_internal.h"
#include "tempo_step.cuh"

namespace tg {

namespace {

constexpr double kLambdaRadar = 0.10;  // m
constexpr double kMeltOutside = 0.9;

struct cd {  // complex double
  double re, im;
};
__device__ __forceinline__ cd mk(double r, double i) { return cd{r, i}; }
__device__ __forceinline__ cd operator+(cd a, cd b) { return mk(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ cd operator-(cd a, cd b) { return mk(a.re - b.re, a.im - b.im); }
__device__ __forceinline__ cd operator*(cd a, cd b) {
  return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
__device__ __forceinline__ cd operator*(double s, cd a) { return mk(s * a.re, s * a.im); }
__device__ __forceinline__ cd operator+(cd a, double s) { return mk(a.re + s, a.im); }
__device__ __forceinline__ cd operator+(double s, cd a) { return mk(s + a.re, a.im); }
__device__ __forceinline__ cd operator-(cd a, double s) { return mk(a.re - s, a.im); }
__device__ __forceinline__ cd operator-(double s, cd a) { return mk(s - a.re, -a.im); }
// quotient with the denominator scaled by its larger component (Smith's method)
__device__ __forceinline__ cd operator/(cd a, cd b) {
  if (fabs(b.re) >= fabs(b.im)) {
    const double r = b.im / b.re, d = b.re + b.im * r;
    return mk((a.re + a.im * r) / d, (a.im - a.re * r) / d);
  }
  const double r = b.re / b.im, d = b.re * r + b.im;
  return mk((a.re * r + a.im) / d, (a.im * r - a.re) / d);
}
__device__ __forceinline__ cd operator/(cd a, double s) { return mk(a.re / s, a.im / s); }
__device__ __forceinline__ double cabs_(cd a) { return hypot(a.re, a.im); }
// principal square root
__device__ __forceinline__ cd csqrt_(cd a) {
  if (a.re == 0.0 && a.im == 0.0) return mk(0.0, a.im);
  const double t = sqrt(0.5 * (fabs(a.re) + cabs_(a)));
  if (a.re >= 0.0) return mk(t, a.im / (2.0 * t));
  return mk(fabs(a.im) / (2.0 * t), copysign(t, a.im));
}
// principal logarithm
__device__ __forceinline__ cd clog_(cd a) { return mk(log(cabs_(a)), atan2(a.im, a.re)); }

// rayleigh_soak_wetgraupel (diags:311-394)
__device__ double rayleigh_soak_wetgraupel(double x_g, double a_geo, double b_geo, double fmelt,
                                           cd m_w, cd m_i) {
  const cd m_air = mk(1.0, 0.0);
  const double fm = fmax(fmin(fmelt, 1.0), 0.0);
  double mra = fmax(fmin(kMeltOutside, 1.0), 0.0);
  mra = mra + (1.0 - mra) * fm;
  const double x_w = x_g * fm;
  const double d_g = a_geo * pow(x_g, b_geo);
  if (!(d_g >= r1)) return 0.0;
  double vg = pi / 6.0 * d_g * d_g * d_g;
  const double rhog = fmax(fmin(x_g / vg, 900.0), 10.0);
  vg = x_g / rhog;
  const double grenz = 1.0 - rhog / 1000.0;
  double volg;
  if (mra <= grenz) {
    volg = vg * (1.0 - mra * fm);
  } else {
    const double fmgrenz = (900.0 - rhog) / (mra * 900.0 - rhog + 900.0 * rhog / 1000.0);
    if (fm <= fmgrenz)
      volg = (1.0 - mra * fm) * vg;
    else
      volg = (x_g - x_w) / 900.0 + x_w / 1000.0;
  }
  const double d_large = pow(6.0 / pi * volg, 1.0 / 3.0);
  const double volice = (x_g - x_w) / (volg * 900.0);
  const double volwater = x_w / (1000.0 * volg);
  const double volair = 1.0 - volice - volwater;
  const double volmix1 = volice / fmax(volice + volwater, 1e-10);
  // ice in water
  cd m1t = m_w * m_w, m2t = m_air * m_air, m3t = m_i * m_i;
  double vol2 = 0.0, vol3 = volmix1;
  cd beta2 = (2.0 * m1t) / (m2t - m1t) * ((m2t / (m2t - m1t)) * clog_(m2t / m1t) - 1.0);
  cd beta3 = (2.0 * m1t) / (m3t - m1t) * ((m3t / (m3t - m1t)) * clog_(m3t / m1t) - 1.0);
  const cd m_tmp = csqrt_(((1.0 - vol2 - vol3) * m1t + (vol2 * beta2) * m2t + (vol3 * beta3) * m3t) /
                          ((1.0 - vol2 - vol3) + vol2 * beta2 + vol3 * beta3));
  // air in the mixture
  m1t = m_tmp * m_tmp;
  m2t = m_air * m_air;
  m3t = (2.0 * m_air) * (2.0 * m_air);
  vol2 = volair;
  vol3 = 0.0;
  beta2 = (2.0 * m1t) / (m2t - m1t) * ((m2t / (m2t - m1t)) * clog_(m2t / m1t) - 1.0);
  beta3 = (2.0 * m1t) / (m3t - m1t) * ((m3t / (m3t - m1t)) * clog_(m3t / m1t) - 1.0);
  const cd m_core = csqrt_(((1.0 - vol2 - vol3) * m1t + (vol2 * beta2) * m2t + (vol3 * beta3) * m3t) /
                           ((1.0 - vol2 - vol3) + vol2 * beta2 + vol3 * beta3));
  const double kk = cabs_((m_core * m_core - 1.0) / (m_core * m_core + 2.0));
  // d_large**6 by binary powering, as Fortran real**integer
  const double d2 = d_large * d_large, d4 = d2 * d2, d6 = d2 * d4;
  return kk * kk * pi * pi * pi * pi * pi * d6 /
         (kLambdaRadar * kLambdaRadar * kLambdaRadar * kLambdaRadar);
}

// Simpson weight of radar bin n (0-based) over bins 0..radar_bins-1 (diags:224-231)
__device__ __forceinline__ double simpson_weight(int n) {
  double w = 0.0;
  for (int m = 1; m <= radar_bins - 1; m += 2) {  // windows (m, m+1, m+2), 1-based
    if (n + 1 == m) w += 1.0 / 3.0;
    if (n + 1 == m + 1) w += 4.0 / 3.0;
    if (n + 1 == m + 2) w += 1.0 / 3.0;
  }
  return w;
}

// reflectivity_from_melting_graupel (diags:206-248)
__device__ double melting_graupel(const TempoConsts<double>& c, const RadarConsts& rc, double rg,
                                  double ng, double ilamg, int idx, double rr) {
  const cd m_w = mk(rc.mw_re, rc.mw_im), m_i = mk(rc.mi_re, rc.mi_im);
  const double sr = fmax(0.01, fmin(1.0 - rg / fmax(rg + rr, r1), 0.99));
  const double fmelt = sr * sr;
  const double lamg = 1.0 / ilamg;
  const double n0_g = ng * c.ogg2 * pow(lamg, c.cge[0][1]);
  double eta = 0.0;
  for (int n = 0; n < radar_bins; n++) {
    const double mass = c.am_g[idx - 1] * pow(rc.gbins[n], double(bm_g));
    const double bs = rayleigh_soak_wetgraupel(mass, c.ocmg[idx - 1], c.obmg, fmelt, m_w, m_i);
    const double f_d = n0_g * pow(rc.gbins[n], double(mu_g)) * exp(-lamg * rc.gbins[n]);
    eta = eta + f_d * bs * simpson_weight(n) * rc.dgbins[n];
  }
  return kLambdaRadar * kLambdaRadar * kLambdaRadar * kLambdaRadar / (pi * pi * pi * pi * pi * rc.k_w) * eta;
}

// reflectivity_from_melting_snow (diags:251-308)
__device__ double melting_snow(const TempoConsts<double>& c, const RadarConsts& rc, double rs,
                               double smob, double smoc, double rr) {
  const cd m_w = mk(rc.mw_re, rc.mw_im), m_i = mk(rc.mi_re, rc.mi_im);
  const double sr = fmax(0.01, fmin(1.0 - rs / (rs + rr), 0.99));
  const double fmelt = sr * sr;
  const double om3 = 1.0 / smoc, m0 = smob * om3, mrat = smob * m0 * m0 * m0;
  const double slam1 = m0 * lam0, slam2 = m0 * lam1;
  double eta = 0.0;
  for (int n = 0; n < radar_bins; n++) {
    const double mass = am_s * pow(rc.sbins[n], double(bm_s));
    const double bs = rayleigh_soak_wetgraupel(mass, c.ocms, c.obms, fmelt, m_w, m_i);
    const double f_d = mrat * (kap0 * exp(-slam1 * rc.sbins[n]) +
                               kap1 * pow(m0 * rc.sbins[n], double(mu_s)) * exp(-slam2 * rc.sbins[n]));
    eta = eta + f_d * bs * simpson_weight(n) * rc.dsbins[n];
  }
  return kLambdaRadar * kLambdaRadar * kLambdaRadar * kLambdaRadar / (pi * pi * pi * pi * pi * rc.k_w) * eta;
}

// one thread per active column: melting level, then the levels below it
template <class S>
__global__ void __launch_bounds__(128) tempo_melt_refl_kernel(const __grid_constant__ StepArgs<S> a,
                                                              const __grid_constant__ TempoConsts<double> c,
                                                              const __grid_constant__ RadarConsts rc) {
  const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= (long)*a.nact) return;
  const int nz = a.nz;
  const long pl = (long)nz * a.ncol_pad, base = pt_base(s, nz);
  const double* mv = reinterpret_cast<const double*>(a.mlw) + base;
  const uint8_t* mb = reinterpret_cast<const uint8_t*>(reinterpret_cast<const double*>(a.mlw) + kMeltN * pl) + base;
  auto val = [&](int q, int k) { return mv[q * pl + (long)k * kSlotTile]; };
  // find_melting_level (diags:124-141), reference level indices
  int k_melt = 1;
  for (int kf = nz - 1; kf >= 1; kf--) {
    const uint8_t m0 = mb[(long)(kf - 1) * kSlotTile], m1 = mb[(long)kf * kSlotTile];
    if ((m0 & MB_WARMRAIN) && (m1 & (MB_QS | MB_QG))) {
      k_melt = max(kf + 1, k_melt);
      break;
    }
  }
  if (k_melt <= 2) return;
  ColGeom g = col_geom(a, a.act[s]);
  for (int kf = 1; kf < k_melt - 1; kf++) {
    const int k = kf - 1;
    const uint8_t m = mb[(long)k * kSlotTile];
    if (!(m & (MB_QS | MB_QG))) continue;
    const double ze_r = val(MV_ZER, k);
    double ze_s = val(MV_ZES, k), ze_g = val(MV_ZEG, k);
    if (m & MB_QS) ze_s = melting_snow(c, rc, val(MV_RS, k), val(MV_SMOB, k), val(MV_SMOC, k), val(MV_RR, k));
    if (m & MB_QG)
      ze_g = melting_graupel(c, rc, val(MV_RG, k), val(MV_NG, k), val(MV_ILAMG, k), int(val(MV_IDX, k)),
                             val(MV_RR, k));
    const double dbz = fmax(-35.0, 10.0 * log10((ze_r + ze_s + ze_g) * 1.e18));
    a.refl10cm[tile3_of(a, g, k)] = S(dbz);
  }
}

}  // namespace

template <class S>
cudaError_t launch_melt_refl(const StepArgs<S>& a, const TempoConsts<double>& c, const RadarConsts& rc,
                             cudaStream_t s) {
  if (a.ncol == 0 || !(a.flags & F_MELT)) return cudaSuccess;
  tempo_melt_refl_kernel<S><<<(unsigned)((a.ncol + 127) / 128), 128, 0, s>>>(a, c, rc);
  return cudaGetLastError();
}
template cudaError_t launch_melt_refl<double>(const StepArgs<double>&, const TempoConsts<double>&,
                                              const RadarConsts&, cudaStream_t);
template cudaError_t launch_melt_refl<float>(const StepArgs<float>&, const TempoConsts<double>&,
                                             const RadarConsts&, cudaStream_t);

}  // namespace tg
