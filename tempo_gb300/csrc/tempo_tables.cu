// tempo_tables.cu -- FP64 construction of TEMPO's lookup tables on the GPU.
//
// Small init-time tables (src/module_mp_tempo_utils.F90): compute_efrw :349-400,
// compute_efsw :403-440, qi_aut_qs :443-490, compute_drop_evap :493-527.
// Large tables (src/module_mp_tempo_tables.F90): qr_acr_qs :493-621,
// qr_acr_qg :624-714, freezewater :717-805.
//
// The collection tables are bin integrals of the form
//     sum_{n2,n} K(n2, n) n_x(n) n_r(n2)     with K >= 0, n_x >= 0, n_r >= 0,
// evaluated here as two FP64 GEMMs (K x n_x, then n_r x (K n_x)) instead of the
// reference's 6-deep loop: the same non-negative terms summed in a different order
// (1.7e11 inner iterations become 1.9e10 multiply-adds).  freezewater keeps the
// reference's descending prefix sums and their early exits, one thread per entry.
// Built with -fmad=false like the FP64 step.
#include <cuda_runtime.h>

#include <cmath>

#include "tempo_internal.h"

namespace tg {

namespace {

__constant__ TempoBins c_bins;

__device__ __forceinline__ double dmax(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double dmin(double a, double b) { return a < b ? a : b; }
__device__ __forceinline__ double ipow_d(double x, int m) {
  unsigned n = m < 0 ? -(unsigned)m : (unsigned)m;
  double y = (n % 2) ? x : 1.0;
  while (n >>= 1) {
    x = x * x;
    if (n % 2) y = y * x;
  }
  return m < 0 ? 1.0 / y : y;
}

// compute_efrw (utils:349-400), one thread per (i, j)
__global__ void k_efrw(double* t_efrw) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nbr * nbc) return;
  int i = idx % nbr + 1, j = idx / nbr + 1;
  const double dri = c_bins.dr[i - 1], dcj = c_bins.dc[j - 1];
  double ef_rw = 0.0, p = dcj / dri;
  if (dri < 50.e-6 || dcj < 3.e-6) {
    ef_rw = 0.0;
  } else if (p > 0.25) {
    double x = dcj * 1.e6;
    if (dri < 75.e-6)
      ef_rw = 0.026794 * x - 0.20604;
    else if (dri < 125.e-6)
      ef_rw = -0.00066842 * x * x + 0.061542 * x - 0.37089;
    else if (dri < 175.e-6)
      ef_rw = 4.091e-06 * x * x * x * x - 0.00030908 * x * x * x + 0.0066237 * x * x -
              0.0013687 * x - 0.073022;
    else if (dri < 250.e-6)
      ef_rw = 9.6719e-5 * x * x * x - 0.0068901 * x * x + 0.17305 * x - 0.65988;
    else if (dri < 350.e-6)
      ef_rw = 9.0488e-5 * x * x * x - 0.006585 * x * x + 0.16606 * x - 0.56125;
    else
      ef_rw = 0.00010721 * x * x * x - 0.0072962 * x * x + 0.1704 * x - 0.46929;
  } else {
    double vtr = -0.1021 + 4.932e3 * dri - 0.9551e6 * dri * dri + 0.07934e9 * dri * dri * dri -
                 0.002362e12 * dri * dri * dri * dri;
    double stokes = dcj * dcj * vtr * rho_w / (9.0 * 1.718e-5 * dri);
    double reynolds = 9.0 * stokes / (p * p * rho_w);
    double f = log(reynolds);
    double g = -0.1007 - 0.358 * f + 0.0261 * f * f;
    double k0 = exp(g);
    double z = log(stokes / (k0 + 1.e-15));
    double h = 0.1465 + 1.302 * z - 0.607 * z * z + 0.293 * z * z * z;
    double yc0 = 2.0 / pi * atan(h);
    ef_rw = (yc0 + p) * (yc0 + p) / ((1. + p) * (1. + p));
  }
  t_efrw[idx] = dmax(0.0, dmin(ef_rw, 0.95));
}

// compute_efsw (utils:403-440)
__global__ void k_efsw(double* t_efsw, const __grid_constant__ TempoConsts<double> tc) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nbs * nbc) return;
  int i = idx % nbs + 1, j = idx / nbs + 1;
  const double dcj = c_bins.dc[j - 1], dsi = c_bins.ds[i - 1];
  double vtc = 1.19e4 * (1.0e4 * dcj * dcj * 0.25);
  double vts = av_s * pow(dsi, bv_s) * exp(-fv_s * dsi) - vtc;
  double ds_m = pow(am_s * pow(dsi, bm_s) / tc.am_r, tc.obmr);
  double p = dcj / ds_m;
  double v = 0.0;
  if (!(p > 0.25 || dsi < d0s || dcj < 6.e-6 || vts < 1.e-3)) {
    double stokes = dcj * dcj * vts * rho_w / (9. * 1.718e-5 * ds_m);
    double reynolds = 9.0 * stokes / (p * p * rho_w);
    double f = log(reynolds);
    double g = -0.1007 - 0.358 * f + 0.0261 * f * f;
    double k0 = exp(g);
    double z = log(stokes / (k0 + 1.e-15));
    double h = 0.1465 + 1.302 * z - 0.607 * z * z + 0.293 * z * z * z;
    double yc0 = 2.0 / pi * atan(h);
    double ef_sw = (yc0 + p) * (yc0 + p) / ((1. + p) * (1. + p));
    v = dmax(0.0, dmin(ef_sw, 0.95));
  }
  t_efsw[idx] = v;
}

// compute_drop_evap (utils:493-527): one thread per (j, k); the reference's inner sum
// over n = 1..i is the running prefix sum taken in the same order.
__global__ void k_drop_evap(double* tpc_wev, double* tnc_wev, const __grid_constant__ TempoConsts<double> tc) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= ntb_c * nbc) return;
  int j = idx % ntb_c + 1, k = idx / ntb_c + 1;
  const double tnck = c_bins.t_nc[k - 1];
  int nu_c = (nu_c_scale / tnck >= 12.5) ? 15 : min(15, (int)round(nu_c_scale / tnck) + 2);
  double lamc = pow(tnck * tc.am_r * tc.ccg[nu_c - 1][1] * tc.ocg1[nu_c - 1] / c_bins.r_c[j - 1],
                    tc.obmr);
  double n0_c = tnck * tc.ocg1[nu_c - 1] * pow(lamc, tc.cce[nu_c - 1][0]);
  double summ = 0.0, summ2 = 0.0;
  for (int i = 1; i <= nbc; i++) {
    double dci = c_bins.dc[i - 1];
    double n_c = n0_c * ipow_d(dci, nu_c) * exp(-lamc * dci) * c_bins.dtc[i - 1];
    double massc = tc.am_r * pow(dci, bm_r);
    summ = summ + massc * n_c;
    summ2 = summ2 + n_c;
    long o = (i - 1) + (long)(j - 1) * nbc + (long)(k - 1) * nbc * ntb_c;
    tpc_wev[o] = summ;
    tnc_wev[o] = summ2;
  }
}

// calc_gamma_p (utils:27-145)
__device__ double gamma_p(double a, double x) {
  if ((x < 0.0) || (a <= 0.0)) return nan("");
  if (x < (a + 1.0)) {
    double aj = a, sum_term = 1.0 / tgamma(aj + 1.0), sum = sum_term;
    for (int k = 1; k <= 100; k++) {
      aj = aj + 1.0;
      sum_term = sum_term * x / aj;
      sum = sum + sum_term;
      if (fabs(sum_term) < (fabs(sum) * 1.e-7)) break;
    }
    return sum * pow(x, a) * exp(-x);
  }
  const double offset = 1.e-30;
  double f0 = offset, b = 1.0 - a + x, d = 1.0 / b, c = b + (1.0 / f0), delta = c * d,
         f = f0 * delta;
  for (int k = 1; k <= 100; k++) {
    double aj = k * (a - k);
    b = b + 2.0;
    d = b + aj * d;
    if (fabs(d) < offset) d = offset;
    c = b + aj / c;
    if (fabs(c) < offset) c = offset;
    d = 1.0 / d;
    delta = c * d;
    f = f * delta;
    if (fabs(delta - 1.0) < 1.e-7) break;
  }
  return 1.0 - exp(-x + a * log(x)) * f / tgamma(a);
}

// qi_aut_qs (utils:443-490), one thread per (i, j)
__global__ void k_qi_aut_qs(double* tpi_ide, double* tps_iaus, double* tni_iaus, const __grid_constant__ TempoConsts<double> tc) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= ntb_i * ntb_i1) return;
  int i = idx % ntb_i + 1, j = idx / ntb_i + 1;
  const double nti = c_bins.nt_i[j - 1], ri = c_bins.r_i[i - 1];
  double lami = pow(tc.am_i * tc.cig[1] * tc.oig1 * nti / ri, tc.obmi);
  double di_mean = (bm_i + mu_i + 1.) / lami;
  double n0_i = nti * tc.oig1 * pow(lami, tc.cie[0]);
  double t1 = 0., t2 = 0., tpi;
  if (di_mean > 5. * d0s) {
    t1 = ri;
    t2 = nti;
    tpi = 0.;
  } else if (di_mean < tc.d0i) {
    tpi = 1.;
  } else {
    double xlimit_intg = lami * d0s;
    tpi = gamma_p(mu_i + 2.0, xlimit_intg);
    for (int n2 = 0; n2 < nbi; n2++) {
      double din = c_bins.di[n2];
      double n_i = n0_i * pow(din, mu_i) * exp(-lami * din) * c_bins.dti[n2];
      if (din >= d0s) {
        t1 = t1 + n_i * tc.am_i * pow(din, bm_i);
        t2 = t2 + n_i;
      }
    }
  }
  tpi_ide[idx] = tpi;
  tps_iaus[idx] = t1;
  tni_iaus[idx] = t2;
}

// ---------------------------------------------------------------------------------
// large tables
// ---------------------------------------------------------------------------------
// rain PSD per bin for (m, k) (tables:531-536): NR[(m-1)*37 + (k-1)][n2]
__global__ void k_rain_psd(double* NR, const __grid_constant__ TempoConsts<double> tc) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= ntb_r * ntb_r1 * nbr) return;
  int n2 = idx % nbr, mk = idx / nbr;
  int m = mk / ntb_r1 + 1, k = mk % ntb_r1 + 1;
  double lam_exp = pow(c_bins.n0r_exp[k - 1] * tc.am_r * tc.crg[0] / c_bins.r_r[m - 1], tc.ore1);
  double lamr = lam_exp * pow(tc.crg[2] * tc.org2 * tc.org1, tc.obmr);
  double n0_r = c_bins.n0r_exp[k - 1] / (tc.crg[1] * lam_exp) * pow(lamr, tc.cre[1]);
  NR[idx] = n0_r * pow(c_bins.dr[n2], mu_r) * exp(-lamr * c_bins.dr[n2]) * c_bins.dtr[n2];
}

__device__ __forceinline__ double poly_a(const double* s, double tc, double X) {
  return s[0] + s[1] * tc + s[2] * X + s[3] * tc * X + s[4] * tc * tc + s[5] * X * X +
         s[6] * tc * tc * X + s[7] * tc * X * X + s[8] * tc * tc * tc + s[9] * X * X * X;
}
// snow PSD per bin for (i, j) (tables:540-551): NS[(j-1)*37 + (i-1)][n]
__global__ void k_snow_psd(double* NS, const __grid_constant__ TempoConsts<double> tc) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= ntb_s * ntb_t * nbs) return;
  int n = idx % nbs, ij = idx / nbs;
  int i = ij % ntb_s + 1, j = ij / ntb_s + 1;
  const double rs = c_bins.r_s[i - 1], tcel = c_bins.tc[j - 1];
  double m2 = rs * tc.oams;  // snow_moments smob/smoc (utils:148-200)
  double a_ = pow(10.0, poly_a(tc.sa, tcel, bm_s));
  double b_ = poly_a(tc.sb, tcel, bm_s);
  double smo2_ = pow(m2 / a_, 1.0 / b_);
  double a1 = pow(10.0, poly_a(tc.sa, tcel, tc.cse[0]));
  double b1 = poly_a(tc.sb, tcel, tc.cse[0]);
  double m3 = a1 * pow(smo2_, b1);
  double om3 = 1.0 / m3;
  double mrat = m2 * (m2 * om3) * (m2 * om3) * (m2 * om3);
  double m0 = pow(m2 * om3, mu_s);
  double slam1 = m2 * om3 * lam0;
  double slam2 = m2 * om3 * lam1;
  const double d = c_bins.ds[n];
  NS[idx] = mrat * (kap0 * exp(-slam1 * d) + kap1 * m0 * pow(d, mu_s) * exp(-slam2 * d)) * c_bins.dts[n];
}
// graupel PSD per bin for (i, j, n3) (tables:668-673): NG[((n3-1)*37 + (j-1))*37 + (i-1)][n]
__global__ void k_graupel_psd(double* NG, const __grid_constant__ TempoConsts<double> tc) {
  long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)nrhg * ntb_g * ntb_g1 * nbg) return;
  int n = (int)(idx % nbg);
  long r = idx / nbg;
  int i = (int)(r % ntb_g1) + 1, j = (int)((r / ntb_g1) % ntb_g) + 1, n3 = (int)(r / (ntb_g1 * ntb_g)) + 1;
  double lam_exp = pow(c_bins.n0g_exp[i - 1] * tc.am_g[n3 - 1] * tc.cgg[0][0] / c_bins.r_g[j - 1], tc.oge1);
  double lamg = lam_exp * pow(tc.cgg[0][2] * tc.ogg2 * tc.ogg1, tc.obmg);
  double n0_g = c_bins.n0g_exp[i - 1] / (tc.cgg[0][1] * lam_exp) * pow(lamg, tc.cge[0][1]);
  NG[idx] = n0_g * pow(c_bins.dg[n], mu_g) * exp(-lamg * c_bins.dg[n]) * c_bins.dtg[n];
}
__device__ __forceinline__ double rain_speed(double d) {  // tables:519-522
  return -0.1021 + 4.932e3 * d - 0.9551e6 * d * d + 0.07934e9 * d * d * d - 0.002362e12 * d * d * d * d;
}
// qr_acr_qs kernels K[a][n2][n] for the 12 outputs in table order (tables:553-616)
__global__ void k_qs_kernels(double* K, const __grid_constant__ TempoConsts<double> tc) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nbr * nbs) return;
  int n = idx % nbs, n2 = idx / nbs;
  const double drr = c_bins.dr[n2], dss = c_bins.ds[n];
  double vr = rain_speed(drr);
  double vs = 1.5 * av_s * pow(dss, bv_s) * exp(-fv_s * dss);
  double massr = tc.am_r * pow(drr, bm_r);
  double masss = am_s * pow(dss, bm_s);
  double dvs = 0.5 * ((vr - vs) + fabs(vr - vs));
  double dvr = 0.5 * ((vs - vr) + fabs(vs - vr));
  double geo = pi * .25 * ef_rs * (dss + drr) * (dss + drr);
  bool big = massr > 1.5 * masss;
  double v[12] = {big ? geo * dvs * masss : 0., big ? geo * dvs * massr : 0.,
                  big ? 0. : geo * dvs * masss, big ? 0. : geo * dvs * massr,
                  big ? geo * dvr * massr : 0., big ? geo * dvr * masss : 0.,
                  big ? 0. : geo * dvr * massr, big ? 0. : geo * dvr * masss,
                  big ? geo * dvs : 0.,         big ? 0. : geo * dvs,
                  big ? geo * dvr : 0.,         big ? 0. : geo * dvr};
  for (int a = 0; a < 12; a++) K[((long)a * nbr + n2) * nbs + n] = v[a];
}
// qr_acr_qg kernels K[n3][a][n2][n] for t1, z1, t2, y1, y2 (tables:681-702)
__global__ void k_qg_kernels(double* K, const __grid_constant__ TempoConsts<double> tc) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nrhg * nbr * nbg) return;
  int n = idx % nbg, n2 = (idx / nbg) % nbr, n3 = idx / (nbg * nbr) + 1;
  const double drr = c_bins.dr[n2], dgg = c_bins.dg[n];
  double vr = rain_speed(drr);
  double vg = tc.av_g[n3 - 1] * pow(dgg, tc.bv_g[n3 - 1]);
  double massr = tc.am_r * pow(drr, bm_r);
  double massg = tc.am_g[n3 - 1] * pow(dgg, bm_g);
  double dvg = 0.5 * ((vr - vg) + fabs(vr - vg));
  double dvr = 0.5 * ((vg - vr) + fabs(vg - vr));
  double geo = pi * .25 * ef_rg * (dgg + drr) * (dgg + drr);
  double v[5] = {geo * dvg * massg, geo * dvg * massr, geo * dvr * massr, geo * dvg, geo * dvr};
  for (int a = 0; a < 5; a++) K[(((long)(n3 - 1) * 5 + a) * nbr + n2) * nbg + n] = v[a];
}

// NT GEMM over K = 100 with FP64 FFMA-free accumulation (-fmad=false):
//   C[m][n] = sum_k A[m*lda + k] * B[n*ldb + k],  64 x 64 tile, 256 threads, 4 x 4 each.
// Epilogue modes: 0 plain store C[m*ldc + n]; 1 qs table (min with r_r on output 1);
// 2 qg table (min with r_r on output 1).  For modes 1/2, row m = (mrain-1)*37 + (krain-1)
// and the row's AoS block starts at rowbase(m).
constexpr int GT = 64, GK = 100, GKC = 25;
__global__ void __launch_bounds__(256) k_gemm_nt(const double* __restrict__ A, long lda,
                                                 const double* __restrict__ B, long ldb,
                                                 double* __restrict__ C, long ldc, int M, int N,
                                                 int mode, int nfam, long batch_a, long batch_b,
                                                 long batch_c) {
  __shared__ double As[GKC][GT + 1];
  __shared__ double Bs[GKC][GT + 1];
  const int bz = blockIdx.z;
  A += batch_a * bz;
  B += batch_b * bz;
  C += batch_c * bz;
  const int m0 = blockIdx.y * GT, n0 = blockIdx.x * GT;
  const int tm = (threadIdx.x / 16) * 4, tn = (threadIdx.x % 16) * 4;
  double acc[4][4] = {};
  for (int kc = 0; kc < GK; kc += GKC) {
    __syncthreads();
    for (int t = threadIdx.x; t < GT * GKC; t += blockDim.x) {
      int r = t / GKC, k = t % GKC;
      As[k][r] = (m0 + r < M) ? A[(long)(m0 + r) * lda + kc + k] : 0.0;
      Bs[k][r] = (n0 + r < N) ? B[(long)(n0 + r) * ldb + kc + k] : 0.0;
    }
    __syncthreads();
    for (int k = 0; k < GKC; k++) {
      double av[4], bv[4];
      for (int i = 0; i < 4; i++) av[i] = As[k][tm + i];
      for (int j = 0; j < 4; j++) bv[j] = Bs[k][tn + j];
      for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) acc[i][j] = acc[i][j] + av[i] * bv[j];
    }
  }
  for (int i = 0; i < 4; i++) {
    int m = m0 + tm + i;
    if (m >= M) continue;
    for (int j = 0; j < 4; j++) {
      int n = n0 + tn + j;
      if (n >= N) continue;
      double v = acc[i][j];
      if (mode == 0) {
        C[(long)m * ldc + n] = v;
      } else {
        // n = entry * nfam + a ; rain row m -> (mr, kr)
        int a = n % nfam;
        int mr = m / ntb_r1 + 1, kr = m % ntb_r1 + 1;
        if (a == 1) v = dmin(v, c_bins.r_r[mr - 1]);
        long entries_per_row = (long)N / nfam;
        long row = (long)(kr - 1) + (long)(mr - 1) * ntb_r1;  // Fortran (.., k, m) order
        C[(row * entries_per_row) * nfam + n] = v;
      }
    }
  }
}

// freezewater prerequisites: rain/cloud PSD per bin and freezing probabilities
__global__ void k_fz_prep(double* NRf, double* NCf, double* PR, double* PC, const __grid_constant__ TempoConsts<double> tc) {
  long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long nNR = (long)ntb_r * ntb_r1 * nbr, nNC = (long)nbc * ntb_c * nbc;
  const long nPR = (long)ntb_in * 45 * nbr, nPC = (long)ntb_in * 45 * nbc;
  const double orho_w = 1.0 / rho_w;
  if (idx < nNR) {  // [i][j][n2]
    int n2 = idx % nbr, j = (idx / nbr) % ntb_r1 + 1, i = idx / (nbr * ntb_r1) + 1;
    double lam_exp = pow(c_bins.n0r_exp[j - 1] * tc.am_r * tc.crg[0] / c_bins.r_r[i - 1], tc.ore1);
    double lamr = lam_exp * pow(tc.crg[2] * tc.org2 * tc.org1, tc.obmr);
    double n0_r = c_bins.n0r_exp[j - 1] / (tc.crg[1] * lam_exp) * pow(lamr, tc.cre[1]);
    NRf[idx] = n0_r * pow(c_bins.dr[n2], mu_r) * exp(-lamr * c_bins.dr[n2]) * c_bins.dtr[n2];
    return;
  }
  idx -= nNR;
  if (idx < nNC) {  // [j][i][n]
    int n = idx % nbc, i = (idx / nbc) % ntb_c + 1, j = idx / (nbc * ntb_c) + 1;
    const double tncj = c_bins.t_nc[j - 1];
    int nu_c = min(15, (int)round(nu_c_scale / tncj) + 2);
    double lamc = pow(tncj * tc.am_r * tc.ccg[nu_c - 1][1] * tc.ocg1[nu_c - 1] / c_bins.r_c[i - 1],
                      tc.obmr);
    double n0_c = tncj * tc.ocg1[nu_c - 1] * pow(lamc, tc.cce[nu_c - 1][0]);
    NCf[idx] = n0_c * ipow_d(c_bins.dc[n], nu_c) * exp(-lamc * c_bins.dc[n]) * c_bins.dtc[n];
    return;
  }
  idx -= nNC;
  if (idx < nPR + nPC) {
    bool rain = idx < nPR;
    long r = rain ? idx : idx - nPR;
    int nb = rain ? nbr : nbc;
    int n = r % nb, k = (r / nb) % 45 + 1, m = r / (nb * 45) + 1;
    double t_adjust = dmax(-3.0, dmin(3.0 - log10(c_bins.nt_in[m - 1]), 3.0));
    double texp = exp((double)k - t_adjust) - 1.0;
    double mass = tc.am_r * pow(rain ? c_bins.dr[n] : c_bins.dc[n], bm_r);
    double vol = mass * orho_w;
    double prob = dmax(0.0, 1.0 - exp(-120.0 * vol * 5.2e-4 * texp));
    (rain ? PR : PC)[r] = prob;
  }
}
// freezewater rain part (tables:751-782): one thread per (i, j, k, m)
__global__ void k_fz_rain(const double* NRf, const double* PR, double* qrfz, const __grid_constant__ TempoConsts<double> tc) {
  long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)ntb_r * ntb_r1 * 45 * ntb_in) return;
  int i = idx % ntb_r + 1, j = (idx / ntb_r) % ntb_r1 + 1;
  int k = (idx / (ntb_r * ntb_r1)) % 45 + 1, m = idx / ((long)ntb_r * ntb_r1 * 45) + 1;
  const double* nr = NRf + ((long)(i - 1) * ntb_r1 + (j - 1)) * nbr;
  const double* pr = PR + ((long)(m - 1) * 45 + (k - 1)) * nbr;
  const double rri = c_bins.r_r[i - 1];
  double sum1 = 0, sum2 = 0, sumn1 = 0, sumn2 = 0;
  for (int n2 = nbr; n2 >= 1; n2--) {
    double n_r = nr[n2 - 1], prob = pr[n2 - 1];
    double massr = tc.am_r * pow(c_bins.dr[n2 - 1], bm_r);
    if (massr < tc.xm0g) {
      sumn1 = sumn1 + prob * n_r;
      sum1 = sum1 + prob * n_r * massr;
    } else {
      sumn2 = sumn2 + prob * n_r;
      sum2 = sum2 + prob * n_r * massr;
    }
    if ((sum1 + sum2) >= rri) break;
  }
  double* o = qrfz + 4 * idx;  // AoS: tpi, tni, tpg, tnr
  o[0] = sum1;
  o[1] = sumn1;
  o[2] = sum2;
  o[3] = sumn2;
}
// freezewater cloud part (tables:784-802): one thread per (i, j, k, m)
__global__ void k_fz_cloud(const double* NCf, const double* PC, double* qcfz, const __grid_constant__ TempoConsts<double> tc) {
  long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)ntb_c * nbc * 45 * ntb_in) return;
  int i = idx % ntb_c + 1, j = (idx / ntb_c) % nbc + 1;
  int k = (idx / ((long)ntb_c * nbc)) % 45 + 1, m = idx / ((long)ntb_c * nbc * 45) + 1;
  const double* ncv = NCf + ((long)(j - 1) * ntb_c + (i - 1)) * nbc;
  const double* pc = PC + ((long)(m - 1) * 45 + (k - 1)) * nbc;
  const double rci = c_bins.r_c[i - 1], tncj = c_bins.t_nc[j - 1];
  double sum1 = 0, sumn2 = 0;
  for (int n = nbc; n >= 1; n--) {
    double prob = pc[n - 1], n_c = ncv[n - 1];
    double massc = tc.am_r * pow(c_bins.dc[n - 1], bm_r);
    sumn2 = dmin(tncj, sumn2 + prob * n_c);
    sum1 = sum1 + prob * n_c * massc;
    if (sum1 >= rci) break;
  }
  double* o = qcfz + 2 * idx;  // AoS: tpi, tni
  o[0] = sum1;
  o[1] = sumn2;
}

__global__ void k_narrow(float* dst, const double* src, long n) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (float)src[i];
}
__global__ void k_aos(double* aos, const double* soa, long n, int nfam, int which, int to_aos) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (to_aos)
    aos[i * nfam + which] = soa[i];
  else
    const_cast<double*>(soa)[i] = aos[i * nfam + which];
}
__global__ void k_emissions(double* nwfa, const double* nwfa2d, long ni, long nk, long nj,
                            int kts_off, double dt) {
  long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= ni * nj) return;
  long i = idx % ni, j = idx / ni;
  long e = i + (long)kts_off * ni + j * ni * nk;
  nwfa[e] = nwfa[e] + nwfa2d[idx] * dt;
}

inline unsigned nblk(long n, int b) { return (unsigned)((n + b - 1) / b); }

}  // namespace

cudaError_t build_small_tables(const DevTables64& t, const TempoBins& bins,
                               const TempoConsts<double>& tc, cudaStream_t s) {
  cudaError_t e = cudaMemcpyToSymbolAsync(c_bins, &bins, sizeof bins, 0, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return e;
  k_efrw<<<nblk(nbr * nbc, 128), 128, 0, s>>>(t.t_efrw);
  k_efsw<<<nblk(nbs * nbc, 128), 128, 0, s>>>(t.t_efsw, tc);
  k_drop_evap<<<nblk(ntb_c * nbc, 128), 128, 0, s>>>(t.tpc_wev, t.tnc_wev, tc);
  k_qi_aut_qs<<<nblk(ntb_i * ntb_i1, 128), 128, 0, s>>>(t.tpi_ide, t.tps_iaus, t.tni_iaus, tc);
  return cudaGetLastError();
}

// work buffer layout (doubles)
namespace {
constexpr long W_NR = (long)ntb_r * ntb_r1 * nbr;                  // rain PSD [mk][n2]
constexpr long W_NS = (long)ntb_s * ntb_t * nbs;                   // snow PSD [ij][n]
constexpr long W_NG = (long)nrhg * ntb_g * ntb_g1 * nbg;           // graupel PSD [n3ji][n]
constexpr long W_KS = 12L * nbr * nbs;                             // qs kernels
constexpr long W_KG = (long)nrhg * 5 * nbr * nbg;                  // qg kernels
constexpr long W_GS = (long)ntb_s * ntb_t * 12 * nbr;              // qs stage-1 [ij][a][n2]
constexpr long W_GG = (long)nrhg * ntb_g * ntb_g1 * 5 * nbr;       // qg stage-1 [n3ji][a][n2]
constexpr long W_NRF = (long)ntb_r * ntb_r1 * nbr;
constexpr long W_NCF = (long)nbc * ntb_c * nbc;
constexpr long W_PR = (long)ntb_in * 45 * nbr;
constexpr long W_PC = (long)ntb_in * 45 * nbc;
constexpr long W_TOTAL = W_NR + W_NS + W_NG + W_KS + W_KG + W_GS + W_GG + W_NRF + W_NCF + W_PR + W_PC;
}  // namespace

size_t big_tables_work_bytes() { return (size_t)W_TOTAL * sizeof(double); }

cudaError_t build_big_tables(const DevTables64& t, const TempoBins& bins,
                             const TempoConsts<double>& tc, double* work,
                             size_t work_bytes, cudaStream_t s) {
  if (work_bytes < big_tables_work_bytes()) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemcpyToSymbolAsync(c_bins, &bins, sizeof bins, 0, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return e;
  double* NR = work;
  double* NS = NR + W_NR;
  double* NG = NS + W_NS;
  double* KS = NG + W_NG;
  double* KG = KS + W_KS;
  double* GS = KG + W_KG;
  double* GG = GS + W_GS;
  double* NRf = GG + W_GG;
  double* NCf = NRf + W_NRF;
  double* PR = NCf + W_NCF;
  double* PC = PR + W_PR;
  k_rain_psd<<<nblk(W_NR, 256), 256, 0, s>>>(NR, tc);
  k_snow_psd<<<nblk(W_NS, 256), 256, 0, s>>>(NS, tc);
  k_graupel_psd<<<nblk(W_NG, 256), 256, 0, s>>>(NG, tc);
  k_qs_kernels<<<nblk((long)nbr * nbs, 256), 256, 0, s>>>(KS, tc);
  k_qg_kernels<<<nblk((long)nrhg * nbr * nbg, 256), 256, 0, s>>>(KG, tc);
  // qs stage 1: GS[ij][a*100 + n2] = sum_n NS[ij][n] * KS[a*100 + n2][n]
  {
    dim3 g(nblk(12 * nbr, GT), nblk(ntb_s * ntb_t, GT), 1);
    k_gemm_nt<<<g, 256, 0, s>>>(NS, nbs, KS, nbs, GS, 12 * nbr, ntb_s * ntb_t, 12 * nbr, 0, 12, 0, 0, 0);
  }
  // qs stage 2: out[mk][ij*12 + a] = sum_n2 NR[mk][n2] * GS[ij][a][n2]
  {
    dim3 g(nblk((long)ntb_s * ntb_t * 12, GT), nblk(ntb_r * ntb_r1, GT), 1);
    k_gemm_nt<<<g, 256, 0, s>>>(NR, nbr, GS, nbr, t.qs, 0, ntb_r * ntb_r1, ntb_s * ntb_t * 12, 1, 12, 0, 0, 0);
  }
  // qg stage 1 (batched over n3): GG[n3][ji][a*100 + n2] = sum_n NG[n3][ji][n] * KG[n3][a*100+n2][n]
  {
    dim3 g(nblk(5 * nbr, GT), nblk(ntb_g * ntb_g1, GT), nrhg);
    k_gemm_nt<<<g, 256, 0, s>>>(NG, nbg, KG, nbg, GG, 5 * nbr, ntb_g * ntb_g1, 5 * nbr, 0, 5,
                                (long)ntb_g * ntb_g1 * nbg, 5L * nbr * nbg, (long)ntb_g * ntb_g1 * 5 * nbr);
  }
  // qg stage 2: out[mk][(n3,j,i)*5 + a] = sum_n2 NR[mk][n2] * GG[n3ji][a][n2]
  {
    dim3 g(nblk((long)nrhg * ntb_g * ntb_g1 * 5, GT), nblk(ntb_r * ntb_r1, GT), 1);
    k_gemm_nt<<<g, 256, 0, s>>>(NR, nbr, GG, nbr, t.qg, 0, ntb_r * ntb_r1, nrhg * ntb_g * ntb_g1 * 5, 2,
                                5, 0, 0, 0);
  }
  // freezewater
  k_fz_prep<<<nblk(W_NRF + W_NCF + W_PR + W_PC, 256), 256, 0, s>>>(NRf, NCf, PR, PC, tc);
  k_fz_rain<<<nblk((long)ntb_r * ntb_r1 * 45 * ntb_in, 128), 128, 0, s>>>(NRf, PR, t.qrfz, tc);
  k_fz_cloud<<<nblk((long)ntb_c * nbc * 45 * ntb_in, 128), 128, 0, s>>>(NCf, PC, t.qcfz, tc);
  return cudaGetLastError();
}

cudaError_t narrow_copy(float* dst, const double* src, long n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_narrow<<<nblk(n, 256), 256, 0, s>>>(dst, src, n);
  return cudaGetLastError();
}
cudaError_t aos_scatter(double* aos, const double* soa, long n, int nfam, int which, cudaStream_t s) {
  k_aos<<<nblk(n, 256), 256, 0, s>>>(aos, soa, n, nfam, which, 1);
  return cudaGetLastError();
}
cudaError_t aos_gather(double* soa, const double* aos, long n, int nfam, int which, cudaStream_t s) {
  k_aos<<<nblk(n, 256), 256, 0, s>>>(const_cast<double*>(aos), soa, n, nfam, which, 0);
  return cudaGetLastError();
}
cudaError_t launch_surface_emissions(double* nwfa, const double* nwfa2d, long ni, long nk, long nj,
                                     int kts_off, double dt, cudaStream_t s) {
  k_emissions<<<nblk(ni * nj, 256), 256, 0, s>>>(nwfa, nwfa2d, ni, nk, nj, kts_off, dt);
  return cudaGetLastError();
}

}  // namespace tg
