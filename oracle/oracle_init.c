/*
 * oracle_init.c -- CPU restatement (test infrastructure) of TEMPO's init-time code:
 * module_mp_tempo_params.F90 (bins, parameters, graupel vars), module_mp_tempo_utils.F90
 * (gamma_p, snow moments, saturation, init tables), table file I/O
 * (module_mp_tempo_driver.F90:532-649, module_mp_tempo_tables.F90:96-444) and the
 * three large table builders (module_mp_tempo_tables.F90:493-805).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle_common.h"
#include "tempo_oracle.h"

/* ------------------------------------------------------------------------------ */
/* bin data (params:194-288).  The mass/number bins are the decimal literals        */
/* d.eE (d=1..9) per decade plus the closing 1.eE; parsing the same decimal strings */
/* gives the same doubles as the Fortran literals.                                  */
/* ------------------------------------------------------------------------------ */
double r_c[ntb_c], r_i[ntb_i], r_r[ntb_r], r_s[ntb_s], r_g[ntb_g], n0r_exp[ntb_r1],
    n0g_exp[ntb_g1], nt_i[ntb_i1], nt_in[ntb_in];
const double ta_na[ntb_arc] = {10., 31.6, 100., 316., 1000., 3160., 10000.};
const double ta_ww[ntb_arw] = {0.01, 0.0316, 0.1, 0.316, 1., 3.16, 10., 31.6, 100.};
const double ta_tk[ntb_art] = {243.15, 253.15, 263.15, 273.15, 283.15, 293.15, 303.15};
/* Field et al. (2005) moment-relation coefficients (params:279-284) */
const double sa[10] = {5.065339, -0.062659, -3.032362, 0.029469, -0.000285,
                       0.31255,  0.000204,  0.003199,  0.,       -0.015952};
const double sb[10] = {0.476221, -0.015896, 0.165977, 0.007468, -0.000141,
                       0.060366, 0.000079,  0.000594, 0.,       -0.003577};
const double tc_tab[ntb_t] = {-0.01, -5., -10., -15., -20., -25., -30., -35., -40.};

static void decade_bins(double *out, int first_exp, int count) {
  char buf[32];
  int n = 0, e = first_exp;
  while (n < count) {
    for (int d = 1; d <= 9 && n < count; d++) {
      if (n == count - 1) d = 1; /* closing bin is 1.e(last+1) */
      snprintf(buf, sizeof buf, "%d.e%d", d, e);
      out[n++] = strtod(buf, NULL);
    }
    e++;
  }
}

/* ------------------------------------------------------------------------------ */
/* module variables                                                                 */
/* ------------------------------------------------------------------------------ */
int dim_nrhg;
double av_g[nrhg], bv_g[nrhg];
double roverrv = 0.622, lfus, rho_not, rho_not0;
double am_i, am_r, am_g[nrhg], olfus, orv, ar_volume, sc3, d0i, xm0s, xm0g, obmi, obmr, oams,
    obms, ocms, oamg[nrhg], ocmg[nrhg], obmg;
double cce[15][5], ccg[15][5], ocg1[15], ocg2[15];
double cie[7], cig[7], oig1, oig2;
double cre[13], crg[13], ore1, org1, org2, org3;
double cse[17], csg[17];
double cge[nrhg][12], cgg[nrhg][12];
double oge1, ogg1, ogg2, ogg3;
double t1_qr_qc, t1_qr_qi, t2_qr_qi, t1_qs_qc, t1_qs_qi, t1_qr_ev, t2_qr_ev, t1_qs_sd, t2_qs_sd,
    t1_qs_me, t2_qs_me, t1_qg_sd, t1_qg_me;
int nic2, nii2, nii3, nir2, nir3, nis2, nig2, nig3, niin2;
double nic1;
double dc[nbc], dtc[nbc], di[nbi], dti[nbi], dr[nbr], dtr[nbr], ds[nbs], dts[nbs], dg[nbg],
    dtg[nbg], t_nc[nbc];
double hbins[nhbins], dhbins[nhbins];
double sbins_radar[radar_bins], dsbins_radar[radar_bins], gbins_radar[radar_bins],
    dgbins_radar[radar_bins];

double *t_efrw, *t_efsw, *tpc_wev, *tnc_wev;
float *tnccn_act;
double *tcg_racg, *tmr_racg, *tcr_gacr, *tnr_racg, *tnr_gacr;
double *tcs_racs1, *tmr_racs1, *tcs_racs2, *tmr_racs2, *tcr_sacr1, *tms_sacr1, *tcr_sacr2,
    *tms_sacr2, *tnr_racs1, *tnr_racs2, *tnr_sacr1, *tnr_sacr2;
double *tpi_qcfz, *tni_qcfz, *tpi_qrfz, *tpg_qrfz, *tni_qrfz, *tnr_qrfz;
double *tps_iaus, *tni_iaus, *tpi_ide;

static const double av_g_init[nrhg] = {45.9173813, 67.0867386, 98.0158463,
                                       122.353378, 143.204224, 161.794724,
                                       178.762115, 194.488785, 209.225876};

/* initialize_graupel_vars (params:411-426) */
void o_initialize_graupel_vars(int hail_flag) {
  for (int m = 0; m < nrhg; m++) {
    av_g[m] = av_g_init[m];
    bv_g[m] = 0.640961647;
  }
  if (hail_flag) {
    av_g[idx_bg1 - 1] = av_g_new;
    bv_g[idx_bg1 - 1] = bv_g_new;
    dim_nrhg = nrhg;
  } else {
    av_g[idx_bg1 - 1] = av_g_old;
    bv_g[idx_bg1 - 1] = bv_g_old;
    dim_nrhg = nrhg1;
  }
}

/* initialize_parameters (params:429-610) */
void o_initialize_parameters(void) {
  am_i = pi * rho_i / 6.0;
  am_r = pi * rho_w / 6.0;
  for (int m = 0; m < nrhg; m++) am_g[m] = pi * rho_g[m] / 6.0;
  ar_volume = 4.0 / 3.0 * pi * pow(2.5e-6, 3.0);
  lfus = lsub - lvap0;
  olfus = 1.0 / lfus;
  roverrv = rdry / rv;
  orv = 1.0 / rv;
  rho_not = 101325.0 / (rdry * 298.0);
  rho_not0 = 101325.0 / (rdry * t0);
  sc3 = pow(sc, 1.0 / 3.0);
  d0i = pow(xm0i / am_i, 1.0 / bm_i);
  xm0s = am_s * pow(d0s, bm_s);
  xm0g = am_g[nrhg - 1] * pow(d0g, bm_g);
  obmi = 1.0 / bm_i;
  obmr = 1.0 / bm_r;
  oams = 1.0 / am_s;
  obms = 1.0 / bm_s;
  ocms = pow(oams, obms);
  obmg = 1.0 / bm_g;
  for (int m = 0; m < nrhg; m++) {
    oamg[m] = 1.0 / am_g[m];
    ocmg[m] = pow(oamg[m], obmg);
  }
  for (int n = 1; n <= 15; n++) {
    CCE(1, n) = n + 1.0;
    CCE(2, n) = bm_r + n + 1.0;
    CCE(3, n) = bm_r + n + 4.0;
    CCE(4, n) = n + bv_c + 1.0;
    CCE(5, n) = bm_r + n + bv_c + 1.0;
    for (int r = 1; r <= 5; r++) CCG(r, n) = tgamma(CCE(r, n));
    OCG1(n) = 1.0 / CCG(1, n);
    OCG2(n) = 1.0 / CCG(2, n);
  }
  CIE(1) = mu_i + 1.0;
  CIE(2) = bm_i + mu_i + 1.0;
  CIE(3) = bm_i + mu_i + bv_i + 1.0;
  CIE(4) = mu_i + bv_i + 1.0;
  CIE(5) = mu_i + 2.0;
  CIE(6) = bm_i * 0.5 + mu_i + bv_i + 1.0;
  CIE(7) = bm_i * 0.5 + mu_i + 1.0;
  for (int n = 1; n <= 7; n++) CIG(n) = tgamma(CIE(n));
  oig1 = 1.0 / CIG(1);
  oig2 = 1.0 / CIG(2);
  CRE(1) = bm_r + 1.0;
  CRE(2) = mu_r + 1.0;
  CRE(3) = bm_r + mu_r + 1.0;
  CRE(4) = bm_r * 2.0 + mu_r + 1.0;
  CRE(5) = mu_r + bv_r + 1.0;
  CRE(6) = bm_r + mu_r + bv_r + 1.0;
  CRE(7) = bm_r * 0.5 + mu_r + bv_r + 1.0;
  CRE(8) = bm_r + mu_r + bv_r + 3.0;
  CRE(9) = mu_r + bv_r + 3.0;
  CRE(10) = mu_r + 2.0;
  CRE(11) = 0.5 * (bv_r + 5.0 + 2.0 * mu_r);
  CRE(12) = bm_r * 0.5 + mu_r + 1.0;
  CRE(13) = bm_r * 2.0 + mu_r + bv_r + 1.0;
  for (int n = 1; n <= 13; n++) CRG(n) = tgamma(CRE(n));
  ore1 = 1.0 / CRE(1);
  org1 = 1.0 / CRG(1);
  org2 = 1.0 / CRG(2);
  org3 = 1.0 / CRG(3);
  CSE(1) = bm_s + 1.0;
  CSE(2) = bm_s + 2.0;
  CSE(3) = bm_s * 2.0;
  CSE(4) = bm_s + bv_s + 1.0;
  CSE(5) = bm_s * 2.0 + bv_s + 1.0;
  CSE(6) = bm_s * 2.0 + 1.0;
  CSE(7) = bm_s + mu_s + 1.0;
  CSE(8) = bm_s + mu_s + 2.0;
  CSE(9) = bm_s + mu_s + 3.0;
  CSE(10) = bm_s + mu_s + bv_s + 1.0;
  CSE(11) = bm_s * 2.0 + mu_s + bv_s + 1.0;
  CSE(12) = bm_s * 2.0 + mu_s + 1.0;
  CSE(13) = bv_s + 2.0;
  CSE(14) = bm_s + bv_s;
  CSE(15) = mu_s + 1.0;
  CSE(16) = 1.0 + (1.0 + bv_s) / 2.0;
  CSE(17) = bm_s + bv_s + 2.0;
  for (int n = 1; n <= 17; n++) CSG(n) = tgamma(CSE(n));
  for (int m = 1; m <= nrhg; m++) {
    CGE(1, m) = bm_g + 1.0;
    CGE(2, m) = mu_g + 1.0;
    CGE(3, m) = bm_g + mu_g + 1.0;
    CGE(4, m) = bm_g * 2. + mu_g + 1.0;
    CGE(10, m) = mu_g + 2.0;
    CGE(12, m) = bm_g * 0.5 + mu_g + 1.0;
  }
  for (int m = 1; m <= nrhg; m++) {
    CGE(5, m) = bm_g * 2.0 + mu_g + BV_G(m) + 1.0;
    CGE(6, m) = bm_g + mu_g + BV_G(m) + 1.0;
    CGE(7, m) = bm_g * 0.5 + mu_g + BV_G(m) + 1.0;
    CGE(8, m) = mu_g + BV_G(m) + 1.0;
    CGE(9, m) = mu_g + BV_G(m) + 3.0;
    CGE(11, m) = 0.5 * (BV_G(m) + 5.0 + 2.0 * mu_g);
  }
  for (int m = 1; m <= nrhg; m++)
    for (int n = 1; n <= 12; n++) CGG(n, m) = tgamma(CGE(n, m));
  oge1 = 1.0 / CGE(1, 1);
  ogg1 = 1.0 / CGG(1, 1);
  ogg2 = 1.0 / CGG(2, 1);
  ogg3 = 1.0 / CGG(3, 1);
  t1_qr_qc = pi * 0.25 * av_r * CRG(9);
  t1_qr_qi = pi * 0.25 * av_r * CRG(9);
  t2_qr_qi = pi * 0.25 * am_r * av_r * CRG(8);
  t1_qs_qc = pi * 0.25 * av_s;
  t1_qs_qi = pi * 0.25 * av_s;
  t1_qr_ev = 0.78 * CRG(10);
  t2_qr_ev = 0.308 * sc3 * sqrt(av_r) * CRG(11);
  t1_qs_sd = 0.86;
  t2_qs_sd = 0.28 * sc3 * sqrt(av_s);
  t1_qs_me = pi * 4.0 * c_sqrd * olfus * 0.86;
  t2_qs_me = pi * 4.0 * c_sqrd * olfus * 0.28 * sc3 * sqrt(av_s);
  t1_qg_sd = 0.86 * CGG(10, 1);
  t1_qg_me = pi * 4.0 * c_cube * olfus * 0.86 * CGG(10, 1);
}

/* create_bins (params:695-722) */
static void create_bins(int numbins, double lowbin, double highbin, double *bins,
                        double *deltabins) {
  double xdx[201];
  xdx[0] = lowbin;
  xdx[numbins] = highbin;
  for (int n = 2; n <= numbins; n++)
    xdx[n - 1] = exp((double)(n - 1) / (double)numbins * log(xdx[numbins] / xdx[0]) + log(xdx[0]));
  for (int n = 1; n <= numbins; n++) bins[n - 1] = sqrt(xdx[n - 1] * xdx[n]);
  if (deltabins)
    for (int n = 1; n <= numbins; n++) deltabins[n - 1] = xdx[n] - xdx[n - 1];
}

/* initialize_bins_for_tables (params:613-658) */
static void initialize_bins_for_tables(void) {
  nic2 = nint(log10(r_c[0]));
  nii2 = nint(log10(r_i[0]));
  nir2 = nint(log10(r_r[0]));
  nis2 = nint(log10(r_s[0]));
  nig2 = nint(log10(r_g[0]));
  nii3 = nint(log10(nt_i[0]));
  nir3 = nint(log10(n0r_exp[0]));
  nig3 = nint(log10(n0g_exp[0]));
  niin2 = nint(log10(nt_in[0]));
  dc[0] = d0c;
  dtc[0] = d0c;
  for (int n = 2; n <= nbc; n++) {
    dc[n - 1] = dc[n - 2] + 1.0e-6;
    dtc[n - 1] = dc[n - 1] - dc[n - 2];
  }
  create_bins(nbi, d0i, 2.0 * d0s, di, dti);
  create_bins(nbr, d0r, 0.005, dr, dtr);
  create_bins(nbs, d0s, 0.02, ds, dts);
  create_bins(nbg, d0g, 0.05, dg, dtg);
  create_bins(nbc, 1.0, 3000.0, t_nc, NULL);
  for (int n = 0; n < nbc; n++) t_nc[n] = t_nc[n] * 1.0e6;
  nic1 = log(t_nc[nbc - 1] / t_nc[0]);
}

/* ------------------------------------------------------------------------------ */
/* utils.F90                                                                        */
/* ------------------------------------------------------------------------------ */
/* calc_gamma_series (utils:54-92) */
static double calc_gamma_series(double a, double x) {
  double aj = a, sum_term = 1.0 / tgamma(aj + 1.0), sum = sum_term;
  for (int k = 1; k <= 100; k++) {
    aj = aj + 1.0;
    sum_term = sum_term * x / aj;
    sum = sum + sum_term;
    if (fabs(sum_term) < (fabs(sum) * 1.e-7)) break;
  }
  return sum * pow(x, a) * exp(-x);
}
/* calc_gamma_cf (utils:95-145) */
static double calc_gamma_cf(double a, double x) {
  const double offset = 1.e-30, smallvalue = 1.e-7;
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
    if (fabs(delta - 1.0) < smallvalue) break;
  }
  return exp(-x + a * log(x)) * f / tgamma(a);
}
/* calc_gamma_p (utils:27-51) */
double o_calc_gamma_p(double a, double x) {
  if ((x < 0.0) || (a <= 0.0)) return NAN;
  if (x < (a + 1.0)) return calc_gamma_series(a, x);
  return 1.0 - calc_gamma_cf(a, x);
}

/* the moment-relation polynomial of snow_moments for moment order X (utils:190-199) */
static inline double poly_a(const double *s, double tc, double X) {
  return s[0] + s[1] * tc + s[2] * X + s[3] * tc * X + s[4] * tc * tc + s[5] * X * X +
         s[6] * tc * tc * X + s[7] * tc * X * X + s[8] * tc * tc * tc + s[9] * X * X * X;
}

/* snow_moments (utils:148-282).  NULL = optional argument absent. */
void o_snow_moments(double rs, double tc, double *smob, double *smoc, double *ns, double *smo0,
                    double *smo1, double *smo2, double *smoe, double *smof, double *smog,
                    double *smoz) {
  double loga_, a_, b_, smo2_, m0, mrat, slam1, slam2;
  *smob = rs * oams;
  if (bm_s > 2.0 - 1.e-3 && bm_s < 2.0 + 1.e-3) {
    loga_ = poly_a(sa, tc, bm_s);
    a_ = pow(10.0, loga_);
    b_ = poly_a(sb, tc, bm_s);
    smo2_ = pow(*smob / a_, 1.0 / b_);
  } else {
    smo2_ = *smob;
  }
  if (smo2) *smo2 = smo2_;
  loga_ = poly_a(sa, tc, CSE(1));
  a_ = pow(10.0, loga_);
  b_ = poly_a(sb, tc, CSE(1));
  *smoc = a_ * pow(smo2_, b_);
  loga_ = sa[0] + sa[1] * tc + sa[4] * tc * tc + sa[8] * tc * tc * tc;
  a_ = pow(10.0, loga_);
  b_ = sb[0] + sb[1] * tc + sb[4] * tc * tc + sb[8] * tc * tc * tc;
  if (smo0) *smo0 = a_ * pow(smo2_, b_);
  loga_ = sa[0] + sa[1] * tc + sa[2] + sa[3] * tc + sa[4] * tc * tc + sa[5] + sa[6] * tc * tc +
          sa[7] * tc + sa[8] * tc * tc * tc + sa[9];
  a_ = pow(10.0, loga_);
  b_ = sb[0] + sb[1] * tc + sb[2] + sb[3] * tc + sb[4] * tc * tc + sb[5] + sb[6] * tc * tc +
       sb[7] * tc + sb[8] * tc * tc * tc + sb[9];
  if (smo1) *smo1 = a_ * pow(smo2_, b_);
  m0 = *smob / *smoc;
  mrat = *smob * m0 * m0 * m0;
  slam1 = m0 * lam0;
  slam2 = m0 * lam1;
  if (ns) *ns = mrat * kap0 / slam1 + mrat * kap1 * pow(m0, mu_s) * CSG(15) / pow(slam2, CSE(15));
  loga_ = poly_a(sa, tc, CSE(13));
  a_ = pow(10.0, loga_);
  b_ = poly_a(sb, tc, CSE(13));
  if (smoe) *smoe = a_ * pow(smo2_, b_);
  loga_ = poly_a(sa, tc, CSE(16));
  a_ = pow(10.0, loga_);
  b_ = poly_a(sb, tc, CSE(16));
  if (smof) *smof = a_ * pow(smo2_, b_);
  loga_ = poly_a(sa, tc, CSE(17));
  a_ = pow(10.0, loga_);
  b_ = poly_a(sb, tc, CSE(17));
  if (smog) *smog = a_ * pow(smo2_, b_);
  loga_ = poly_a(sa, tc, CSE(3));
  a_ = pow(10.0, loga_);
  b_ = poly_a(sb, tc, CSE(3));
  /* utils:280 uses the smo2 argument, which is always passed together with smoz */
  if (smoz) *smoz = a_ * pow(smo2 ? *smo2 : smo2_, b_);
}

/* calc_rslf (utils:285-309) */
double o_calc_rslf(double p, double t) {
  const double c0 = .611583699E03, c1 = .444606896E02, c2 = .143177157e01, c3 = .264224321e-1,
               c4 = .299291081e-3, c5 = .203154182e-5, c6 = .702620698e-8,
               c7 = .379534310e-11, c8 = -.321582393e-13;
  double x = fmax2(-80.0, t - 273.16);
  double esl = c0 + x * (c1 + x * (c2 + x * (c3 + x * (c4 + x * (c5 + x * (c6 + x * (c7 + x * c8)))))));
  esl = fmin2(esl, p * 0.15);
  return .622 * esl / (p - esl);
}
/* calc_rsif (utils:312-331) */
double o_calc_rsif(double p, double t) {
  const double c0 = .609868993e03, c1 = .499320233e02, c2 = .184672631e01, c3 = .402737184e-1,
               c4 = .565392987e-3, c5 = .521693933e-5, c6 = .307839583e-7,
               c7 = .105785160e-9, c8 = .161444444e-12;
  double x = fmax2(-80.0, t - 273.16);
  double esi = c0 + x * (c1 + x * (c2 + x * (c3 + x * (c4 + x * (c5 + x * (c6 + x * (c7 + x * c8)))))));
  esi = fmin2(esi, p * 0.15);
  return .622 * esi / fmax2(1.e-4, (p - esi));
}
/* get_nuc (utils:334-346) */
int o_get_nuc(double nc) {
  if ((nu_c_scale / nc) >= 12.5) return 15;
  return imin(15, nint(nu_c_scale / nc) + 2);
}

/* compute_efrw (utils:349-400) */
static void compute_efrw(void) {
  for (int j = 1; j <= nbc; j++) {
    for (int i = 1; i <= nbr; i++) {
      double ef_rw = 0.0, p = dc[j - 1] / dr[i - 1];
      double dri = dr[i - 1], dcj = dc[j - 1];
      if (dri < 50.e-6 || dcj < 3.e-6) {
        T_EFRW(i, j) = 0.0;
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
      T_EFRW(i, j) = fmax2(0.0, fmin2(ef_rw, 0.95));
    }
  }
}

/* compute_efsw (utils:403-440) */
static void compute_efsw(void) {
  for (int j = 1; j <= nbc; j++) {
    double dcj = dc[j - 1];
    double vtc = 1.19e4 * (1.0e4 * dcj * dcj * 0.25);
    for (int i = 1; i <= nbs; i++) {
      double dsi = ds[i - 1];
      double vts = av_s * pow(dsi, bv_s) * exp(-fv_s * dsi) - vtc;
      double ds_m = pow(am_s * pow(dsi, bm_s) / am_r, obmr);
      double p = dcj / ds_m;
      if (p > 0.25 || dsi < d0s || dcj < 6.e-6 || vts < 1.e-3) {
        T_EFSW(i, j) = 0.0;
      } else {
        double stokes = dcj * dcj * vts * rho_w / (9. * 1.718e-5 * ds_m);
        double reynolds = 9.0 * stokes / (p * p * rho_w);
        double f = log(reynolds);
        double g = -0.1007 - 0.358 * f + 0.0261 * f * f;
        double k0 = exp(g);
        double z = log(stokes / (k0 + 1.e-15));
        double h = 0.1465 + 1.302 * z - 0.607 * z * z + 0.293 * z * z * z;
        double yc0 = 2.0 / pi * atan(h);
        double ef_sw = (yc0 + p) * (yc0 + p) / ((1. + p) * (1. + p));
        T_EFSW(i, j) = fmax2(0.0, fmin2(ef_sw, 0.95));
      }
    }
  }
}

/* qi_aut_qs (utils:443-490) */
static void qi_aut_qs(void) {
  double n_i[nbi];
  for (int j = 1; j <= ntb_i1; j++) {
    for (int i = 1; i <= ntb_i; i++) {
      double lami = pow(am_i * CIG(2) * oig1 * nt_i[j - 1] / r_i[i - 1], obmi);
      double di_mean = (bm_i + mu_i + 1.) / lami;
      double n0_i = nt_i[j - 1] * oig1 * pow(lami, CIE(1));
      double t1 = 0., t2 = 0.;
      if (di_mean > 5. * d0s) {
        t1 = r_i[i - 1];
        t2 = nt_i[j - 1];
        IAUS(tpi_ide, i, j) = 0.;
      } else if (di_mean < d0i) {
        t1 = 0.;
        t2 = 0.;
        IAUS(tpi_ide, i, j) = 1.;
      } else {
        double xlimit_intg = lami * d0s;
        IAUS(tpi_ide, i, j) = o_calc_gamma_p(mu_i + 2.0, xlimit_intg);
        for (int n2 = 1; n2 <= nbi; n2++) {
          n_i[n2 - 1] = n0_i * pow(di[n2 - 1], mu_i) * exp(-lami * di[n2 - 1]) * dti[n2 - 1];
          if (di[n2 - 1] >= d0s) {
            t1 = t1 + n_i[n2 - 1] * am_i * pow(di[n2 - 1], bm_i);
            t2 = t2 + n_i[n2 - 1];
          }
        }
      }
      IAUS(tps_iaus, i, j) = t1;
      IAUS(tni_iaus, i, j) = t2;
    }
  }
}

/* compute_drop_evap (utils:493-527) */
static void compute_drop_evap(void) {
  double n_c[nbc], massc[nbc];
  for (int n = 0; n < nbc; n++) massc[n] = am_r * pow(dc[n], bm_r);
  for (int k = 1; k <= nbc; k++) {
    int nu_c = o_get_nuc(t_nc[k - 1]);
    for (int j = 1; j <= ntb_c; j++) {
      double lamc = pow(t_nc[k - 1] * am_r * CCG(2, nu_c) * OCG1(nu_c) / r_c[j - 1], obmr);
      double n0_c = t_nc[k - 1] * OCG1(nu_c) * pow(lamc, CCE(1, nu_c));
      for (int i = 1; i <= nbc; i++) {
        n_c[i - 1] = n0_c * ipow(dc[i - 1], nu_c) * exp(-lamc * dc[i - 1]) * dtc[i - 1];
        double summ = 0., summ2 = 0.;
        for (int n = 1; n <= i; n++) {
          summ = summ + massc[n - 1] * n_c[n - 1];
          summ2 = summ2 + n_c[n - 1];
        }
        TPC_WEV(i, j, k) = summ;
        TNC_WEV(i, j, k) = summ2;
      }
    }
  }
}

static double *xalloc(long n) {
  double *p = (double *)calloc((size_t)n, sizeof(double));
  if (!p) {
    fprintf(stderr, "oracle: out of memory\n");
    abort();
  }
  return p;
}

static int g_initialized = 0;
static int g_hail = 1;

int oracle_init(int hailaware_flag) {
  static int bins_ready = 0;
  if (!bins_ready) {
    decade_bins(r_c, -6, ntb_c);
    decade_bins(r_i, -10, ntb_i);
    decade_bins(r_r, -6, ntb_r);
    decade_bins(r_s, -6, ntb_s);
    decade_bins(r_g, -6, ntb_g);
    decade_bins(n0r_exp, 6, ntb_r1);
    decade_bins(n0g_exp, 2, ntb_g1);
    decade_bins(nt_i, 0, ntb_i1);
    decade_bins(nt_in, 0, ntb_in);
    bins_ready = 1;
  }
  g_hail = hailaware_flag ? 1 : 0;
  o_initialize_graupel_vars(g_hail);
  o_initialize_parameters();
  initialize_bins_for_tables();
  if (!t_efrw) {
    t_efrw = xalloc((long)nbr * nbc);
    t_efsw = xalloc((long)nbs * nbc);
    tpc_wev = xalloc((long)nbc * ntb_c * nbc);
    tnc_wev = xalloc((long)nbc * ntb_c * nbc);
    tps_iaus = xalloc((long)ntb_i * ntb_i1);
    tni_iaus = xalloc((long)ntb_i * ntb_i1);
    tpi_ide = xalloc((long)ntb_i * ntb_i1);
    tnccn_act = (float *)calloc(CCN_COUNT, sizeof(float));
    tcg_racg = xalloc(QG_COUNT);
    tmr_racg = xalloc(QG_COUNT);
    tcr_gacr = xalloc(QG_COUNT);
    tnr_racg = xalloc(QG_COUNT);
    tnr_gacr = xalloc(QG_COUNT);
    double **qs[12] = {&tcs_racs1, &tmr_racs1, &tcs_racs2, &tmr_racs2, &tcr_sacr1, &tms_sacr1,
                       &tcr_sacr2, &tms_sacr2, &tnr_racs1, &tnr_racs2, &tnr_sacr1, &tnr_sacr2};
    for (int a = 0; a < 12; a++) *qs[a] = xalloc(QS_COUNT);
    tpi_qcfz = xalloc(QCFZ_COUNT);
    tni_qcfz = xalloc(QCFZ_COUNT);
    tpi_qrfz = xalloc(QRFZ_COUNT);
    tpg_qrfz = xalloc(QRFZ_COUNT);
    tni_qrfz = xalloc(QRFZ_COUNT);
    tnr_qrfz = xalloc(QRFZ_COUNT);
  }
  compute_efrw();
  compute_efsw();
  compute_drop_evap();
  qi_aut_qs();
  create_bins(nhbins, 500.e-6, 0.075, hbins, dhbins); /* initialize_bins_for_hail_size */
  /* initialize_bins_for_radar (params:674-692): snow 100 um to 2 cm, graupel to 5 cm */
  create_bins(radar_bins, 100.e-6, 0.02, sbins_radar, dsbins_radar);
  create_bins(radar_bins, 100.e-6, 0.05, gbins_radar, dgbins_radar);
  g_initialized = 1;
  return 0;
}

/* ------------------------------------------------------------------------------ */
/* table file I/O (driver:532-649; tables:96-444)                                   */
/* ------------------------------------------------------------------------------ */
static void bswap8(void *p, long n) {
  uint8_t *b = (uint8_t *)p;
  for (long i = 0; i < n; i++, b += 8)
    for (int k = 0; k < 4; k++) {
      uint8_t t = b[k];
      b[k] = b[7 - k];
      b[7 - k] = t;
    }
}
static void bswap4(void *p, long n) {
  uint8_t *b = (uint8_t *)p;
  for (long i = 0; i < n; i++, b += 4) {
    uint8_t t = b[0];
    b[0] = b[3];
    b[3] = t;
    t = b[1];
    b[1] = b[2];
    b[2] = t;
  }
}
static int host_is_little(void) {
  uint16_t x = 1;
  return *(uint8_t *)&x == 1;
}

static int read_stream(const char *path, double **arrs, int narr, long count) {
  FILE *f = fopen(path, "rb");
  if (!f) return -1;
  for (int a = 0; a < narr; a++) {
    if ((long)fread(arrs[a], 8, (size_t)count, f) != count) {
      fclose(f);
      return -2;
    }
    if (host_is_little()) bswap8(arrs[a], count);
  }
  fclose(f);
  return 0;
}
static int write_stream(const char *path, double **arrs, int narr, long count) {
  FILE *f = fopen(path, "wb");
  if (!f) return -1;
  double *tmp = xalloc(count);
  for (int a = 0; a < narr; a++) {
    memcpy(tmp, arrs[a], (size_t)count * 8);
    if (host_is_little()) bswap8(tmp, count);
    if ((long)fwrite(tmp, 8, (size_t)count, f) != count) {
      free(tmp);
      fclose(f);
      return -2;
    }
  }
  free(tmp);
  fclose(f);
  return 0;
}

int oracle_read_ccn(const char *path) {
  FILE *f = fopen(path, "rb");
  if (!f) return -1;
  uint8_t head[4], tail[4];
  if (fread(head, 1, 4, f) != 4) {
    fclose(f);
    return -2;
  }
  long nread = (long)fread(tnccn_act, 4, CCN_COUNT, f);
  if (nread != CCN_COUNT || fread(tail, 1, 4, f) != 4) {
    fclose(f);
    return -2;
  }
  fclose(f);
  uint32_t marker = ((uint32_t)head[0] << 24) | ((uint32_t)head[1] << 16) |
                    ((uint32_t)head[2] << 8) | head[3];
  if (marker != (uint32_t)(CCN_COUNT * 4) || memcmp(head, tail, 4) != 0) return -3;
  if (host_is_little()) bswap4(tnccn_act, CCN_COUNT);
  return 0;
}

#define FZ_ARRS double *fz[6] = {tpi_qrfz, tni_qrfz, tpg_qrfz, tnr_qrfz, tpi_qcfz, tni_qcfz}
#define QS_ARRS                                                                          \
  double *qsa[12] = {tcs_racs1, tmr_racs1, tcs_racs2, tmr_racs2, tcr_sacr1, tms_sacr1, \
                     tcr_sacr2, tms_sacr2, tnr_racs1, tnr_racs2, tnr_sacr1, tnr_sacr2}
#define QG_ARRS double *qga[5] = {tcg_racg, tmr_racg, tcr_gacr, tnr_racg, tnr_gacr}

int oracle_read_freezewater(const char *path) {
  FZ_ARRS;
  int rc = read_stream(path, fz, 4, QRFZ_COUNT);
  if (rc) return rc;
  /* the two cloud-water arrays follow the four rain arrays */
  FILE *f = fopen(path, "rb");
  if (!f) return -1;
  fseek(f, 4L * QRFZ_COUNT * 8, SEEK_SET);
  for (int a = 4; a < 6; a++) {
    if ((long)fread(fz[a], 8, QCFZ_COUNT, f) != QCFZ_COUNT) {
      fclose(f);
      return -2;
    }
    if (host_is_little()) bswap8(fz[a], QCFZ_COUNT);
  }
  fclose(f);
  return 0;
}
int oracle_write_freezewater(const char *path) {
  FZ_ARRS;
  FILE *f = fopen(path, "wb");
  if (!f) return -1;
  for (int a = 0; a < 6; a++) {
    long cnt = a < 4 ? QRFZ_COUNT : QCFZ_COUNT;
    double *tmp = xalloc(cnt);
    memcpy(tmp, fz[a], (size_t)cnt * 8);
    if (host_is_little()) bswap8(tmp, cnt);
    fwrite(tmp, 8, (size_t)cnt, f);
    free(tmp);
  }
  fclose(f);
  return 0;
}
int oracle_read_qr_acr_qs(const char *path) {
  QS_ARRS;
  return read_stream(path, qsa, 12, QS_COUNT);
}
int oracle_write_qr_acr_qs(const char *path) {
  QS_ARRS;
  return write_stream(path, qsa, 12, QS_COUNT);
}
int oracle_read_qr_acr_qg(const char *path) {
  QG_ARRS;
  return read_stream(path, qga, 5, QG_COUNT);
}
int oracle_write_qr_acr_qg(const char *path) {
  QG_ARRS;
  return write_stream(path, qga, 5, QG_COUNT);
}

/* ------------------------------------------------------------------------------ */
/* table builders (tables:493-805)                                                  */
/* ------------------------------------------------------------------------------ */
static void set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

/* rain fall speed polynomial at the rain bins (tables:519-522, 644-648) */
static void rain_bin_speeds(double *vr) {
  for (int n2 = 0; n2 < nbr; n2++) {
    double d = dr[n2];
    vr[n2] = -0.1021 + 4.932e3 * d - 0.9551e6 * d * d + 0.07934e9 * d * d * d -
             0.002362e12 * d * d * d * d;
  }
}
/* exponential rain PSD per bin for table indices (m,k) (tables:531-536) */
static void rain_psd(int m, int k, double *n_r) {
  double lam_exp = pow(n0r_exp[k - 1] * am_r * CRG(1) / r_r[m - 1], ore1);
  double lamr = lam_exp * pow(CRG(3) * org2 * org1, obmr);
  double n0_r = n0r_exp[k - 1] / (CRG(2) * lam_exp) * pow(lamr, CRE(2));
  for (int n2 = 0; n2 < nbr; n2++)
    n_r[n2] = n0_r * pow(dr[n2], mu_r) * exp(-lamr * dr[n2]) * dtr[n2];
}
/* snow PSD per bin for table indices (i,j) (tables:540-551) */
static void snow_psd(int i, int j, double *n_s) {
  double m2, m3;
  o_snow_moments(r_s[i - 1], tc_tab[j - 1], &m2, &m3, NULL, NULL, NULL, NULL, NULL, NULL, NULL,
                 NULL);
  double om3 = 1.0 / m3;
  double mrat = m2 * (m2 * om3) * (m2 * om3) * (m2 * om3);
  double m0 = pow(m2 * om3, mu_s);
  double slam1 = m2 * om3 * lam0;
  double slam2 = m2 * om3 * lam1;
  for (int n = 0; n < nbs; n++)
    n_s[n] = mrat * (kap0 * exp(-slam1 * ds[n]) + kap1 * m0 * pow(ds[n], mu_s) * exp(-slam2 * ds[n])) *
             dts[n];
}
/* graupel PSD per bin for table indices (i,j,n3) (tables:668-673) */
static void graupel_psd(int i, int j, int n3, double *n_g) {
  double lam_exp = pow(n0g_exp[i - 1] * AM_G(n3) * CGG(1, 1) / r_g[j - 1], oge1);
  double lamg = lam_exp * pow(CGG(3, 1) * ogg2 * ogg1, obmg);
  double n0_g = n0g_exp[i - 1] / (CGG(2, 1) * lam_exp) * pow(lamg, CGE(2, 1));
  for (int n = 0; n < nbg; n++) n_g[n] = n0_g * pow(dg[n], mu_g) * exp(-lamg * dg[n]) * dtg[n];
}

/* qr_acr_qs, one output entry, reference loop order (tables:553-616).  Expects the
 * hail-aware parameter set to be active. */
static void qs_entry_core(int i, int j, int k, int m, double out[12]) {
  double vr[nbr], vs[nbs], n_r[nbr], n_s[nbs];
  rain_bin_speeds(vr);
  for (int n = 0; n < nbs; n++) vs[n] = 1.5 * av_s * pow(ds[n], bv_s) * exp(-fv_s * ds[n]);
  rain_psd(m, k, n_r);
  snow_psd(i, j, n_s);
  double t1 = 0, t2 = 0, t3 = 0, t4 = 0, z1 = 0, z2 = 0, z3 = 0, z4 = 0, y1 = 0, y2 = 0, y3 = 0,
         y4 = 0;
  for (int n2 = 0; n2 < nbr; n2++) {
    double massr = am_r * pow(dr[n2], bm_r);
    for (int n = 0; n < nbs; n++) {
      double masss = am_s * pow(ds[n], bm_s);
      double dvs = 0.5 * ((vr[n2] - vs[n]) + fabs(vr[n2] - vs[n]));
      double dvr = 0.5 * ((vs[n] - vr[n2]) + fabs(vs[n] - vr[n2]));
      double geo = pi * .25 * ef_rs * (ds[n] + dr[n2]) * (ds[n] + dr[n2]);
      if (massr > 1.5 * masss) {
        t1 = t1 + geo * dvs * masss * n_s[n] * n_r[n2];
        z1 = z1 + geo * dvs * massr * n_s[n] * n_r[n2];
        y1 = y1 + geo * dvs * n_s[n] * n_r[n2];
      } else {
        t3 = t3 + geo * dvs * masss * n_s[n] * n_r[n2];
        z3 = z3 + geo * dvs * massr * n_s[n] * n_r[n2];
        y3 = y3 + geo * dvs * n_s[n] * n_r[n2];
      }
      if (massr > 1.5 * masss) {
        t2 = t2 + geo * dvr * massr * n_s[n] * n_r[n2];
        y2 = y2 + geo * dvr * n_s[n] * n_r[n2];
        z2 = z2 + geo * dvr * masss * n_s[n] * n_r[n2];
      } else {
        t4 = t4 + geo * dvr * massr * n_s[n] * n_r[n2];
        y4 = y4 + geo * dvr * n_s[n] * n_r[n2];
        z4 = z4 + geo * dvr * masss * n_s[n] * n_r[n2];
      }
    }
  }
  out[0] = t1;
  out[1] = fmin2(z1, r_r[m - 1]);
  out[2] = t3;
  out[3] = z3;
  out[4] = t2;
  out[5] = z2;
  out[6] = t4;
  out[7] = z4;
  out[8] = y1;
  out[9] = y3;
  out[10] = y2;
  out[11] = y4;
}
void oracle_qr_acr_qs_entry(int i, int j, int k, int m, double out[12]) {
  int saved = g_hail;
  o_initialize_graupel_vars(1);
  o_initialize_parameters();
  qs_entry_core(i, j, k, m, out);
  o_initialize_graupel_vars(saved);
  o_initialize_parameters();
}

/* qr_acr_qg, one output entry, reference loop order (tables:675-708).  Expects the
 * hail-aware parameter set to be active. */
static void qg_entry_core(int i, int j, int n3, int k, int m, double out[5]) {
  double vr[nbr], vg[nbg], n_r[nbr], n_g[nbg];
  rain_bin_speeds(vr);
  for (int n = 0; n < nbg; n++) vg[n] = AV_G(n3) * pow(dg[n], BV_G(n3));
  rain_psd(m, k, n_r);
  graupel_psd(i, j, n3, n_g);
  double t1 = 0, t2 = 0, z1 = 0, z2 = 0, y1 = 0, y2 = 0;
  for (int n2 = 0; n2 < nbr; n2++) {
    double massr = am_r * pow(dr[n2], bm_r);
    for (int n = 0; n < nbg; n++) {
      double massg = AM_G(n3) * pow(dg[n], bm_g);
      double dvg = 0.5 * ((vr[n2] - vg[n]) + fabs(vr[n2] - vg[n]));
      double dvr = 0.5 * ((vg[n] - vr[n2]) + fabs(vg[n] - vr[n2]));
      double geo = pi * .25 * ef_rg * (dg[n] + dr[n2]) * (dg[n] + dr[n2]);
      t1 = t1 + geo * dvg * massg * n_g[n] * n_r[n2];
      z1 = z1 + geo * dvg * massr * n_g[n] * n_r[n2];
      y1 = y1 + geo * dvg * n_g[n] * n_r[n2];
      t2 = t2 + geo * dvr * massr * n_g[n] * n_r[n2];
      y2 = y2 + geo * dvr * n_g[n] * n_r[n2];
      z2 = z2 + geo * dvr * massg * n_g[n] * n_r[n2];
    }
  }
  (void)z2; /* computed but never stored by the reference */
  out[0] = t1;
  out[1] = fmin2(z1, r_r[m - 1]);
  out[2] = t2;
  out[3] = y1;
  out[4] = y2;
}
void oracle_qr_acr_qg_entry(int i, int j, int n3, int k, int m, double out[5]) {
  int saved = g_hail;
  o_initialize_graupel_vars(1);
  o_initialize_parameters();
  qg_entry_core(i, j, n3, k, m, out);
  o_initialize_graupel_vars(saved);
  o_initialize_parameters();
}

/* qr_acr_qs for the whole table.  Factored form: every accumulator is
 *   sum_{n2,n} K(n2,n) n_s(n) n_r(n2) = sum_{n2} n_r(n2) [sum_n K(n2,n) n_s(n)]
 * with K >= 0, so only the summation order differs from the reference. */
int oracle_build_qr_acr_qs(int naive, int nthreads) {
  set_threads(nthreads);
  int saved = g_hail;
  o_initialize_graupel_vars(1);
  o_initialize_parameters();
  QS_ARRS;
  if (naive) {
#pragma omp parallel for collapse(2) schedule(dynamic)
    for (int m = 1; m <= ntb_r; m++)
      for (int k = 1; k <= ntb_r1; k++)
        for (int j = 1; j <= ntb_t; j++)
          for (int i = 1; i <= ntb_s; i++) {
            double out[12];
            qs_entry_core(i, j, k, m, out);
            for (int a = 0; a < 12; a++) QS4(qsa[a], i, j, k, m) = out[a];
          }
    o_initialize_graupel_vars(saved);
    o_initialize_parameters();
    return 0;
  }
  double vr[nbr], vs[nbs];
  rain_bin_speeds(vr);
  for (int n = 0; n < nbs; n++) vs[n] = 1.5 * av_s * pow(ds[n], bv_s) * exp(-fv_s * ds[n]);
  /* kernels K_a(n2,n) for the 12 accumulators, in output order */
  double *K = xalloc(12L * nbr * nbs);
  for (int n2 = 0; n2 < nbr; n2++) {
    double massr = am_r * pow(dr[n2], bm_r);
    for (int n = 0; n < nbs; n++) {
      double masss = am_s * pow(ds[n], bm_s);
      double dvs = 0.5 * ((vr[n2] - vs[n]) + fabs(vr[n2] - vs[n]));
      double dvr = 0.5 * ((vs[n] - vr[n2]) + fabs(vs[n] - vr[n2]));
      double geo = pi * .25 * ef_rs * (ds[n] + dr[n2]) * (ds[n] + dr[n2]);
      int big = massr > 1.5 * masss;
      double v[12] = {big ? geo * dvs * masss : 0, big ? geo * dvs * massr : 0,
                      big ? 0 : geo * dvs * masss, big ? 0 : geo * dvs * massr,
                      big ? geo * dvr * massr : 0, big ? geo * dvr * masss : 0,
                      big ? 0 : geo * dvr * massr, big ? 0 : geo * dvr * masss,
                      big ? geo * dvs : 0,         big ? 0 : geo * dvs,
                      big ? geo * dvr : 0,         big ? 0 : geo * dvr};
      for (int a = 0; a < 12; a++) K[((long)a * nbr + n2) * nbs + n] = v[a];
    }
  }
  double *NR = xalloc((long)ntb_r * ntb_r1 * nbr);
  for (int m = 1; m <= ntb_r; m++)
    for (int k = 1; k <= ntb_r1; k++) rain_psd(m, k, NR + (((long)(m - 1) * ntb_r1 + (k - 1)) * nbr));
#pragma omp parallel for collapse(2) schedule(dynamic)
  for (int j = 1; j <= ntb_t; j++)
    for (int i = 1; i <= ntb_s; i++) {
      double n_s[nbs], G[12][nbr];
      snow_psd(i, j, n_s);
      for (int a = 0; a < 12; a++)
        for (int n2 = 0; n2 < nbr; n2++) {
          const double *Kr = K + ((long)a * nbr + n2) * nbs;
          double s = 0;
          for (int n = 0; n < nbs; n++) s += Kr[n] * n_s[n];
          G[a][n2] = s;
        }
      for (int m = 1; m <= ntb_r; m++)
        for (int k = 1; k <= ntb_r1; k++) {
          const double *nr_ = NR + (((long)(m - 1) * ntb_r1 + (k - 1)) * nbr);
          for (int a = 0; a < 12; a++) {
            double s = 0;
            for (int n2 = 0; n2 < nbr; n2++) s += nr_[n2] * G[a][n2];
            if (a == 1) s = fmin2(s, r_r[m - 1]);
            QS4(qsa[a], i, j, k, m) = s;
          }
        }
    }
  free(K);
  free(NR);
  o_initialize_graupel_vars(saved);
  o_initialize_parameters();
  return 0;
}

/* qr_acr_qg for the whole table (factored as in oracle_build_qr_acr_qs). */
int oracle_build_qr_acr_qg(int naive, int nthreads) {
  set_threads(nthreads);
  int saved = g_hail;
  o_initialize_graupel_vars(1);
  o_initialize_parameters();
  QG_ARRS;
  if (naive) {
#pragma omp parallel for collapse(2) schedule(dynamic)
    for (int m = 1; m <= ntb_r; m++)
      for (int k = 1; k <= ntb_r1; k++)
        for (int n3 = 1; n3 <= nrhg; n3++)
          for (int j = 1; j <= ntb_g; j++)
            for (int i = 1; i <= ntb_g1; i++) {
              double out[5];
              qg_entry_core(i, j, n3, k, m, out);
              for (int a = 0; a < 5; a++) QG5(qga[a], i, j, n3, k, m) = out[a];
            }
    o_initialize_graupel_vars(saved);
    o_initialize_parameters();
    return 0;
  }
  double vr[nbr];
  rain_bin_speeds(vr);
  /* kernels for t1 (dvg*massg), z1 (dvg*massr), t2 (dvr*massr), y1 (dvg), y2 (dvr) */
  double *K = xalloc((long)nrhg * 5 * nbr * nbg);
  for (int n3 = 1; n3 <= nrhg; n3++)
    for (int n2 = 0; n2 < nbr; n2++) {
      double massr = am_r * pow(dr[n2], bm_r);
      for (int n = 0; n < nbg; n++) {
        double vg = AV_G(n3) * pow(dg[n], BV_G(n3));
        double massg = AM_G(n3) * pow(dg[n], bm_g);
        double dvg = 0.5 * ((vr[n2] - vg) + fabs(vr[n2] - vg));
        double dvr = 0.5 * ((vg - vr[n2]) + fabs(vg - vr[n2]));
        double geo = pi * .25 * ef_rg * (dg[n] + dr[n2]) * (dg[n] + dr[n2]);
        double v[5] = {geo * dvg * massg, geo * dvg * massr, geo * dvr * massr, geo * dvg,
                       geo * dvr};
        for (int a = 0; a < 5; a++) K[(((long)(n3 - 1) * 5 + a) * nbr + n2) * nbg + n] = v[a];
      }
    }
  double *NR = xalloc((long)ntb_r * ntb_r1 * nbr);
  for (int m = 1; m <= ntb_r; m++)
    for (int k = 1; k <= ntb_r1; k++) rain_psd(m, k, NR + (((long)(m - 1) * ntb_r1 + (k - 1)) * nbr));
#pragma omp parallel for collapse(3) schedule(dynamic)
  for (int n3 = 1; n3 <= nrhg; n3++)
    for (int j = 1; j <= ntb_g; j++)
      for (int i = 1; i <= ntb_g1; i++) {
        double n_g[nbg], G[5][nbr];
        graupel_psd(i, j, n3, n_g);
        for (int a = 0; a < 5; a++)
          for (int n2 = 0; n2 < nbr; n2++) {
            const double *Kr = K + (((long)(n3 - 1) * 5 + a) * nbr + n2) * nbg;
            double s = 0;
            for (int n = 0; n < nbg; n++) s += Kr[n] * n_g[n];
            G[a][n2] = s;
          }
        for (int m = 1; m <= ntb_r; m++)
          for (int k = 1; k <= ntb_r1; k++) {
            const double *nr_ = NR + (((long)(m - 1) * ntb_r1 + (k - 1)) * nbr);
            for (int a = 0; a < 5; a++) {
              double s = 0;
              for (int n2 = 0; n2 < nbr; n2++) s += nr_[n2] * G[a][n2];
              if (a == 1) s = fmin2(s, r_r[m - 1]);
              QG5(qga[a], i, j, n3, k, m) = s;
            }
          }
      }
  free(K);
  free(NR);
  o_initialize_graupel_vars(saved);
  o_initialize_parameters();
  return 0;
}

/* freezewater (tables:717-805).  The per-bin drop PSD and freezing probability do not
 * depend on the loop indices that enclose them in the reference, so they are
 * evaluated once with the same expressions; the prefix sums and their early exits
 * are kept in the reference's order. */
int oracle_build_freezewater(int nthreads) {
  set_threads(nthreads);
  int saved = g_hail;
  o_initialize_graupel_vars(1);
  o_initialize_parameters();
  double massr[nbr], massc[nbc];
  double orho_w = 1.0 / rho_w;
  for (int n2 = 0; n2 < nbr; n2++) massr[n2] = am_r * pow(dr[n2], bm_r);
  for (int n = 0; n < nbc; n++) massc[n] = am_r * pow(dc[n], bm_r);
  double *NR = xalloc((long)ntb_r * ntb_r1 * nbr); /* [i][j][n2] */
  for (int j = 1; j <= ntb_r1; j++)
    for (int i = 1; i <= ntb_r; i++) {
      double lam_exp = pow(n0r_exp[j - 1] * am_r * CRG(1) / r_r[i - 1], ore1);
      double lamr = lam_exp * pow(CRG(3) * org2 * org1, obmr);
      double n0_r = n0r_exp[j - 1] / (CRG(2) * lam_exp) * pow(lamr, CRE(2));
      double *o = NR + (((long)(i - 1) * ntb_r1 + (j - 1)) * nbr);
      for (int n2 = 0; n2 < nbr; n2++)
        o[n2] = n0_r * pow(dr[n2], mu_r) * exp(-lamr * dr[n2]) * dtr[n2];
    }
  double *NC = xalloc((long)nbc * ntb_c * nbc); /* [j][i][n] */
  for (int j = 1; j <= nbc; j++) {
    int nu_c = imin(15, nint(nu_c_scale / t_nc[j - 1]) + 2);
    for (int i = 1; i <= ntb_c; i++) {
      double lamc = pow(t_nc[j - 1] * am_r * CCG(2, nu_c) * OCG1(nu_c) / r_c[i - 1], obmr);
      double n0_c = t_nc[j - 1] * OCG1(nu_c) * pow(lamc, CCE(1, nu_c));
      double *o = NC + (((long)(j - 1) * ntb_c + (i - 1)) * nbc);
      for (int n = 0; n < nbc; n++)
        o[n] = n0_c * ipow(dc[n], nu_c) * exp(-lamc * dc[n]) * dtc[n];
    }
  }
#pragma omp parallel for collapse(2) schedule(dynamic)
  for (int m = 1; m <= ntb_in; m++)
    for (int k = 1; k <= 45; k++) {
      double t_adjust = fmax2(-3.0, fmin2(3.0 - log10(nt_in[m - 1]), 3.0));
      double texp = exp((double)k - t_adjust) - 1.0;
      double probr[nbr], probc[nbc];
      for (int n2 = 0; n2 < nbr; n2++) {
        double vol = massr[n2] * orho_w;
        probr[n2] = fmax2(0.0, 1.0 - exp(-120.0 * vol * 5.2e-4 * texp));
      }
      for (int n = 0; n < nbc; n++) {
        double vol = massc[n] * orho_w;
        probc[n] = fmax2(0.0, 1.0 - exp(-120.0 * vol * 5.2e-4 * texp));
      }
      for (int j = 1; j <= ntb_r1; j++)
        for (int i = 1; i <= ntb_r; i++) {
          const double *nr_ = NR + (((long)(i - 1) * ntb_r1 + (j - 1)) * nbr);
          double sum1 = 0, sum2 = 0, sumn1 = 0, sumn2 = 0;
          for (int n2 = nbr; n2 >= 1; n2--) {
            double n_r = nr_[n2 - 1], prob = probr[n2 - 1];
            if (massr[n2 - 1] < xm0g) {
              sumn1 = sumn1 + prob * n_r;
              sum1 = sum1 + prob * n_r * massr[n2 - 1];
            } else {
              sumn2 = sumn2 + prob * n_r;
              sum2 = sum2 + prob * n_r * massr[n2 - 1];
            }
            if ((sum1 + sum2) >= r_r[i - 1]) break;
          }
          QRFZ(tpi_qrfz, i, j, k, m) = sum1;
          QRFZ(tni_qrfz, i, j, k, m) = sumn1;
          QRFZ(tpg_qrfz, i, j, k, m) = sum2;
          QRFZ(tnr_qrfz, i, j, k, m) = sumn2;
        }
      for (int j = 1; j <= nbc; j++)
        for (int i = 1; i <= ntb_c; i++) {
          const double *nc_ = NC + (((long)(j - 1) * ntb_c + (i - 1)) * nbc);
          double sum1 = 0, sumn2 = 0;
          for (int n = nbc; n >= 1; n--) {
            double prob = probc[n - 1], n_c = nc_[n - 1];
            sumn2 = fmin2(t_nc[j - 1], sumn2 + prob * n_c);
            sum1 = sum1 + prob * n_c * massc[n - 1];
            if (sum1 >= r_c[i - 1]) break;
          }
          QCFZ(tpi_qcfz, i, j, k, m) = sum1;
          QCFZ(tni_qcfz, i, j, k, m) = sumn2;
        }
    }
  free(NR);
  free(NC);
  o_initialize_graupel_vars(saved);
  o_initialize_parameters();
  return 0;
}

/* ------------------------------------------------------------------------------ */
/* accessors                                                                        */
/* ------------------------------------------------------------------------------ */
double *oracle_table_ptr(const char *name, long *count) {
  struct {
    const char *n;
    double **p;
    long c;
  } tab[] = {{"t_efrw", &t_efrw, (long)nbr * nbc},      {"t_efsw", &t_efsw, (long)nbs * nbc},
             {"tpc_wev", &tpc_wev, (long)nbc * ntb_c * nbc},
             {"tnc_wev", &tnc_wev, (long)nbc * ntb_c * nbc},
             {"tps_iaus", &tps_iaus, (long)ntb_i * ntb_i1},
             {"tni_iaus", &tni_iaus, (long)ntb_i * ntb_i1},
             {"tpi_ide", &tpi_ide, (long)ntb_i * ntb_i1},
             {"tcg_racg", &tcg_racg, QG_COUNT},         {"tmr_racg", &tmr_racg, QG_COUNT},
             {"tcr_gacr", &tcr_gacr, QG_COUNT},         {"tnr_racg", &tnr_racg, QG_COUNT},
             {"tnr_gacr", &tnr_gacr, QG_COUNT},         {"tcs_racs1", &tcs_racs1, QS_COUNT},
             {"tmr_racs1", &tmr_racs1, QS_COUNT},       {"tcs_racs2", &tcs_racs2, QS_COUNT},
             {"tmr_racs2", &tmr_racs2, QS_COUNT},       {"tcr_sacr1", &tcr_sacr1, QS_COUNT},
             {"tms_sacr1", &tms_sacr1, QS_COUNT},       {"tcr_sacr2", &tcr_sacr2, QS_COUNT},
             {"tms_sacr2", &tms_sacr2, QS_COUNT},       {"tnr_racs1", &tnr_racs1, QS_COUNT},
             {"tnr_racs2", &tnr_racs2, QS_COUNT},       {"tnr_sacr1", &tnr_sacr1, QS_COUNT},
             {"tnr_sacr2", &tnr_sacr2, QS_COUNT},       {"tpi_qrfz", &tpi_qrfz, QRFZ_COUNT},
             {"tni_qrfz", &tni_qrfz, QRFZ_COUNT},       {"tpg_qrfz", &tpg_qrfz, QRFZ_COUNT},
             {"tnr_qrfz", &tnr_qrfz, QRFZ_COUNT},       {"tpi_qcfz", &tpi_qcfz, QCFZ_COUNT},
             {"tni_qcfz", &tni_qcfz, QCFZ_COUNT}};
  for (size_t a = 0; a < sizeof tab / sizeof tab[0]; a++)
    if (!strcmp(name, tab[a].n)) {
      if (count) *count = tab[a].c;
      return *tab[a].p;
    }
  if (count) *count = 0;
  return NULL;
}
float *oracle_ccn_ptr(long *count) {
  if (count) *count = CCN_COUNT;
  return tnccn_act;
}

double oracle_param(const char *name, int idx) {
#define S(nm, v)                            \
  if (!strcmp(name, nm)) return (double)(v)
#define A(nm, arr, n)                       \
  if (!strcmp(name, nm)) return (idx >= 0 && idx < (n)) ? (double)((arr)[idx]) : NAN
  S("dim_nrhg", dim_nrhg);
  S("am_i", am_i);
  S("am_r", am_r);
  S("roverrv", roverrv);
  S("lfus", lfus);
  S("olfus", olfus);
  S("orv", orv);
  S("rho_not", rho_not);
  S("rho_not0", rho_not0);
  S("ar_volume", ar_volume);
  S("sc3", sc3);
  S("d0i", d0i);
  S("xm0s", xm0s);
  S("xm0g", xm0g);
  S("ocms", ocms);
  S("oig1", oig1);
  S("oig2", oig2);
  S("ore1", ore1);
  S("org1", org1);
  S("org2", org2);
  S("org3", org3);
  S("oge1", oge1);
  S("ogg1", ogg1);
  S("ogg2", ogg2);
  S("ogg3", ogg3);
  S("t1_qr_qc", t1_qr_qc);
  S("t1_qr_qi", t1_qr_qi);
  S("t2_qr_qi", t2_qr_qi);
  S("t1_qs_qc", t1_qs_qc);
  S("t1_qs_qi", t1_qs_qi);
  S("t1_qr_ev", t1_qr_ev);
  S("t2_qr_ev", t2_qr_ev);
  S("t1_qs_sd", t1_qs_sd);
  S("t2_qs_sd", t2_qs_sd);
  S("t1_qs_me", t1_qs_me);
  S("t2_qs_me", t2_qs_me);
  S("t1_qg_sd", t1_qg_sd);
  S("t1_qg_me", t1_qg_me);
  S("nic1", nic1);
  S("nic2", nic2);
  S("nii2", nii2);
  S("nii3", nii3);
  S("nir2", nir2);
  S("nir3", nir3);
  S("nis2", nis2);
  S("nig2", nig2);
  S("nig3", nig3);
  S("niin2", niin2);
  A("am_g", am_g, nrhg);
  A("av_g", av_g, nrhg);
  A("bv_g", bv_g, nrhg);
  A("ocmg", ocmg, nrhg);
  A("cce", &cce[0][0], 75);
  A("ccg", &ccg[0][0], 75);
  A("ocg1", ocg1, 15);
  A("ocg2", ocg2, 15);
  A("cie", cie, 7);
  A("cig", cig, 7);
  A("cre", cre, 13);
  A("crg", crg, 13);
  A("cse", cse, 17);
  A("csg", csg, 17);
  A("cge", &cge[0][0], 108);
  A("cgg", &cgg[0][0], 108);
  A("dc", dc, nbc);
  A("dtc", dtc, nbc);
  A("di", di, nbi);
  A("dti", dti, nbi);
  A("dr", dr, nbr);
  A("dtr", dtr, nbr);
  A("ds", ds, nbs);
  A("dts", dts, nbs);
  A("dg", dg, nbg);
  A("dtg", dtg, nbg);
  A("t_nc", t_nc, nbc);
  A("hbins", hbins, nhbins);
  A("dhbins", dhbins, nhbins);
  A("r_c", r_c, ntb_c);
  A("r_i", r_i, ntb_i);
  A("r_r", r_r, ntb_r);
  A("r_s", r_s, ntb_s);
  A("r_g", r_g, ntb_g);
  A("n0r_exp", n0r_exp, ntb_r1);
  A("n0g_exp", n0g_exp, ntb_g1);
  A("nt_i", nt_i, ntb_i1);
  A("nt_in", nt_in, ntb_in);
  A("tc", tc_tab, ntb_t);
#undef S
#undef A
  return NAN;
}

double oracle_calc_gamma_p(double a, double x) { return o_calc_gamma_p(a, x); }
double oracle_calc_rslf(double p, double t) { return o_calc_rslf(p, t); }
double oracle_calc_rsif(double p, double t) { return o_calc_rsif(p, t); }
void oracle_snow_moments(double rs, double tc, double out[10]) {
  o_snow_moments(rs, tc, &out[0], &out[1], &out[2], &out[3], &out[4], &out[5], &out[6], &out[7],
                 &out[8], &out[9]);
}
void oracle_default_cfgs(ocfg_t *c) {
  memset(c, 0, sizeof *c);
  c->aerosolaware_flag = 1;
  c->hailaware_flag = 1;
  c->cloud_condensation_flag = 1;
  strcpy(c->single_moment_nc_opt, "land");
  c->refl10cm_flag = 1;
  c->re_cloud_flag = 1;
  c->re_ice_flag = 1;
  c->re_snow_flag = 1;
  c->max_hail_diameter_flag = 1;
}
