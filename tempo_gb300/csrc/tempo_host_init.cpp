// tempo_host_init.cpp -- host-side derivation of the scheme constants and table bins.
//
// Restates tempo_init's scalar set-up: initialize_graupel_vars
// (src/module_mp_tempo_params.F90:411-426), initialize_parameters (:429-610),
// initialize_bins_for_tables (:613-658), initialize_bins_for_hail_size (:661-671)
// and create_bins (:695-722).  Gamma values use the C library tgamma, the same
// routine the Fortran GAMMA intrinsic calls under gfortran.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "tempo_consts.h"

namespace tg {

namespace {

// The mass/number bins are the decimal literals d.eE (d = 1..9) of consecutive
// decades closed by 1.e(last+1) (params:194-263); parsing those strings yields the
// same doubles as the Fortran literals.
void decade_bins(double* out, int first_exp, int count) {
  char buf[32];
  int n = 0, e = first_exp;
  while (n < count) {
    for (int d = 1; d <= 9 && n < count; d++) {
      const int digit = (n == count - 1) ? 1 : d;
      std::snprintf(buf, sizeof buf, "%d.e%d", digit, e);
      out[n++] = std::strtod(buf, nullptr);
    }
    e++;
  }
}

void create_bins(int numbins, double lowbin, double highbin, double* bins, double* deltabins) {
  double xdx[201];
  xdx[0] = lowbin;
  xdx[numbins] = highbin;
  for (int n = 2; n <= numbins; n++)
    xdx[n - 1] = std::exp((double)(n - 1) / (double)numbins * std::log(xdx[numbins] / xdx[0]) +
                          std::log(xdx[0]));
  for (int n = 1; n <= numbins; n++) bins[n - 1] = std::sqrt(xdx[n - 1] * xdx[n]);
  if (deltabins)
    for (int n = 1; n <= numbins; n++) deltabins[n - 1] = xdx[n] - xdx[n - 1];
}

int nint_host(double x) { return (int)std::lround(x); }

}  // namespace

void make_bins(TempoBins* b) {
  decade_bins(b->r_c, -6, ntb_c);
  decade_bins(b->r_i, -10, ntb_i);
  decade_bins(b->r_r, -6, ntb_r);
  decade_bins(b->r_s, -6, ntb_s);
  decade_bins(b->r_g, -6, ntb_g);
  decade_bins(b->n0r_exp, 6, ntb_r1);
  decade_bins(b->n0g_exp, 2, ntb_g1);
  decade_bins(b->nt_i, 0, ntb_i1);
  decade_bins(b->nt_in, 0, ntb_in);
  const double tcv[ntb_t] = {-0.01, -5., -10., -15., -20., -25., -30., -35., -40.};
  std::memcpy(b->tc, tcv, sizeof tcv);
  const double am_i = pi * rho_i / 6.0;
  const double d0i = std::pow(xm0i / am_i, 1.0 / bm_i);
  b->dc[0] = d0c;
  b->dtc[0] = d0c;
  for (int n = 2; n <= nbc; n++) {
    b->dc[n - 1] = b->dc[n - 2] + 1.0e-6;
    b->dtc[n - 1] = b->dc[n - 1] - b->dc[n - 2];
  }
  create_bins(nbi, d0i, 2.0 * d0s, b->di, b->dti);
  create_bins(nbr, d0r, 0.005, b->dr, b->dtr);
  create_bins(nbs, d0s, 0.02, b->ds, b->dts);
  create_bins(nbg, d0g, 0.05, b->dg, b->dtg);
  create_bins(nbc, 1.0, 3000.0, b->t_nc, nullptr);
  for (int n = 0; n < nbc; n++) b->t_nc[n] = b->t_nc[n] * 1.0e6;
}

void make_consts(TempoConsts<double>* c, bool hailaware) {
  std::memset(c, 0, sizeof *c);
  static const double av_g_init[nrhg] = {45.9173813, 67.0867386, 98.0158463,
                                         122.353378, 143.204224, 161.794724,
                                         178.762115, 194.488785, 209.225876};
  static const double rho_g[nrhg] = {50., 100., 200., 300., 400., 500., 600., 700., 800.};
  for (int m = 0; m < nrhg; m++) {
    c->av_g[m] = av_g_init[m];
    c->bv_g[m] = 0.640961647;
  }
  c->av_g[idx_bg1 - 1] = hailaware ? av_g_new : av_g_old;
  c->bv_g[idx_bg1 - 1] = hailaware ? bv_g_new : bv_g_old;
  c->dim_nrhg = hailaware ? nrhg : 1;

  c->am_i = pi * rho_i / 6.0;
  c->am_r = pi * rho_w / 6.0;
  for (int m = 0; m < nrhg; m++) c->am_g[m] = pi * rho_g[m] / 6.0;
  c->ar_volume = 4.0 / 3.0 * pi * std::pow(2.5e-6, 3.0);
  c->lfus = lsub - lvap0;
  c->olfus = 1.0 / c->lfus;
  c->roverrv = rdry / rv;
  c->orv = 1.0 / rv;
  c->rho_not = 101325.0 / (rdry * 298.0);
  c->rho_not0 = 101325.0 / (rdry * t0);
  c->sc3 = std::pow(sc, 1.0 / 3.0);
  c->d0i = std::pow(xm0i / c->am_i, 1.0 / bm_i);
  c->xm0s = am_s * std::pow(d0s, bm_s);
  c->xm0g = c->am_g[nrhg - 1] * std::pow(d0g, bm_g);
  c->obmi = 1.0 / bm_i;
  c->obmr = 1.0 / bm_r;
  c->oams = 1.0 / am_s;
  c->obms = 1.0 / bm_s;
  c->ocms = std::pow(c->oams, c->obms);
  c->obmg = 1.0 / bm_g;
  for (int m = 0; m < nrhg; m++) {
    c->oamg[m] = 1.0 / c->am_g[m];
    c->ocmg[m] = std::pow(c->oamg[m], c->obmg);
  }
  for (int n = 1; n <= 15; n++) {
    double* e = c->cce[n - 1];
    e[0] = n + 1.0;
    e[1] = bm_r + n + 1.0;
    e[2] = bm_r + n + 4.0;
    e[3] = n + bv_c + 1.0;
    e[4] = bm_r + n + bv_c + 1.0;
    for (int r = 0; r < 5; r++) c->ccg[n - 1][r] = std::tgamma(e[r]);
    c->ocg1[n - 1] = 1.0 / c->ccg[n - 1][0];
    c->ocg2[n - 1] = 1.0 / c->ccg[n - 1][1];
  }
  c->cie[0] = mu_i + 1.0;
  c->cie[1] = bm_i + mu_i + 1.0;
  c->cie[2] = bm_i + mu_i + bv_i + 1.0;
  c->cie[3] = mu_i + bv_i + 1.0;
  c->cie[4] = mu_i + 2.0;
  c->cie[5] = bm_i * 0.5 + mu_i + bv_i + 1.0;
  c->cie[6] = bm_i * 0.5 + mu_i + 1.0;
  for (int n = 0; n < 7; n++) c->cig[n] = std::tgamma(c->cie[n]);
  c->oig1 = 1.0 / c->cig[0];
  c->oig2 = 1.0 / c->cig[1];
  double* cre = c->cre;
  cre[0] = bm_r + 1.0;
  cre[1] = mu_r + 1.0;
  cre[2] = bm_r + mu_r + 1.0;
  cre[3] = bm_r * 2.0 + mu_r + 1.0;
  cre[4] = mu_r + bv_r + 1.0;
  cre[5] = bm_r + mu_r + bv_r + 1.0;
  cre[6] = bm_r * 0.5 + mu_r + bv_r + 1.0;
  cre[7] = bm_r + mu_r + bv_r + 3.0;
  cre[8] = mu_r + bv_r + 3.0;
  cre[9] = mu_r + 2.0;
  cre[10] = 0.5 * (bv_r + 5.0 + 2.0 * mu_r);
  cre[11] = bm_r * 0.5 + mu_r + 1.0;
  cre[12] = bm_r * 2.0 + mu_r + bv_r + 1.0;
  for (int n = 0; n < 13; n++) c->crg[n] = std::tgamma(cre[n]);
  c->ore1 = 1.0 / cre[0];
  c->org1 = 1.0 / c->crg[0];
  c->org2 = 1.0 / c->crg[1];
  c->org3 = 1.0 / c->crg[2];
  double* cse = c->cse;
  cse[0] = bm_s + 1.0;
  cse[1] = bm_s + 2.0;
  cse[2] = bm_s * 2.0;
  cse[3] = bm_s + bv_s + 1.0;
  cse[4] = bm_s * 2.0 + bv_s + 1.0;
  cse[5] = bm_s * 2.0 + 1.0;
  cse[6] = bm_s + mu_s + 1.0;
  cse[7] = bm_s + mu_s + 2.0;
  cse[8] = bm_s + mu_s + 3.0;
  cse[9] = bm_s + mu_s + bv_s + 1.0;
  cse[10] = bm_s * 2.0 + mu_s + bv_s + 1.0;
  cse[11] = bm_s * 2.0 + mu_s + 1.0;
  cse[12] = bv_s + 2.0;
  cse[13] = bm_s + bv_s;
  cse[14] = mu_s + 1.0;
  cse[15] = 1.0 + (1.0 + bv_s) / 2.0;
  cse[16] = bm_s + bv_s + 2.0;
  for (int n = 0; n < 17; n++) c->csg[n] = std::tgamma(cse[n]);
  for (int m = 0; m < nrhg; m++) {
    double* g = c->cge[m];
    g[0] = bm_g + 1.0;
    g[1] = mu_g + 1.0;
    g[2] = bm_g + mu_g + 1.0;
    g[3] = bm_g * 2. + mu_g + 1.0;
    g[9] = mu_g + 2.0;
    g[11] = bm_g * 0.5 + mu_g + 1.0;
    g[4] = bm_g * 2.0 + mu_g + c->bv_g[m] + 1.0;
    g[5] = bm_g + mu_g + c->bv_g[m] + 1.0;
    g[6] = bm_g * 0.5 + mu_g + c->bv_g[m] + 1.0;
    g[7] = mu_g + c->bv_g[m] + 1.0;
    g[8] = mu_g + c->bv_g[m] + 3.0;
    g[10] = 0.5 * (c->bv_g[m] + 5.0 + 2.0 * mu_g);
    for (int n = 0; n < 12; n++) c->cgg[m][n] = std::tgamma(g[n]);
  }
  c->oge1 = 1.0 / c->cge[0][0];
  c->ogg1 = 1.0 / c->cgg[0][0];
  c->ogg2 = 1.0 / c->cgg[0][1];
  c->ogg3 = 1.0 / c->cgg[0][2];
  c->t1_qr_qc = pi * 0.25 * av_r * c->crg[8];
  c->t1_qr_qi = pi * 0.25 * av_r * c->crg[8];
  c->t2_qr_qi = pi * 0.25 * c->am_r * av_r * c->crg[7];
  c->t1_qs_qc = pi * 0.25 * av_s;
  c->t1_qs_qi = pi * 0.25 * av_s;
  c->t1_qr_ev = 0.78 * c->crg[9];
  c->t2_qr_ev = 0.308 * c->sc3 * std::sqrt(av_r) * c->crg[10];
  c->t1_qs_sd = 0.86;
  c->t2_qs_sd = 0.28 * c->sc3 * std::sqrt(av_s);
  c->t1_qs_me = pi * 4.0 * c_sqrd * c->olfus * 0.86;
  c->t2_qs_me = pi * 4.0 * c_sqrd * c->olfus * 0.28 * c->sc3 * std::sqrt(av_s);
  c->t1_qg_sd = 0.86 * c->cgg[0][9];
  c->t1_qg_me = pi * 4.0 * c_cube * c->olfus * 0.86 * c->cgg[0][9];

  TempoBins b;
  make_bins(&b);
  c->nic2 = nint_host(std::log10(b.r_c[0]));
  c->nii2 = nint_host(std::log10(b.r_i[0]));
  c->nir2 = nint_host(std::log10(b.r_r[0]));
  c->nis2 = nint_host(std::log10(b.r_s[0]));
  c->nig2 = nint_host(std::log10(b.r_g[0]));
  c->nii3 = nint_host(std::log10(b.nt_i[0]));
  c->nir3 = nint_host(std::log10(b.n0r_exp[0]));
  c->nig3 = nint_host(std::log10(b.n0g_exp[0]));
  c->niin2 = nint_host(std::log10(b.nt_in[0]));
  c->nic1 = std::log(b.t_nc[nbc - 1] / b.t_nc[0]);
  c->dr1 = b.dr[0];
  c->drn = b.dr[nbr - 1];
  c->ds1 = b.ds[0];
  c->dsn = b.ds[nbs - 1];
  c->t_nc1 = b.t_nc[0];
  c->r_c1 = b.r_c[0];
  c->r_r1 = b.r_r[0];
  c->r_s1 = b.r_s[0];
  c->r_g1 = b.r_g[0];
  c->nt_in1 = b.nt_in[0];
  create_bins(nhbins, 500.e-6, 0.075, c->hbins, c->dhbins);
  const double ta_na[ntb_arc] = {10., 31.6, 100., 316., 1000., 3160., 10000.};
  const double ta_ww[ntb_arw] = {0.01, 0.0316, 0.1, 0.316, 1., 3.16, 10., 31.6, 100.};
  const double ta_tk[ntb_art] = {243.15, 253.15, 263.15, 273.15, 283.15, 293.15, 303.15};
  std::memcpy(c->ta_na, ta_na, sizeof ta_na);
  std::memcpy(c->ta_ww, ta_ww, sizeof ta_ww);
  std::memcpy(c->ta_tk, ta_tk, sizeof ta_tk);
  // Field et al. (2005) snow moment-relation coefficients (params:279-284)
  const double sa[10] = {5.065339, -0.062659, -3.032362, 0.029469, -0.000285,
                         0.31255,  0.000204,  0.003199,  0.,       -0.015952};
  const double sb[10] = {0.476221, -0.015896, 0.165977, 0.007468, -0.000141,
                         0.060366, 0.000079,  0.000594, 0.,       -0.003577};
  std::memcpy(c->sa, sa, sizeof sa);
  std::memcpy(c->sb, sb, sizeof sb);
  c->rain_n0_k = std::pow(c->crg[2] * c->org2 * c->org1, bm_r);
  c->graupel_n0_k = std::pow(c->cgg[0][2] * c->ogg2 * c->ogg1, bm_g);
  c->graupel_lam_k = std::pow(c->cgg[0][2] * c->ogg2 * c->ogg1, c->obmg);
  for (int nu = 1; nu <= 15; nu++)
    c->dc_g_k[nu - 1] = std::pow(c->ccg[nu - 1][2] * c->ocg2[nu - 1], c->obmr);
  const double meanpath = 0.0256e-6, da[2] = {0.04e-6, 0.8e-6};
  for (int i = 0; i < 2; i++)
    c->aer_cc[i] = 1.0 + 2.0 * meanpath / da[i] * (1.257 + 0.4 * std::exp(-(0.55 * da[i] / meanpath)));
  for (int m = kP10Min; m <= kP10Max; m++) c->p10[m - kP10Min] = ipow_binary(10.0, m);
  for (int i = 0; i < ntb_arc; i++) c->ln_ta_na[i] = std::log(c->ta_na[i]);
  for (int i = 0; i < ntb_arw; i++) c->ln_ta_ww[i] = std::log(c->ta_ww[i]);
}

void narrow_consts(const TempoConsts<double>& d, TempoConsts<float>* f) {
  // TempoConsts is a standard-layout aggregate of R-typed scalars/arrays plus the
  // int block; narrow member by member through a flat walk of each section.
  auto nar = [](const double* s, float* o, int n) {
    for (int i = 0; i < n; i++) o[i] = (float)s[i];
  };
#define NAR(m) nar(&d.m, &f->m, 1)
#define NARA(m) nar(&d.m[0], &f->m[0], (int)(sizeof(d.m) / sizeof(double)))
#define NAR2(m) nar(&d.m[0][0], &f->m[0][0], (int)(sizeof(d.m) / sizeof(double)))
  NARA(av_g); NARA(bv_g);
  NAR(am_i); NAR(am_r); NARA(am_g); NAR(olfus); NAR(lfus); NAR(orv); NAR(ar_volume);
  NAR(sc3); NAR(d0i); NAR(xm0s); NAR(xm0g); NAR(obmi); NAR(obmr); NAR(oams); NAR(obms);
  NAR(ocms); NAR(obmg); NARA(oamg); NARA(ocmg); NAR(roverrv); NAR(rho_not); NAR(rho_not0);
  NAR2(cce); NAR2(ccg); NARA(ocg1); NARA(ocg2); NARA(cie); NARA(cig); NAR(oig1); NAR(oig2);
  NARA(cre); NARA(crg); NAR(ore1); NAR(org1); NAR(org2); NAR(org3); NARA(cse); NARA(csg);
  NAR2(cge); NAR2(cgg); NAR(oge1); NAR(ogg1); NAR(ogg2); NAR(ogg3);
  NAR(t1_qr_qc); NAR(t1_qr_qi); NAR(t2_qr_qi); NAR(t1_qs_qc); NAR(t1_qs_qi); NAR(t1_qr_ev);
  NAR(t2_qr_ev); NAR(t1_qs_sd); NAR(t2_qs_sd); NAR(t1_qs_me); NAR(t2_qs_me); NAR(t1_qg_sd);
  NAR(t1_qg_me); NAR(nic1);
  NAR(dr1); NAR(drn); NAR(ds1); NAR(dsn); NAR(t_nc1); NAR(r_c1); NAR(r_r1); NAR(r_s1);
  NAR(r_g1); NAR(nt_in1); NAR(rain_n0_k); NAR(graupel_n0_k); NAR(graupel_lam_k);
  NARA(dc_g_k); NARA(aer_cc); NARA(ln_ta_na); NARA(ln_ta_ww); NARA(hbins); NARA(dhbins); NARA(ta_na); NARA(ta_ww); NARA(ta_tk);
  NARA(sa); NARA(sb);
  // powers of ten in float arithmetic (not narrowed doubles): the mixed form's decade
  // searches divide by exactly what the float powering gives
  for (int m = kP10Min; m <= kP10Max; m++) f->p10[m - kP10Min] = ipow_binary(10.0f, m);
#undef NAR
#undef NARA
#undef NAR2
  f->nic2 = d.nic2; f->nii2 = d.nii2; f->nii3 = d.nii3; f->nir2 = d.nir2; f->nir3 = d.nir3;
  f->nis2 = d.nis2; f->nig2 = d.nig2; f->nig3 = d.nig3; f->niin2 = d.niin2;
  f->dim_nrhg = d.dim_nrhg;
}

// refractive index of water after Ray (1972), Appl. Opt. 11, 1836 (diags:144-173)
static std::complex<double> water_ray(double lambda, double t) {
  const double pi_ = 3.1415926535897932384626434;
  double epsinf = 5.27137 + 0.02164740 * t - 0.00131198 * t * t;
  double epss = 78.54 * (1.0 - 4.579e-3 * (t - 25.0) + 1.190e-5 * (t - 25.0) * (t - 25.0) -
                         2.800e-8 * (t - 25.0) * (t - 25.0) * (t - 25.0));
  double alpha = -16.8129 / (t + 273.16) + 0.0609265;
  double lambdas = 0.00033836 * std::exp(2513.98 / (t + 273.16)) * 1e-2;
  double nenner = 1.0 + 2.0 * std::pow(lambdas / lambda, 1.0 - alpha) * std::sin(alpha * pi_ * 0.5) +
                  std::pow(lambdas / lambda, 2.0 - 2.0 * alpha);
  double epsr = epsinf + ((epss - epsinf) * (std::pow(lambdas / lambda, 1.0 - alpha) *
                                                 std::sin(alpha * pi_ * 0.5) + 1.0)) / nenner;
  double epsi = ((epss - epsinf) * (std::pow(lambdas / lambda, 1.0 - alpha) * std::cos(alpha * pi_ * 0.5) +
                                    0.0)) / nenner + lambda * 1.25664 / 1.88496;
  return std::sqrt(std::complex<double>(epsr, -epsi));
}
// refractive index of ice after Maetzler (1998) (diags:176-203)
static std::complex<double> ice_maetzler(double lambda, double t) {
  double c = 2.99e8, tk = t + 273.16, f = c / lambda * 1e-9;
  double b1 = 0.0207, b2 = 1.16e-11, b = 335.0;
  double deltabeta = std::exp(-10.02 + 0.0364 * (tk - 273.16));
  double e = std::exp(b / tk) - 1.0;
  double betam = (b1 / tk) * (std::exp(b / tk) / (e * e)) + b2 * f * f;
  double beta = betam + deltabeta;
  double theta = 300.0 / tk - 1.0;
  double alfa = (0.00504 + 0.0062 * theta) * std::exp(-22.1 * theta);
  std::complex<double> ri = 3.1884 + 9.1e-4 * (tk - 273.16);
  ri = ri + std::complex<double>(0.0, (alfa / f + beta * f));
  return std::sqrt(std::conj(ri));
}

void make_radar_consts(RadarConsts* r) {
  create_bins(radar_bins, 100.e-6, 0.02, r->sbins, r->dsbins);
  create_bins(radar_bins, 100.e-6, 0.05, r->gbins, r->dgbins);
  const std::complex<double> mw = water_ray(0.10, 0.0), mi = ice_maetzler(0.10, 0.0);
  r->mw_re = mw.real();
  r->mw_im = mw.imag();
  r->mi_re = mi.real();
  r->mi_im = mi.imag();
  const double kw1 = std::abs((mw * mw - 1.0) / (mw * mw + 2.0));
  r->k_w = kw1 * kw1;
}


// ---- bin edges of the log-based table indices ------------------------------------
namespace {
uint64_t dbits(double x) {
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
}
double dval(uint64_t u) {
  double x;
  std::memcpy(&x, &u, 8);
  return x;
}
// least positive double x in [lo, hi] with f(x) >= m, for f non-decreasing, f(lo) < m
// <= f(hi); positive doubles order as their bit patterns
template <class F>
double least_with(F f, int m, double lo, double hi) {
  uint64_t a = dbits(lo), b = dbits(hi);
  while (b - a > 1) {
    const uint64_t mid = a + (b - a) / 2;
    if (f(dval(mid)) >= m)
      b = mid;
    else
      a = mid;
  }
  return dval(b);
}
}  // namespace

void make_index_edges(const TempoBins& b, double* e) {
  const double dr1 = b.dr[0], drn = b.dr[nbr - 1], ds1 = b.ds[0], dsn = b.ds[nbs - 1];
  const double t_nc1 = b.t_nc[0], nic1 = std::log(b.t_nc[nbc - 1] / b.t_nc[0]);
  // the reference's expressions, evaluated as the reference evaluates them
  auto f_r = [&](double x) { return std::min(1 + (int)(nbr * std::log(x / dr1) / std::log(drn / dr1)), nbr); };
  auto f_s = [&](double x) { return std::min(1 + (int)(nbs * std::log(x / ds1) / std::log(dsn / ds1)), nbs); };
  auto f_n = [&](double x) {
    return std::max(1, std::min((int)std::lround(1.0 + (double)nbc * std::log(x / t_nc1) / nic1), nbc));
  };
  const double lo = 1e-30, hi = 1e30;
  e[kEdgesR] = e[kEdgesS] = e[kEdgesN] = 0.0;
  for (int m = 2; m <= nbr; m++) e[kEdgesR + m - 1] = least_with(f_r, m, lo, hi);
  for (int m = 2; m <= nbs; m++) e[kEdgesS + m - 1] = least_with(f_s, m, lo, hi);
  for (int m = 2; m <= nbc; m++) e[kEdgesN + m - 1] = least_with(f_n, m, lo, hi);
}

}  // namespace tg
