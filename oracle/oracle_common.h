/*
 * oracle_common.h -- module-level state of the CPU restatement (test infrastructure).
 * Mirrors module_mp_tempo_params.F90 (constants :39-167, bins :194-288, variables
 * :291-377).  Every real is a double (-fdefault-real-8 semantics of
 * Makefile.gfortran:29); the CCN table is FP32 like table_sp (params:128).
 */
#ifndef ORACLE_COMMON_H
#define ORACLE_COMMON_H
#include <math.h>
#include <stdlib.h>

/* ---- parameters that can be changed (params:27-125) ---- */
#define idx_bg1 6
static const double av_r = 4854.0, bv_r = 1.0, av_s = 40.0, bv_s = 0.55, fv_s = 100.0,
                    bv_c = 2.0, bv_i = 1.0, av_g_old = 442.0, bv_g_old = 0.89,
                    av_g_new = 161.794724, bv_g_new = 0.640961647, fv_r = 195.0,
                    av_c = 0.316946e8, a_coeff = 0.47244157, b_coeff = 0.54698726,
                    av_i = 1493.9, am_s = 0.069, bm_s = 2.0, bm_g = 3.0, bm_i = 3.0,
                    bm_r = 3.0, rho_i = 890.0, xm0i = 1.e-12, d0c = 1.e-6, d0r = 50.e-6,
                    d0s = 300.e-6, d0g = 350.e-6, d0r_max = 2.5e-3, c_cube = 0.5,
                    c_sqrd = 0.15, mu_r = 0.0, mu_s = 0.6357, mu_g = 0.0, mu_i = 0.0,
                    nu_c_scale = 1000.e6, naccn0 = 300.0e6, naccn1 = 50.0e6, nain0 = 1.5e6,
                    nain1 = 0.5e6, nwfa_default = 11.1e6, aero_max = 9999.e6,
                    hgfrz = 235.16, nt_c_o = 50.e6, nt_c_l = 100.e6, nt_c_max = 1999.e6,
                    nt_c_min = 2.0, tno = 5.0, ato = 0.304, demott_nuc_ssati = 0.25,
                    demott_nuc_tempc = -20.0, max_ni = 4999.e3, icenuc_max = 1000.e3,
                    rime_threshold = 2.0, rime_conversion = 0.95, ef_si = 0.05, ef_rs = 0.95,
                    ef_rg = 0.75, ef_ri = 0.95, autocon_nr_factor = 10.0,
                    timestep_conversion_rime_to_rain = 120.0;
#define nifa_default (nain1 * 0.01)
#define nu_c_max 15
#define nu_c_min 2
static const double rho_s = 100.0;

/* ---- parameters that should not be changed (params:128-167) ---- */
#define nrhg 9
#define nrhg1 1
static const double min_qv = 1.e-10, r1 = 1.e-12, r2 = 1.e-6, low_limit_mass_for_precip = 1.e-9,
                    eps = 1.e-15, meters3_to_liters = 1000.0, gonv_min = 1.e2, gonv_max = 1.e6,
                    sc = 0.632, earth_gravity = 9.8;
static const double rho_g[nrhg] = {50., 100., 200., 300., 400., 500., 600., 700., 800.};
static const double pi = 3.1415926536, t0 = 273.15, rho_w = 1000.0, lsub = 2.834e6,
                    lvap0 = 2.5e6, rv = 461.5, rdry = 287.04, cp = 1004.0, r_uni = 8.314;
static const double kap0 = 490.6, kap1 = 17.46, lam0 = 20.78, lam1 = 3.29;

/* ---- table dimensions (params:170-191) ---- */
#define nbins 100
#define nbc nbins
#define nbr nbins
#define nbs nbins
#define nbi nbins
#define nbg nbins
#define ntb_i 64
#define ntb_i1 55
#define ntb_c 37
#define ntb_t 9
#define ntb_g1 37
#define ntb_s 37
#define ntb_g 37
#define ntb_r 37
#define ntb_r1 37
#define ntb_t1 45
#define ntb_in 55
#define ntb_arc 7
#define ntb_arw 9
#define ntb_art 7
#define ntb_arr 5
#define ntb_ark 4
#define nhbins 50

/* ---- table bin data (params:194-288), defined in oracle_init.c ---- */
extern double r_c[ntb_c], r_i[ntb_i], r_r[ntb_r], r_s[ntb_s], r_g[ntb_g], n0r_exp[ntb_r1],
    n0g_exp[ntb_g1], nt_i[ntb_i1], nt_in[ntb_in];
extern const double ta_na[ntb_arc], ta_ww[ntb_arw], ta_tk[ntb_art], sa[10], sb[10],
    tc_tab[ntb_t];

/* ---- module variables set at init (params:291-377) ---- */
extern int dim_nrhg;
extern double av_g[nrhg], bv_g[nrhg];
extern double roverrv, lfus, rho_not, rho_not0;
extern double am_i, am_r, am_g[nrhg], olfus, orv, ar_volume, sc3, d0i, xm0s, xm0g, obmi, obmr,
    oams, obms, ocms, oamg[nrhg], ocmg[nrhg], obmg;
extern double cce[15][5], ccg[15][5], ocg1[15], ocg2[15]; /* [n-1][row-1] = Fortran (row,n) */
extern double cie[7], cig[7], oig1, oig2;
extern double cre[13], crg[13], ore1, org1, org2, org3;
extern double cse[17], csg[17];
extern double cge[nrhg][12], cgg[nrhg][12]; /* [m-1][n-1] = Fortran (n,m) */
extern double oge1, ogg1, ogg2, ogg3;
extern double t1_qr_qc, t1_qr_qi, t2_qr_qi, t1_qs_qc, t1_qs_qi, t1_qr_ev, t2_qr_ev, t1_qs_sd,
    t2_qs_sd, t1_qs_me, t2_qs_me, t1_qg_sd, t1_qg_me;
extern int nic2, nii2, nii3, nir2, nir3, nis2, nig2, nig3, niin2;
extern double nic1;
extern double dc[nbc], dtc[nbc], di[nbi], dti[nbi], dr[nbr], dtr[nbr], ds[nbs], dts[nbs],
    dg[nbg], dtg[nbg], t_nc[nbc];
extern double hbins[nhbins], dhbins[nhbins];
/* radar bins of melting snow and graupel (initialize_bins_for_radar, params:674-692) */
#define radar_bins 50
extern double sbins_radar[radar_bins], dsbins_radar[radar_bins], gbins_radar[radar_bins],
    dgbins_radar[radar_bins];

/* Fortran-order tables (column-major, 1-based accessors below) */
extern double *t_efrw, *t_efsw;             /* (nbr|nbs, nbc) */
extern double *tpc_wev, *tnc_wev;           /* (nbc, ntb_c, nbc) */
extern float *tnccn_act;                    /* (7,9,7,5,4) */
extern double *tcg_racg, *tmr_racg, *tcr_gacr, *tnr_racg, *tnr_gacr; /* (37,37,9,37,37) */
extern double *tcs_racs1, *tmr_racs1, *tcs_racs2, *tmr_racs2, *tcr_sacr1, *tms_sacr1,
    *tcr_sacr2, *tms_sacr2, *tnr_racs1, *tnr_racs2, *tnr_sacr1, *tnr_sacr2; /* (37,9,37,37) */
extern double *tpi_qcfz, *tni_qcfz;         /* (37,100,45,55) */
extern double *tpi_qrfz, *tpg_qrfz, *tni_qrfz, *tnr_qrfz; /* (37,37,45,55) */
extern double *tps_iaus, *tni_iaus, *tpi_ide; /* (64,55) */

/* 1-based Fortran accessors */
#define CCE(r, n) cce[(n)-1][(r)-1]
#define CCG(r, n) ccg[(n)-1][(r)-1]
#define OCG1(n) ocg1[(n)-1]
#define OCG2(n) ocg2[(n)-1]
#define CIE(n) cie[(n)-1]
#define CIG(n) cig[(n)-1]
#define CRE(n) cre[(n)-1]
#define CRG(n) crg[(n)-1]
#define CSE(n) cse[(n)-1]
#define CSG(n) csg[(n)-1]
#define CGE(n, m) cge[(m)-1][(n)-1]
#define CGG(n, m) cgg[(m)-1][(n)-1]
#define AM_G(m) am_g[(m)-1]
#define AV_G(m) av_g[(m)-1]
#define BV_G(m) bv_g[(m)-1]
#define RHO_G(m) rho_g[(m)-1]
#define OCMG(m) ocmg[(m)-1]

#define T_EFRW(i, j) t_efrw[((i)-1) + (long)((j)-1) * nbr]
#define T_EFSW(i, j) t_efsw[((i)-1) + (long)((j)-1) * nbs]
#define TNC_WEV(i, j, k) tnc_wev[((i)-1) + (long)((j)-1) * nbc + (long)((k)-1) * nbc * ntb_c]
#define TPC_WEV(i, j, k) tpc_wev[((i)-1) + (long)((j)-1) * nbc + (long)((k)-1) * nbc * ntb_c]
#define TNCCN(i, j, k, l, m)                                                              \
  tnccn_act[((i)-1) + (long)((j)-1) * ntb_arc + (long)((k)-1) * ntb_arc * ntb_arw +     \
            (long)((l)-1) * ntb_arc * ntb_arw * ntb_art +                                 \
            (long)((m)-1) * ntb_arc * ntb_arw * ntb_art * ntb_arr]
#define QG5(a, i, j, n3, k, m)                                                            \
  a[((i)-1) + (long)((j)-1) * ntb_g1 + (long)((n3)-1) * ntb_g1 * ntb_g +                \
    (long)((k)-1) * ntb_g1 * ntb_g * nrhg + (long)((m)-1) * ntb_g1 * ntb_g * nrhg * ntb_r1]
#define QS4(a, i, j, k, m)                                                                \
  a[((i)-1) + (long)((j)-1) * ntb_s + (long)((k)-1) * ntb_s * ntb_t +                   \
    (long)((m)-1) * ntb_s * ntb_t * ntb_r1]
#define QCFZ(a, i, j, k, m)                                                               \
  a[((i)-1) + (long)((j)-1) * ntb_c + (long)((k)-1) * ntb_c * nbc +                     \
    (long)((m)-1) * ntb_c * nbc * ntb_t1]
#define QRFZ(a, i, j, k, m)                                                               \
  a[((i)-1) + (long)((j)-1) * ntb_r + (long)((k)-1) * ntb_r * ntb_r1 +                  \
    (long)((m)-1) * ntb_r * ntb_r1 * ntb_t1]
#define IAUS(a, i, j) a[((i)-1) + (long)((j)-1) * ntb_i]

#define QG_COUNT ((long)ntb_g1 * ntb_g * nrhg * ntb_r1 * ntb_r)
#define QS_COUNT ((long)ntb_s * ntb_t * ntb_r1 * ntb_r)
#define QCFZ_COUNT ((long)ntb_c * nbc * ntb_t1 * ntb_in)
#define QRFZ_COUNT ((long)ntb_r * ntb_r1 * ntb_t1 * ntb_in)
#define CCN_COUNT ((long)ntb_arc * ntb_arw * ntb_art * ntb_arr * ntb_ark)

/* ---- Fortran intrinsic semantics ---- */
/* real ** integer: binary powering, reciprocal for negative exponents (the libgcc
 * __powidf2 algorithm that gfortran emits for variable integer exponents). */
static inline double ipow(double x, int m) {
  unsigned int n = m < 0 ? -(unsigned int)m : (unsigned int)m;
  double y = (n % 2) ? x : 1.0;
  while (n >>= 1) {
    x = x * x;
    if (n % 2) y = y * x;
  }
  return m < 0 ? 1.0 / y : y;
}
/* nint: round half away from zero */
static inline int nint(double x) { return (int)lround(x); }
static inline double fmax2(double a, double b) { return a > b ? a : b; }
static inline double fmin2(double a, double b) { return a < b ? a : b; }
static inline double fmax3(double a, double b, double c) { return fmax2(fmax2(a, b), c); }
static inline double fmin3(double a, double b, double c) { return fmin2(fmin2(a, b), c); }
static inline int imax(int a, int b) { return a > b ? a : b; }
static inline int imin(int a, int b) { return a < b ? a : b; }

/* utils.F90 */
double o_calc_gamma_p(double a, double x);
void o_snow_moments(double rs, double tc, double *smob, double *smoc, double *ns, double *smo0,
                    double *smo1, double *smo2, double *smoe, double *smof, double *smog,
                    double *smoz);
double o_calc_rslf(double p, double t);
double o_calc_rsif(double p, double t);
int o_get_nuc(double nc);
void o_initialize_graupel_vars(int hail_flag);
void o_initialize_parameters(void);

#endif
