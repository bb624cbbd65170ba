// tempo_consts.h -- parameters of the TEMPO scheme shared by host init code and the
// sm_103a kernels.  Fixed parameters are the `parameter` constants of
// src/module_mp_tempo_params.F90:27-191; TempoConsts holds the values that
// tempo_init derives at run time (params:411-658) and is copied to __constant__
// memory once per context.
#pragma once

#ifdef __CUDACC__
#define TG_HD __host__ __device__
#else
#define TG_HD
#endif

namespace tg {

// ---- fixed parameters (params:39-167) ----
constexpr double av_r = 4854.0, bv_r = 1.0, av_s = 40.0, bv_s = 0.55, fv_s = 100.0;
constexpr double bv_c = 2.0, bv_i = 1.0, av_g_old = 442.0, bv_g_old = 0.89;
constexpr double av_g_new = 161.794724, bv_g_new = 0.640961647, fv_r = 195.0;
constexpr double av_c = 0.316946e8, a_coeff = 0.47244157, b_coeff = 0.54698726;
constexpr double av_i = 1493.9, am_s = 0.069, bm_s = 2.0, bm_g = 3.0, bm_i = 3.0, bm_r = 3.0;
constexpr double rho_i = 890.0, xm0i = 1.e-12, d0c = 1.e-6, d0r = 50.e-6, d0s = 300.e-6;
constexpr double d0g = 350.e-6, d0r_max = 2.5e-3, c_cube = 0.5, c_sqrd = 0.15;
constexpr double mu_r = 0.0, mu_s = 0.6357, mu_g = 0.0, mu_i = 0.0, nu_c_scale = 1000.e6;
constexpr double naccn0 = 300.0e6, naccn1 = 50.0e6, nain0 = 1.5e6, nain1 = 0.5e6;
constexpr double nwfa_default = 11.1e6, nifa_default = nain1 * 0.01, aero_max = 9999.e6;
constexpr double hgfrz = 235.16, nt_c_o = 50.e6, nt_c_l = 100.e6, nt_c_max = 1999.e6;
constexpr double nt_c_min = 2.0, tno = 5.0, ato = 0.304, rho_s = 100.0;
constexpr double demott_nuc_ssati = 0.25, demott_nuc_tempc = -20.0, max_ni = 4999.e3;
constexpr double icenuc_max = 1000.e3, rime_threshold = 2.0, rime_conversion = 0.95;
constexpr double ef_si = 0.05, ef_rs = 0.95, ef_rg = 0.75, ef_ri = 0.95;
constexpr double autocon_nr_factor = 10.0, timestep_conversion_rime_to_rain = 120.0;
constexpr double min_qv = 1.e-10, r1 = 1.e-12, r2 = 1.e-6, low_limit_mass_for_precip = 1.e-9;
constexpr double eps = 1.e-15, meters3_to_liters = 1000.0, gonv_min = 1.e2, gonv_max = 1.e6;
constexpr double sc = 0.632, earth_gravity = 9.8;
constexpr double pi = 3.1415926536, t0 = 273.15, rho_w = 1000.0, lsub = 2.834e6;
constexpr double lvap0 = 2.5e6, rv = 461.5, rdry = 287.04, cp = 1004.0, r_uni = 8.314;
constexpr double kap0 = 490.6, kap1 = 17.46, lam0 = 20.78, lam1 = 3.29;
constexpr int idx_bg1 = 6, nrhg = 9, nu_c_max = 15, nu_c_min = 2;

// ---- table dimensions (params:170-191) ----
constexpr int nbins = 100, nbc = 100, nbr = 100, nbs = 100, nbi = 100, nbg = 100;
constexpr int ntb_i = 64, ntb_i1 = 55, ntb_c = 37, ntb_t = 9, ntb_g1 = 37, ntb_s = 37;
constexpr int ntb_g = 37, ntb_r = 37, ntb_r1 = 37, ntb_t1 = 45, ntb_in = 55;
constexpr int ntb_arc = 7, ntb_arw = 9, ntb_art = 7, ntb_arr = 5, ntb_ark = 4, nhbins = 50;

constexpr long QG_COUNT = (long)ntb_g1 * ntb_g * nrhg * ntb_r1 * ntb_r;  // per array
constexpr long QS_COUNT = (long)ntb_s * ntb_t * ntb_r1 * ntb_r;
constexpr long QCFZ_COUNT = (long)ntb_c * nbc * ntb_t1 * ntb_in;
constexpr long QRFZ_COUNT = (long)ntb_r * ntb_r1 * ntb_t1 * ntb_in;
constexpr long CCN_COUNT = (long)ntb_arc * ntb_arw * ntb_art * ntb_arr * ntb_ark;

// real ** integer as the reference's compiled code evaluates it (binary powering, a
// reciprocal for negative exponents); host and device share it
template <class T>
TG_HD inline T ipow_binary(T x, int m) {
  unsigned n = m < 0 ? -(unsigned)m : (unsigned)m;
  T y = (n % 2) ? x : T(1);
  while (n >>= 1) {
    x = x * x;
    if (n % 2) y = y * x;
  }
  return m < 0 ? T(1) / y : y;
}
// 10**m for the decade searches of the table indices, every m a finite positive float's
// decade can take; other m fall back to the powering
constexpr int kP10Min = -46, kP10Max = 39, kP10Count = kP10Max - kP10Min + 1;

// ---- run-time derived values (params:411-658, utils) ----
template <class R>
struct TempoConsts {
  R av_g[nrhg], bv_g[nrhg];
  R am_i, am_r, am_g[nrhg], olfus, lfus, orv, ar_volume, sc3, d0i, xm0s, xm0g;
  R obmi, obmr, oams, obms, ocms, obmg, oamg[nrhg], ocmg[nrhg];
  R roverrv, rho_not, rho_not0;
  R cce[15][5], ccg[15][5], ocg1[15], ocg2[15];  // [n-1][row-1] <-> Fortran (row, n)
  R cie[7], cig[7], oig1, oig2;
  R cre[13], crg[13], ore1, org1, org2, org3;
  R cse[17], csg[17];
  R cge[nrhg][12], cgg[nrhg][12];  // [m-1][n-1] <-> Fortran (n, m)
  R oge1, ogg1, ogg2, ogg3;
  R t1_qr_qc, t1_qr_qi, t2_qr_qi, t1_qs_qc, t1_qs_qi, t1_qr_ev, t2_qr_ev, t1_qs_sd;
  R t2_qs_sd, t1_qs_me, t2_qs_me, t1_qg_sd, t1_qg_me;
  R nic1;
  int nic2, nii2, nii3, nir2, nir3, nis2, nig2, nig3, niin2, dim_nrhg;
  // bin values used by the step (first/last bins, log ratios)
  R dr1, drn, ds1, dsn, t_nc1;
  R r_c1, r_r1, r_s1, r_g1, nt_in1;
  R hbins[nhbins], dhbins[nhbins];
  R ta_na[ntb_arc], ta_ww[ntb_arw], ta_tk[ntb_art];
  R sa[10], sb[10];
  // powers of constants that the reference evaluates at every use, computed once here
  // with the same expression (host libm): (crg(3) org2 org1)**bm_r (main:2546),
  // (cgg(3,1) ogg2 ogg1)**bm_g (main:2579) and **obmg (main:1207),
  // (ccg(3,nu) ocg2(nu))**obmr (main:2318), and the Cunningham slip correction of the
  // two aerosol diameters (aerosols:106; 0 = 0.04 um, 1 = 0.8 um)
  R rain_n0_k, graupel_n0_k, graupel_lam_k, dc_g_k[15], aer_cc[2];
  // ipow_binary(R(10), m) in R's own arithmetic, m = kP10Min..kP10Max
  R p10[kP10Count];
  // logarithms of the CCN activation table's aerosol-number and vertical-velocity
  // grid values (main:2222-2223, 2236-2237)
  R ln_ta_na[ntb_arc], ln_ta_ww[ntb_arw];
};

// Fills a double-precision constant set exactly as tempo_init does for the given
// hail-aware flag (graupel vars, initialize_parameters, bins).  Host only.
void make_consts(TempoConsts<double>* c, bool hailaware);
// Melting-layer 10-cm reflectivity (diags:124-395), always evaluated in FP64: the
// radar bins of snow and graupel (initialize_bins_for_radar, params:674-692) and the
// refractive indices of water and ice at 0 C for a 10-cm wavelength with the
// dielectric factor |K_w|^2 (complex_water_ray, complex_ice_maetzler).  Host only.
constexpr int radar_bins = 50;
struct RadarConsts {
  double sbins[radar_bins], dsbins[radar_bins], gbins[radar_bins], dgbins[radar_bins];
  double mw_re, mw_im, mi_re, mi_im, k_w;
};
void make_radar_consts(RadarConsts* r);

// Narrows every member to float for the mixed-precision kernels.
void narrow_consts(const TempoConsts<double>& d, TempoConsts<float>* f);

// Constants of the thermodynamic island, in the island type (double, or the
// double-float pair of the mixed form split once on the host).
template <class I>
struct IslandConsts {
  I rho_not, orv, roverrv, lfus;
};
template <class I>
inline void make_island_consts(const TempoConsts<double>& d, IslandConsts<I>* o) {
  o->rho_not = I(d.rho_not);
  o->orv = I(d.orv);
  o->roverrv = I(d.roverrv);
  o->lfus = I(d.lfus);
}

// Bin arrays needed by the table builders (host copies; params:613-722).
struct TempoBins {
  double dc[nbc], dtc[nbc], di[nbi], dti[nbi], dr[nbr], dtr[nbr], ds[nbs], dts[nbs];
  double dg[nbg], dtg[nbg], t_nc[nbc];
  double r_c[ntb_c], r_i[ntb_i], r_r[ntb_r], r_s[ntb_s], r_g[ntb_g];
  double n0r_exp[ntb_r1], n0g_exp[ntb_g1], nt_i[ntb_i1], nt_in[ntb_in], tc[ntb_t];
};
void make_bins(TempoBins* b);

// Least values of the bins of the three table indices that the reference computes
// with libm's log of a state value (main:2341, 2391, 2607): the rain-cloud
// efficiency bin of mvd_r (nbr bins), the snow-cloud efficiency bin of the snow
// diameter (nbs) and the droplet-number bin of nc (nbc).  edges[off + m - 1] is the
// least double x whose index is >= m (edges[off] = 0), found on the host by bisection
// over doubles with the host's libm, so that the device takes the bin the host
// arithmetic gives for the same value.
constexpr int kEdgesR = 0, kEdgesS = nbr, kEdgesN = nbr + nbs, kEdgesCount = nbr + nbs + nbc;
void make_index_edges(const TempoBins& b, double* edges);

}  // namespace tg
