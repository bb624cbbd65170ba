/*
 * tempo_oracle.h -- CPU FP64 restatement of NCAR/TEMPO v3.1.1 (test infrastructure).
 *
 * This is the oracle, not the product.  Only tests/, __graft_entry__.smoke() and
 * bench.py's cpu_baseline / --impl reference legs may load it.  It restates, in
 * plain C with Fortran semantics (-fdefault-real-8: every real is a double, every
 * unsuffixed literal is a double; nint rounds half away from zero; real**integer is
 * integer power; real**real is libm pow), the reference routines:
 *
 *   src/module_mp_tempo_params.F90  : constants :39-167, bins :194-288,
 *                                     initialize_graupel_vars :411-426,
 *                                     initialize_parameters :429-610,
 *                                     initialize_bins_for_tables :613-658,
 *                                     initialize_bins_for_hail_size :661-671,
 *                                     create_bins :695-722
 *   src/module_mp_tempo_utils.F90   : calc_gamma_p :27-145, snow_moments :148-282,
 *                                     calc_rslf/rsif :285-331, get_nuc :334-346,
 *                                     compute_efrw :349-400, compute_efsw :403-440,
 *                                     qi_aut_qs :443-490, compute_drop_evap :493-527
 *   src/module_mp_tempo_aerosols.F90: all (:14-118)
 *   src/module_mp_tempo_diags.F90   : effective_radius :13-56, reflectivity_10cm :59-121
 *                                     (without melting), max_hail_diam :398-438,
 *                                     freezing_rain :441-456
 *   src/module_mp_tempo_main.F90    : tempo_main :73-864 and every routine it calls,
 *                                     semilagrangian_sedimentation :1562-1749 included;
 *                                     the ML path excepted
 *   src/module_mp_tempo_driver.F90  : tempo_run :187-513, read_table_* :532-649
 *   src/module_mp_tempo_tables.F90  : qr_acr_qs :493-621, qr_acr_qg :624-714,
 *                                     freezewater :717-805, write_table_* :96-444
 *
 * Parity pins: the reference's own known-answer unit tests
 * (test/unittests/test_tempo_{init,utils,main}_suite.F90) are checked against this
 * restatement in tests/test_oracle_pins.py.  Full-step outputs have no reference
 * golden values (the reference's integration tests assert nothing and no Fortran
 * compiler is available here), so step parity rests on this restatement.
 */
#ifndef TEMPO_ORACLE_H
#define TEMPO_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* module_mp_tempo_cfgs.F90:14-35 (ty_tempo_cfgs); logicals as int 0/1 */
typedef struct {
  int aerosolaware_flag;
  int hailaware_flag;
  int ml_for_bl_nc_flag;
  int ml_for_nc_flag;
  int semi_sedi_flag;
  int refl10cm_from_melting_flag;
  int turn_off_micro_flag;
  int cloud_condensation_flag;
  int verbose;
  int check_tables;
  char single_moment_nc_opt[32];
  int refl10cm_flag;
  int re_cloud_flag;
  int re_ice_flag;
  int re_snow_flag;
  int max_hail_diameter_flag;
  int rain_med_vol_diam_flag;
  int graupel_med_vol_diam_flag;
  int cloud_number_mixing_ratio_flag;
} ocfg_t;

/* module_mp_tempo_driver.F90:18-34 (ty_tempo_driver_diags).  Tile-shaped arrays,
 * i fastest: 2-D (its:ite, jts:jte), 3-D (its:ite, kts:kte, jts:jte).  NULL = not
 * requested.  The caller owns them. */
typedef struct {
  double *rain_precip, *ice_liquid_equiv_precip, *snow_liquid_equiv_precip,
      *graupel_liquid_equiv_precip, *frozen_fraction, *frz_rain_precip,
      *max_hail_diameter_sfc, *max_hail_diameter_column;
  double *refl10cm, *re_cloud, *re_ice, *re_snow, *rain_med_vol_diam,
      *graupel_med_vol_diam, *cloud_number_mixing_ratio;
} odiag_t;

void oracle_default_cfgs(ocfg_t *cfg);

/* tempo_init without the table reads: graupel vars, parameters, bins, small tables.
 * Returns 0 on success. */
int oracle_init(int hailaware_flag);

/* read_table_ccn (driver:625-649): Fortran sequential unformatted big-endian FP32. */
int oracle_read_ccn(const char *path);
/* read_table_{freezewater,qr_acr_qs,qr_acr_qg}: stream, big-endian FP64. */
int oracle_read_freezewater(const char *path);
int oracle_read_qr_acr_qs(const char *path);
int oracle_read_qr_acr_qg(const char *path);
int oracle_write_freezewater(const char *path);
int oracle_write_qr_acr_qs(const char *path);
int oracle_write_qr_acr_qg(const char *path);

/* Table builders (tables.F90:493-805).  They always use hail-aware graupel
 * parameters, like tempo_build_tables (tables.F90:31,50); the caller's hail flag is
 * restored afterwards.  `naive`=1 keeps the reference's loop and summation order
 * (slow); 0 evaluates the same non-negative double sums as factored bilinear forms
 * (orders of magnitude faster, identical to ~1e-15 relative).  nthreads<=0: all. */
int oracle_build_freezewater(int nthreads);
int oracle_build_qr_acr_qs(int naive, int nthreads);
int oracle_build_qr_acr_qg(int naive, int nthreads);
/* One entry of qr_acr_qg / qr_acr_qs in the reference's exact loop order (1-based
 * Fortran indices); out receives the stored outputs in table order. */
void oracle_qr_acr_qg_entry(int i, int j, int n3, int k, int m, double out[5]);
void oracle_qr_acr_qs_entry(int i, int j, int k, int m, double out[12]);

/* Access to the module tables (for export to the GPU product and for tests). */
double *oracle_table_ptr(const char *name, long *count);
float *oracle_ccn_ptr(long *count);
/* Scalar module values by name (e.g. "ccg", "dc", "dim_nrhg", "am_g"); idx is 0-based
 * into the flattened Fortran-order array.  Returns NaN for unknown names. */
double oracle_param(const char *name, int idx);

/* Unit-test exports (test_tempo_main_suite.F90 / test_tempo_utils_suite.F90). */
double oracle_calc_gamma_p(double a, double x);
void oracle_get_cloud_table_index(double rc, double nc, int *idx_c, int *idx_n);
void oracle_get_snow_table_index(double rs, int *idx_s);
void oracle_get_temperature_table_index(double tempk, int *idx_t);
void oracle_get_rain_table_index(double rr, double ilamr, int *idx_r, int *idx_r1);
void oracle_get_graupel_table_index(double rg, double ilamg, int idx, int *idx_g, int *idx_g1);
void oracle_get_ice_table_index(double ri, double ni, int *idx_i, int *idx_i1);
double oracle_calc_rslf(double p, double t);
double oracle_calc_rsif(double p, double t);
void oracle_snow_moments(double rs, double tc, double out[10]);

/* Weights of the cloud-number network of the ML path (ml:33-98 layout: scaler means
 * and variances [7], weights00 [24 x 7 column-major], bias00 [24], weights01 [24],
 * bias01 [1]). */
int oracle_set_ml(const double *mean, const double *var, const double *w00, const double *b00,
                  const double *w01, const double *b01);

/* tempo_run (driver:187-513).  Arrays are (ims:ime, kms:kme, jms:jme), i fastest.
 * NULL means "optional argument not present".  bounds = ids,ide,jds,jde,kds,kde,
 * ims,ime,jms,jme,kms,kme,its,ite,jts,jte,kts,kte.  Columns run in parallel on
 * `nthreads` OpenMP threads (<=0: all).  Returns 0, or a negative code for
 * unsupported optional paths (ML, melting radar). */
int oracle_run(const ocfg_t *cfg, double dt, int itimestep,
               double *t, double *th, const double *pii, const double *p, const double *w,
               const double *dz, double *qv, double *qc, double *qr, double *qi, double *qs,
               double *qg, double *ni, double *nr, double *nc, double *nwfa, double *nifa,
               double *ng, double *qb, const double *qc_bl, const double *qcfrac_bl,
               const int *land_input, const int bounds[18], odiag_t *diags, int nthreads);

/* Per-call counters of the last oracle_run: [0] columns, [1] early-exit columns,
 * [2..6] max substeps rain/graupel/snow/ice/cloud(=1). */
void oracle_last_stats(long out[8]);

/* Oracle-only instrumentation: when flags != NULL, oracle_run writes per tile column
 * (2-D diagnostic layout) the bits of the index computations that the column's step
 * passed within one rounding of their discontinuity (nint at a half-integer, int at
 * an integer): 1 = before or in sedimentation (graupel density class, substep
 * count: can move every later field of the column), 2 = graupel density class in
 * the final check (moves only that level's graupel diagnostics).  NULL turns it off. */
void oracle_set_tie_sink(int *flags);

#ifdef __cplusplus
}
#endif
#endif
