/*
 * tempo_gb300.h -- C ABI of the GB300 (sm_103a) TEMPO column-microphysics step.
 *
 * This is the drop-in boundary for the host model's column loop.  Each entry point
 * replaces one routine of the Fortran reference (NCAR/TEMPO v3.1.1) and keeps its
 * argument list and argument meaning; a Fortran host binds it with ISO_C_BINDING
 * (optional arguments map to NULL pointers, logical flags to int 0/1).
 *
 * Conventions
 *   - Every entry point returns an int status: TEMPO_OK (0) or a negative
 *     tempo_status_t code.  Nothing aborts the process (the reference `error stop`s).
 *   - tempo_last_error() returns a thread-local message for the last failure.
 *   - A context owns its device tables and buffers; calls on one context are not
 *     thread-safe, distinct contexts are independent (one context per host thread or
 *     per CUDA stream).
 *   - 3-D arrays are (ims:ime, kms:kme, jms:jme) with i fastest, exactly as in
 *     tempo_run; the step updates them in place on the tile its:ite, kts:kte,
 *     jts:jte.  Diagnostic arrays are tile-shaped (its:ite, [kts:kte,] jts:jte).
 */
#ifndef TEMPO_GB300_H
#define TEMPO_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  TEMPO_OK = 0,
  TEMPO_ERR_ARG = -1,         /* NULL required pointer, bad bounds, dt <= 0, ... */
  TEMPO_ERR_UNSUPPORTED = -2, /* optional path this library does not implement (the ML
                                 boundary-layer cloud path; derivatives of the
                                 semi-Lagrangian, melting-layer and ML cloud-number paths) */
  TEMPO_ERR_TABLE = -3,       /* missing, truncated or malformed lookup table */
  TEMPO_ERR_CUDA = -4,        /* CUDA runtime failure (message has the CUDA error string) */
  TEMPO_ERR_NOMEM = -5,       /* host or device allocation failed */
  TEMPO_ERR_STATE = -6,       /* context not initialised / wrong precision for the call /
                                 the calling thread's current device is not the context's */
  /* -7 is not used (no entry point waits on the device with a time limit) */
  TEMPO_ERR_NONFINITE = -8    /* non-finite or non-physical input found by the validation
                                 pass (tempo_set_validation); the state is left untouched */
} tempo_status_t;

/* ty_tempo_cfgs (src/module_mp_tempo_cfgs.F90:14-35); same field order and defaults
 * as tempo_default_cfgs() returns.  Logicals are int 0/1. */
typedef struct {
  int aerosolaware_flag;          /* .true.  */
  int hailaware_flag;             /* .true.  */
  int ml_for_bl_nc_flag;          /* .false. */
  int ml_for_nc_flag;             /* .false. */
  int semi_sedi_flag;             /* .false. */
  int refl10cm_from_melting_flag; /* .false. */
  int turn_off_micro_flag;        /* .false. */
  int cloud_condensation_flag;    /* .true.  */
  int verbose;                    /* .false. */
  int check_tables;               /* .false. */
  char single_moment_nc_opt[32];  /* 'land' | 'ocean' | number in m^-3 */
  int refl10cm_flag;              /* .true.  */
  int re_cloud_flag;              /* .true.  */
  int re_ice_flag;                /* .true.  */
  int re_snow_flag;               /* .true.  */
  int max_hail_diameter_flag;     /* .true.  */
  int rain_med_vol_diam_flag;     /* .false. */
  int graupel_med_vol_diam_flag;  /* .false. */
  int cloud_number_mixing_ratio_flag; /* .false. */
} tempo_cfgs_t;

/* ty_tempo_driver_diags (src/module_mp_tempo_driver.F90:18-34).  Caller-owned,
 * tile-shaped; NULL = not requested.  The element type follows the run call
 * (double for *_c / *_dev_c, float for *_f32 variants); host pointers for the
 * host-memory calls, device pointers for the *_dev_* calls. */
typedef struct {
  void *rain_precip, *ice_liquid_equiv_precip, *snow_liquid_equiv_precip,
      *graupel_liquid_equiv_precip, *frozen_fraction, *frz_rain_precip,
      *max_hail_diameter_sfc, *max_hail_diameter_column;           /* 2-D */
  void *refl10cm, *re_cloud, *re_ice, *re_snow, *rain_med_vol_diam,
      *graupel_med_vol_diam, *cloud_number_mixing_ratio;           /* 3-D */
} tempo_diags_t;

/* Arithmetic of the step kernels. */
typedef enum {
  TEMPO_PREC_FP64 = 0,  /* plain FP64 drop-in: every real is a double, no FMA contraction */
  TEMPO_PREC_MIXED = 1  /* FP32 bulk; temperature/vapour state, saturation differences,
                           sedimentation flux divergence and precipitation sums in FP64 */
} tempo_precision_t;

typedef struct tempo_ctx tempo_ctx_t;

/* Device pointers to one state of the column step, in the layout of tempo_run's
 * arrays; the element type is given by the call (double or float).  NULL = absent
 * (the optional arguments of tempo_run). */
typedef struct {
  void *t, *th;
  const void *pii, *p, *w, *dz;
  void *qv, *qc, *qr, *qi, *qs, *qg, *ni, *nr, *nc, *nwfa, *nifa, *ng, *qb;
  const int *land_input;
} tempo_state_t;

/* Library identification; never fails. */
const char *tempo_version(void);
/* Thread-local message of the last failing call ("" if none). */
const char *tempo_last_error(void);
/* Reference defaults of ty_tempo_cfgs (cfgs:15-34). */
int tempo_default_cfgs(tempo_cfgs_t *cfgs);

/* tempo_init (src/module_mp_tempo_driver.F90:42-182).  The eight flag arguments are
 * the reference's optional logicals (NULL = not present); present ones are written
 * into *tempo_cfgs.  table_dir holds ccn_activate.bin and, unless build_tables is
 * nonzero, the three big-endian stream tables (qr_acr_qg_data_tempo_v3,
 * qr_acr_qs_data_tempo_v3, freeze_water_data_tempo_v3).  build_tables != 0 builds
 * the three tables on the GPU in FP64 instead of reading them (the reference builds
 * them offline with tools/build_tables.F90).  device: CUDA ordinal, or -1 for the
 * calling thread's current device.  On success *ctx receives a new context.  Table
 * files are checked as tempo_check_table_c does (existence, size, record markers,
 * value range) and a bad file gives TEMPO_ERR_TABLE with the file's name. */
int tempo_init_c(const int *aerosolaware_flag, const int *hailaware_flag,
                 const int *semi_sedi_flag, const int *cloud_condensation_flag,
                 const int *refl10cm_from_melting_flag, const int *ml_for_bl_nc_flag,
                 const int *ml_for_nc_flag, const int *force_init_flag,
                 tempo_cfgs_t *tempo_cfgs, const char *table_dir, int build_tables,
                 int device, tempo_ctx_t **ctx);

/* Releases the context and its device memory. NULL is a no-op. */
int tempo_ctx_destroy(tempo_ctx_t *ctx);

/* Selects the kernel arithmetic for later run calls (default TEMPO_PREC_FP64). */
int tempo_set_precision(tempo_ctx_t *ctx, int precision);

/* check_before_table_read (src/module_mp_tempo_driver.F90:652-700) for one table file,
 * on the host only (no device, no context): name is "ccn_activate" (Fortran sequential
 * record of 8820 big-endian FP32 activated fractions, driver:625-649), "qr_acr_qg",
 * "qr_acr_qs" or "freezewater" (big-endian FP64 stream files, driver:532-622).  Beyond
 * the reference's existence and size checks it decodes the file: record markers, every
 * value finite, collection and freezing values >= 0 and below 1e30 (a file written in
 * the other byte order fails here), activated fractions in [0, 1].  TEMPO_OK or
 * TEMPO_ERR_TABLE with the reason in tempo_last_error(); TEMPO_ERR_ARG for an unknown
 * name. */
int tempo_check_table_c(const char *name, const char *path);

/* No reference counterpart (the reference trusts its inputs).  With on != 0, every later
 * run first scans the tile's inputs: temperature (t, or th and pii), p, dz, qv and every
 * present mass, number, aerosol and volume array must be finite; t (or th and pii), p and
 * dz must be > 0.  A failed scan returns TEMPO_ERR_NONFINITE naming the first bad field
 * and (i, k, j) index, before any array is modified.  Host-array runs scan on the host
 * before the copy; device-array runs scan with one kernel and wait for its result (the
 * call then synchronises with its stream).  Off by default. */
int tempo_set_validation(tempo_ctx_t *ctx, int on);

/* tempo_run (src/module_mp_tempo_driver.F90:187-513) on host arrays of doubles (the
 * reference's default kind_phys).  Copies the tile to the device, runs the step,
 * copies results back and synchronises.  Large tiles (from 2^18 columns) go in up to
 * 8 slabs of rows j, each slab's copies on two copy streams overlapping the other
 * slabs' steps on the context's stream; only the tile's rows are copied.  Optional
 * arrays: t or (th and pii); nc, nwfa, nifa, ng, qb, land_input, qcfrac, qifrac and
 * the *_bl / thten_* inputs (qcfrac, qifrac, qvten_bl, qcten_bl, qiten_bl, thten_*
 * are accepted and, as in the reference, unused).  qc_bl with qcfrac_bl adds the
 * boundary-layer cloud to re_cloud (main:832-857) and needs the cloud-number network
 * (tempo_set_ml_cloud_number_c; TEMPO_ERR_STATE without it). */
int tempo_run_c(tempo_ctx_t *ctx, const tempo_cfgs_t *tempo_cfgs, double dt, int itimestep,
                double *t, double *th, const double *pii, const double *p, const double *w,
                const double *dz, double *qv, double *qc, double *qr, double *qi, double *qs,
                double *qg, double *ni, double *nr, double *nc, double *nwfa, double *nifa,
                double *ng, double *qb, const double *qc_bl, const double *qcfrac_bl,
                double *qcfrac, double *qifrac, const double *thten_bl, const double *qvten_bl,
                const double *qcten_bl, const double *qiten_bl, const double *thten_lwrad,
                const double *thten_swrad, const int *land_input, int ids, int ide, int jds,
                int jde, int kds, int kde, int ims, int ime, int jms, int jme, int kms, int kme,
                int its, int ite, int jts, int jte, int kts, int kte, tempo_diags_t *tempo_diags);

/* tempo_run (src/module_mp_tempo_driver.F90:187-513) on host arrays of floats: the
 * reference built with -DSINGLE_PREC (src/machine.F90:13-17), whose tempo_run keeps the
 * same argument list with real(wp) = real(4).  Same arguments, order and meaning as
 * tempo_run_c; the step runs in the context's precision (TEMPO_PREC_MIXED for FP32
 * storage). */
int tempo_run_f32_c(tempo_ctx_t *ctx, const tempo_cfgs_t *tempo_cfgs, float dt, int itimestep,
                    float *t, float *th, const float *pii, const float *p, const float *w,
                    const float *dz, float *qv, float *qc, float *qr, float *qi, float *qs,
                    float *qg, float *ni, float *nr, float *nc, float *nwfa, float *nifa,
                    float *ng, float *qb, const float *qc_bl, const float *qcfrac_bl,
                    float *qcfrac, float *qifrac, const float *thten_bl, const float *qvten_bl,
                    const float *qcten_bl, const float *qiten_bl, const float *thten_lwrad,
                    const float *thten_swrad, const int *land_input, int ids, int ide, int jds,
                    int jde, int kds, int kde, int ims, int ime, int jms, int jme, int kms,
                    int kme, int its, int ite, int jts, int jte, int kts, int kte,
                    tempo_diags_t *tempo_diags);

/* tempo_run on DEVICE arrays (doubles) already resident in HBM, enqueued on `stream`
 * (a cudaStream_t); returns after enqueueing.  Same
 * arguments as tempo_run_c minus the inert ones.  A NULL stream is the CUDA default
 * stream, so the call orders with other work issued there.  The calling thread's
 * current device must be the context's device (the stream and the arrays belong to
 * it); otherwise TEMPO_ERR_STATE before any work is enqueued. */
int tempo_run_dev_c(tempo_ctx_t *ctx, const tempo_cfgs_t *tempo_cfgs, double dt,
                    int itimestep, double *t, double *th, const double *pii, const double *p,
                    const double *w, const double *dz, double *qv, double *qc, double *qr,
                    double *qi, double *qs, double *qg, double *ni, double *nr, double *nc,
                    double *nwfa, double *nifa, double *ng, double *qb, const int *land_input,
                    int ims, int ime, int jms, int jme, int kms, int kme, int its, int ite,
                    int jts, int jte, int kts, int kte, tempo_diags_t *tempo_diags,
                    void *stream);

/* tempo_run on DEVICE arrays of floats (FP32 storage). */
int tempo_run_dev_f32_c(tempo_ctx_t *ctx, const tempo_cfgs_t *tempo_cfgs, float dt,
                        int itimestep, float *t, float *th, const float *pii, const float *p,
                        const float *w, const float *dz, float *qv, float *qc, float *qr,
                        float *qi, float *qs, float *qg, float *ni, float *nr, float *nc,
                        float *nwfa, float *nifa, float *ng, float *qb, const int *land_input,
                        int ims, int ime, int jms, int jme, int kms, int kme, int its, int ite,
                        int jts, int jte, int kts, int kte, tempo_diags_t *tempo_diags,
                        void *stream);

/* No reference counterpart.  tempo_run_dev_f32_c (TEMPO_PREC_MIXED) that allocates no
 * memory: for hosts that must not allocate device memory inside their time step (a
 * model whose device memory pool is sized once at start-up with no headroom, or one
 * that must not let a physics call synchronise the device, as cudaFree does).  The
 * step's scratch is a fixed 64 MiB device array of the library.  The array is reserved
 * on a device when the library's device code is loaded there; with CUDA's lazy module
 * loading (the default) that is the first use of the library's kernels on the device,
 * so make the first call of this entry point (which also looks up the array's address,
 * with that device current) before the host sizes its memory pool, before any stream
 * capture and before any phase in which the host forbids CUDA runtime set-up.  The
 * calling thread's current device must be the context's device (TEMPO_ERR_STATE
 * otherwise, before any work).  Every call reuses the array and finds the previous
 * call's contents there; the step clears what must start at zero (its active-column
 * counter) itself.  Tiles that need more scratch (about 245 * nz + 45 bytes per column:
 * about 4 200 columns at 65 levels) are rejected with TEMPO_ERR_ARG.  The scratch is
 * shared by every context on a device: calls on one device must not overlap (issue
 * them on one stream, or wait for one call's work before the next starts on another
 * stream); overlapping calls race on the scratch.  The call records no kernel timing:
 * after it, tempo_kernel_times_c returns TEMPO_ERR_STATE until a timed run.  Results
 * equal tempo_run_dev_f32_c's. */
int tempo_run_dev_f32_noalloc_c(tempo_ctx_t *ctx, const tempo_cfgs_t *tempo_cfgs, float dt,
                                int itimestep, float *t, float *th, const float *pii,
                                const float *p, const float *w, const float *dz, float *qv,
                                float *qc, float *qr, float *qi, float *qs, float *qg, float *ni,
                                float *nr, float *nc, float *nwfa, float *nifa, float *ng,
                                float *qb, const int *land_input, int ims, int ime, int jms,
                                int jme, int kms, int kme, int its, int ite, int jts, int jte,
                                int kts, int kte, tempo_diags_t *tempo_diags, void *stream);

/* One domain of a multi-domain batch: its time step, step count, device arrays (floats)
 * and tile bounds, with the meaning they have in tempo_run_dev_f32_c. */
typedef struct {
  float dt;
  int itimestep;
  tempo_state_t state;   /* device arrays; NULL = absent, as in tempo_run */
  tempo_diags_t diags;   /* device arrays, tile-shaped; NULL = not requested */
  int ims, ime, jms, jme, kms, kme, its, ite, jts, jte, kts, kte;
} tempo_domain_t;

/* No reference counterpart (a host with several domains calls tempo_run once per
 * domain).  The mixed step (TEMPO_PREC_MIXED, FP32 device arrays) of `ndomains`
 * independent domains, each with its own levels, dt, arrays and step count, as ONE
 * sequence of launches on `stream`: every kernel of the step runs over the active work of
 * all domains at once (the points kernel drawing (domain, point) items from one work
 * queue), so small domains do not leave the GPU idle.  Each domain's results equal those
 * of its own tempo_run_dev_f32_c call.  1 <= ndomains <= 256; the semi-Lagrangian,
 * melting-layer and ML cloud-number paths are not supported (TEMPO_ERR_UNSUPPORTED).
 * Uses the context's scratch (grown with cudaMalloc on demand), the sedimentation
 * variant and point order of the context; returns after enqueueing.  The calling
 * thread's current device must be the context's. */
int tempo_run_batch_dev_f32_c(tempo_ctx_t *ctx, const tempo_cfgs_t *tempo_cfgs, int ndomains,
                              const tempo_domain_t *domains, void *stream);

/* tempo_aerosol_surface_emissions (src/module_mp_tempo_driver.F90:516-529) on device
 * arrays: nwfa(i,kts,j) += nwfa2d(i,j)*dt over the memory range.  The calling thread's
 * current device must be the context's (otherwise TEMPO_ERR_STATE, nothing enqueued). */
int tempo_aerosol_surface_emissions_dev_c(tempo_ctx_t *ctx, double dt, double *nwfa,
                                          const double *nwfa2d, int ims, int ime, int jms,
                                          int jme, int kms, int kme, int kts, void *stream);

/* Table export/import in the reference's file formats (big-endian stream FP64,
 * src/module_mp_tempo_tables.F90:96-444, read back by driver:532-622).  name is one
 * of "qr_acr_qg", "qr_acr_qs", "freezewater". */
int tempo_write_table_c(tempo_ctx_t *ctx, const char *name, const char *path);

/* Copies a lookup table or derived constant array from the context to host memory in
 * the reference's Fortran order (e.g. "tcg_racg", "t_efrw", "tnc_wev", "tpi_ide").
 * count is the element count of host_out (doubles); *needed receives the size. */
int tempo_get_table_c(tempo_ctx_t *ctx, const char *name, double *host_out, long count,
                      long *needed);

/* Rebuilds the three large tables on the GPU in FP64 (tables.F90:493-805 semantics)
 * and reports the device time in milliseconds. */
int tempo_build_tables_c(tempo_ctx_t *ctx, float *elapsed_ms);

/* Per-call counters of the last run on this context: [0] columns, [1] early-exit
 * columns, [2..6] max sedimentation substeps rain/graupel/snow/ice/cloud, [7]
 * kernel launches. */
int tempo_last_stats_c(tempo_ctx_t *ctx, long out[8]);

/* No reference counterpart.  With on != 0, each later run records CUDA events on its
 * stream around its kernels; tempo_kernel_times_c waits for the last run's events and
 * returns five durations in milliseconds: prep, the regime-order kernels (0 in
 * level-major order), points, sedim, final.  It returns TEMPO_ERR_STATE when the last
 * run recorded no events (timing off, or tempo_run_dev_f32_noalloc_c). */
int tempo_set_kernel_timing(tempo_ctx_t *ctx, int on);
int tempo_kernel_times_c(tempo_ctx_t *ctx, float ms[5]);

/* No reference counterpart.  Autotuner of the mixed form on FP32 device storage.  For
 * each of 22 candidates it copies the given state and runs `reps` consecutive steps
 * (itimestep, itimestep + 1, ...) on the copy -- the caller's arrays are not modified
 * -- timing kernels with CUDA events on `stream`, and scores the candidate by its
 * median step time.  Candidates 0-15: every variant of the per-level kernel (block
 * shape, barriers, register budget) in each order of the points (candidate v: variant
 * v % 8, order v / 8, as tempo_set_points_variant and tempo_set_points_order take
 * them), timed over the regime-order and per-level kernels; candidates 16-27: the
 * sedimentation variants 0-11 (tempo_set_sedim_variant) with the best of 0-15, timed
 * over the sedimentation kernel.  The best of each group is kept for later runs (all
 * precisions).  Tune on a state like the ones the runs will see: the work of a step
 * depends on the state it starts from.  Arguments as tempo_run_dev_f32_c; times_ms
 * (optional, `count` entries) receives each candidate's median time, *chosen
 * (optional) the per-level candidate kept.  Needs device memory for a copy of every
 * array the step writes. */
int tempo_autotune_dev_f32_c(tempo_ctx_t *ctx, const tempo_cfgs_t *tempo_cfgs, float dt,
                             int itimestep, float *t, float *th, const float *pii,
                             const float *p, const float *w, const float *dz, float *qv,
                             float *qc, float *qr, float *qi, float *qs, float *qg, float *ni,
                             float *nr, float *nc, float *nwfa, float *nifa, float *ng,
                             float *qb, const int *land_input, int ims, int ime, int jms,
                             int jme, int kms, int kme, int its, int ite, int jts, int jte,
                             int kts, int kte, tempo_diags_t *tempo_diags, void *stream,
                             int reps, float *times_ms, int count, int *chosen);
/* No reference counterpart.  Tangent-linear step on device arrays: x is advanced by one
 * step exactly as tempo_run_dev_c does (fp64 != 0: the FP64 step on doubles; else the
 * all-FP32 step on floats), and dx, the tangent of the differentiated inputs (t or th,
 * qv, qc, nc, qr, nr, qi, ni, qs, qg and, hail-aware, ng and qb; NULL entries = zero),
 * is replaced by the tangent of the outputs.  ddiags receives the tangents of the
 * requested diagnostics.  Branches, clips and table bins are those of the trajectory
 * from x.  Returns after the step has finished.  The calling thread's current device
 * must be the context's (otherwise TEMPO_ERR_STATE before any work). */
int tempo_tl_dev_c(tempo_ctx_t *ctx, const tempo_cfgs_t *tempo_cfgs, double dt, int itimestep,
                   int fp64, tempo_state_t *x, tempo_state_t *dx, tempo_diags_t *tempo_diags,
                   tempo_diags_t *tangent_diags, int ims, int ime, int jms, int jme, int kms,
                   int kme, int its, int ite, int jts, int jte, int kts, int kte, void *stream);

/* No reference counterpart.  Adjoint step on device arrays: x is the state before the
 * step (not modified); lam holds on entry the adjoints of the step's outputs (same
 * fields as dx of tempo_tl_dev_c; NULL entries = zero) and on return the adjoints of
 * its inputs; lam_diags (optional) gives the adjoints of the surface precipitation
 * (rain, ice, snow, graupel) and of refl10cm (dBZ).  Needs device memory for the
 * recomputed trajectory and checkpoints (about 10x the state).  Returns after the
 * adjoint has finished.  As for tempo_tl_dev_c, the calling thread's current device must
 * be the context's. */
int tempo_adjoint_dev_c(tempo_ctx_t *ctx, const tempo_cfgs_t *tempo_cfgs, double dt,
                        int itimestep, int fp64, const tempo_state_t *x, tempo_state_t *lam,
                        const tempo_diags_t *lam_diags, int ims, int ime, int jms, int jme,
                        int kms, int kme, int its, int ite, int jts, int jte, int kts, int kte,
                        void *stream);

/* The cloud-number network of the ML path, as init_ml_data stores it for the reference
 * (src/module_mp_tempo_driver.F90:703-735, src/module_mp_tempo_ml.F90:33-98): input
 * scaler means and variances (7 each; inputs qc, qr, qi, qs, p, T, w), weights00 (24 x 7,
 * column-major as reshape(nc_ml_w00, [24, 7])), bias00 (24), weights01 (24), bias01 (1).
 * Needed by runs with ml_for_nc_flag and no nc array: the single-moment cloud number of
 * each level is then the network's prediction (main:364-371) instead of a constant.  The
 * weights are the host's data (the library ships none); they are copied to the device. */
int tempo_set_ml_cloud_number_c(tempo_ctx_t *ctx, const double *mean, const double *var,
                                const double *weights00, const double *bias00,
                                const double *weights01, const double *bias01);

/* No reference counterpart.  Selects the per-level kernel variant directly (0..7). */
int tempo_set_points_variant(tempo_ctx_t *ctx, int variant);

/* No reference counterpart.  Order in which the per-level kernel's threads take the
 * active points: 0 (the default) = level-major; 1 = grouped by regime (species present
 * in the input state and the side of 0 C) inside windows of 32768 consecutive
 * level-major points, one extra kernel per step, so that a warp's points take the same
 * branches.  The order never changes a result, only which thread computes a point.
 * tempo_run_dev_f32_noalloc_c always runs level-major. */
int tempo_set_points_order(tempo_ctx_t *ctx, int order);

/* No reference counterpart.  Selects the sedimentation kernel variant directly (0..11):
 * variant % 3 + 1 levels whose loads a substep's sweep issues together; for variants
 * 3-5 and 9-11 a column's species split over two threads (rain and snow; graupel, ice
 * and cloud); variants 0-5 run a species' substeps level by level (one pass over the
 * column) when a warp's substep counts are at most 8, variants 6-11 substep by substep.
 * Variant 0 is the default.  Every variant computes the same values. */
int tempo_set_sedim_variant(tempo_ctx_t *ctx, int variant);

/* No reference counterpart.  Number of row slabs of later host-array runs (1..8; 0,
 * the default, takes one slab per 2^17 tile columns, at most 8, at least 1; from four
 * slabs on, the first and last hold a quarter and the second and second-to-last half
 * the rows of the others).  Never changes a result. */
int tempo_set_host_slabs(tempo_ctx_t *ctx, int slabs);

/* No reference counterpart.  The context's kernel choices: out[0] the per-level kernel
 * variant, out[1] the point order, out[2] the sedimentation variant. */
int tempo_tuning_c(tempo_ctx_t *ctx, int out[3]);

/* No reference counterpart.  With on != 0, a run captures its work (counter resets and
 * the step's kernels) into a CUDA graph the first time it sees a given argument set
 * (pointers, bounds, dt, flags, precision, kernel variants and point order) and replays
 * the graph on later runs with the same set; up to 16 graphs are kept per context.
 * With kernel timing on, the graph carries the timing events. */
int tempo_set_graphs(tempo_ctx_t *ctx, int on);

#ifdef __cplusplus
}
#endif
#endif
