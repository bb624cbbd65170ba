// tempo_types.h -- plain data structures shared by the host ABI layer and the kernels:
// the device table set, the launch arguments of the column step, option flags and
// the scratch field layout.  No device code here, so host C++ can include it.
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define TG_HD __host__ __device__
#else
#define TG_HD
#endif

namespace tg {

// Device lookup tables.  The large collection/freezing tables are stored
// array-of-structures: one Fortran-order entry holds all arrays of its family next
// to each other, so one lookup touches one or two 32-byte sectors.
template <class R>
struct Tables {
  const R* t_efrw;    // (nbr, nbc)
  const R* t_efsw;    // (nbs, nbc)
  const R* tnc_wev;   // (nbc, ntb_c, nbc)
  const R* tps_iaus;  // (ntb_i, ntb_i1)
  const R* tni_iaus;
  const R* tpi_ide;
  const float* tnccn; // (7,9,7,5,4) FP32 as in the file
  const R* qg;        // [Fortran (i,j,n3,k,m) flat][5]: tcg_racg,tmr_racg,tcr_gacr,tnr_racg,tnr_gacr
  const R* qs;        // [Fortran (i,j,k,m) flat][12]: tcs_racs1,tmr_racs1,tcs_racs2,tmr_racs2,
                      //   tcr_sacr1,tms_sacr1,tcr_sacr2,tms_sacr2,tnr_racs1,tnr_racs2,tnr_sacr1,tnr_sacr2
  const R* qrfz;      // [Fortran (i,j,k,m) flat][4]: tpi_qrfz,tni_qrfz,tpg_qrfz,tnr_qrfz
  const R* qcfz;      // [Fortran (i,j,k,m) flat][2]: tpi_qcfz,tni_qcfz
  const double* edges;  // [kEdgesCount] least values of the log-index bins (tempo_consts.h)
};

enum : uint32_t {
  F_NC = 1u << 0,     // nc present (2-moment cloud / aerosol-aware cloud number)
  F_NWFA = 1u << 1,   // nwfa present
  F_NIFA = 1u << 2,   // nifa present
  F_HAIL = 1u << 3,   // ng and qb present (2-moment graupel with predicted density)
  F_QB = 1u << 4,     // qb present (graupel_fallspeed density path)
  F_LAND = 1u << 5,   // land_input present
  F_FIRST = 1u << 6,  // itimestep == 1
  F_NOMICRO = 1u << 7,  // turn_off_micro_flag
  F_COND = 1u << 8,     // cloud_condensation_flag
  F_REFL = 1u << 9, F_RE = 1u << 10, F_MHD = 1u << 11, F_MVDR = 1u << 12,
  F_MVDG = 1u << 13, F_NCMR = 1u << 14, F_USE_T = 1u << 15,
  F_DT_RIME = 1u << 16,  // dt > timestep_conversion_rime_to_rain
  F_SEMI = 1u << 17,     // semi_sedi_flag: semi-Lagrangian rain and graupel sedimentation
  F_MELT = 1u << 18,     // refl10cm_from_melting_flag (with refl10cm requested)
  F_MLNC = 1u << 19,     // ml_for_nc_flag without nc: cloud number from the network
  F_BLRE = 1u << 20      // qc_bl and qcfrac_bl given: boundary-layer cloud in re_cloud
};

// per-point scratch fields in the island type (thermodynamic and sedimentation islands)
enum SDField : int {
  SD_TTEN, SD_QV, SD_RHO,
  SD_XRR, SD_XNR, SD_XRG, SD_XNG, SD_XRB, SD_XRS, SD_XRI, SD_XNI, SD_XRC, SD_XNC,
  SD_TQR, SD_TNR, SD_TQG, SD_TNG, SD_TQB, SD_TQS, SD_TQI, SD_TNI, SD_TQC, SD_TNC,
  SD_ODZ, SD_OZR,  // 1 / dz and 1 / (dz rho) of the level (mixed form: sedimentation factors)
  SD_N
};
// per-point scratch fields in the bulk type R (fall-speed candidates; < 0 = absent)
enum SRField : int {
  SR_VTR, SR_VTNR, SR_VTG, SR_VTNG, SR_VTSA, SR_VTSB, SR_VTI, SR_VTNI, SR_VTC, SR_VTNC, SR_N
};
// per-column scratch in the island type: precipitation sums of the sedimentation
enum SCField : int { SC_PR, SC_PG, SC_PS, SC_PI, SC_PC, SC_N };
// per-point existence bits after phase A (any(l_q*) drives the sedimentation)
enum PMaskBit : uint8_t { PM_QR = 1, PM_QG = 2, PM_QS = 4, PM_QI = 8, PM_QC = 16 };
// per-column bits
enum CMaskBit : uint8_t { CM_GINIT = 1 };

// One step's arguments.  The step runs as four kernels over the tile's columns:
// prep (per column: early-exit test, compaction of active columns into slots),
// points (per active level: phase A), sedim (per active column: sedimentation),
// final (per active level: phase C).  Scratch is indexed by active-column slot s: a
// field plane per scratch field, point (level k, slot s) at pt_off(s, k, nz).
template <class S>
struct StepArgs {
  S *t, *th;
  const S *pii, *p, *w, *dz;
  S *qv, *qc, *qr, *qi, *qs, *qg, *ni, *nr, *nc, *nwfa, *nifa, *ng, *qb;
  const int* land;
  // diagnostics (tile shaped; NULL = off)
  S *rain_precip, *ice_precip, *snow_precip, *graupel_precip, *frozen_fraction, *frz_rain,
      *mhd_sfc, *mhd_col;
  S *refl10cm, *re_cloud, *re_ice, *re_snow, *mvd_r, *mvd_g, *ncmr;
  long NI, NK;        // memory extents ime-ims+1, kme-kms+1
  int i0, k0, j0;     // tile origin in memory: its-ims, kts-kms, jts-jms
  int ti, tj, nz;     // tile extents
  long ncol, ncol_pad;
  double dt;
  double odt;         // 1 / dt
  float dt_hi, dt_lo, odt_f;  // dt as a double-float pair and 1/dt in float (mixed form)
  double nc_single;   // single-moment cloud number (m^-3) when nc is absent and no land
  double niccn3, niin3;  // decay rates of the aerosol initial profiles (aerosols:14-73)
  uint32_t flags;
  // scratch planes of nz * ncol_pad points in the layout of pt_off
  void* sd;           // Isl<R>[SD_N] planes
  void* sr;           // R[SR_N] planes
  void* sc;           // Isl<R>[SC_N][ncol_pad]
  void* hgt;          // Cst<R> plane: level heights for the aerosol initial profiles
                      // (written only when nwfa or nifa is absent)
  int* act;           // [ncol_pad] column of each active slot
  unsigned int* nact; // [0] active-slot counter, [1] work-queue counter of the
                      // persistent points kernel (both zero before prep)
  uint8_t* pmask;     // plane: species present at the point after phase A
  uint8_t* cmask;     // [ncol_pad]
  unsigned long long* stats;  // [0] early exits, [1..5] max substeps
  void* slw;          // Isl<R>[kSlRows][nz + 2][ncol_pad]: semi-Lagrangian work rows (F_SEMI)
  void* mlw;          // melting-reflectivity record (F_MELT): double[kMeltN] planes, then
                      // a byte plane of MeltBit flags
  const double* mlnet;  // cloud-number network (F_MLNC), kMlNet values in the layout of
                        // tempo_set_ml_cloud_number_c
  void* ncw;          // R plane: the network's cloud number per point (F_MLNC)
  const S *qc_bl, *qcfrac_bl;  // boundary-layer cloud water and fraction (F_BLRE)
  // phase A's points in regime order: thread q takes level-major point ord[q] (point p
  // at level p / nact of slot p % nact); NULL = level-major order
  unsigned* ord;
  // decision trace of a test build (TEMPO_TRACE): kTracePoint ints per (tile column,
  // level) point, column c's level k at (c * nz + k) * kTracePoint, then kTraceColumn
  // ints per tile column; NULL = off.  Product builds never write it.
  int* trace;
};

// A multi-domain batch (tempo_run_batch_dev_f32_c): nd tiles, each with its own step
// arguments (levels, dt, arrays, scratch), stepped by one sequence of launches.  Work
// items are numbered across the batch: tile columns domain after domain (col_start), and,
// after prep, active slots (slot_start) and level-major points (pt_start).
constexpr int kMaxDomains = 256;
template <class S>
struct BatchArgs {
  const StepArgs<S>* dom;  // [nd] each domain's step arguments (device copy)
  const long* col_start;   // [nd + 1] first batch column of each domain
  unsigned* slot_start;    // [nd + 1] first batch slot of each domain (written after prep)
  unsigned* pt_start;      // [nd + 1] first batch point of each domain (written after prep)
  unsigned* queue;         // work queue of the persistent points kernel (zeroed after prep)
  unsigned* ord;           // batch points in regime order (NULL: domain by domain, level-major)
  int nd;
  long ncol;               // sum of the domains' tile columns
  long npts_max;           // sum of the domains' columns x levels (grid bound of the point kernels)
};

// Layout of the decision trace (test builds compiled with TEMPO_TRACE).  The oracle
// records the same layout, so a test compares every table index and branch decision
// of a step with the oracle's.  Per point: the existence and limit bits of each pass of
// the check routines (0 initial checks, 1 checks on temporaries after the rates, 2 the
// cloud check after condensation, 3 the rain check after evaporation, 4 the final
// checks), the table indices of each rate routine, the over-depletion limiter's
// branches.  Per column: substep counts and top levels of the sedimentation.
enum TraceSlot : int {
  TR_CHECK = 0,   // + pass (0..4): TraceCheckBit | idx_bg << 12 | nu_c << 16
  TR_RW = 5,      // warm_rain: efrw rain bin | int(mvd_c 1e6) << 8 | branch bits << 16
  TR_RS = 6,      // rain-snow: idx_s | idx_t << 6 | idx_r1 << 12 | idx_r << 18 | taken << 24
  TR_RG = 7,      // rain-graupel: idx_g1 | idx_g << 6 | idx_r1 << 12 | idx_r << 18 | taken << 24
  TR_FZR = 8,     // rain freezing: idx_r | idx_r1 << 6 | idx_tc << 12 | idx_in << 18 | taken << 24
  TR_FZC = 9,     // cloud freezing: idx_c | idx_n << 8 | taken << 16
  TR_ICE = 10,    // ice_processes: idx_i | idx_i1 << 8 | taken << 16
  TR_RIME = 11,   // riming: efsw snow bin | int(mvd_c 1e6) << 8 | taken << 16
  TR_EVAP = 12,   // droplet evaporation: idx_d | idx_c << 8 | idx_n << 16 | taken << 24
  TR_LIMIT = 13,  // check_over_depletion: one bit per rescaled group
  TR_RANGE = 14,  // table indices found out of their table's range (RangeSite bits; the
                  // index is clamped before the read).  The oracle never sets it.
  kTracePoint = 16
};
// table-read sites whose indices the test build checks against the table's bounds
enum RangeSite : int {
  RG_EFRW = 1, RG_EFSW = 2, RG_QS = 4, RG_QG = 8, RG_QRFZ = 16, RG_QCFZ = 32, RG_ICE = 64,
  RG_EVAP = 128
};
enum TraceCheckBit : int {
  TB_QC = 1, TB_QC_HIT = 2, TB_QR = 4, TB_QR_HIT = 8, TB_QI = 16, TB_QI_HIT = 32,
  TB_QS = 64, TB_QG = 128, TB_QG_HIT = 256
};
constexpr int kTraceColumn = 10;  // substeps rain, graupel, snow, ice; ktop rain, graupel, snow, ice, cloud; spare
// regimes of a point (tempo_step.cuh: point_regime)
constexpr int kRegimes = 64;
// size of the cloud-number network: scaler means and variances (7 + 7), weights00
// (24 x 7, column-major), bias00 (24), weights01 (24), bias01 (1)
constexpr int kMlNet = 7 + 7 + 168 + 24 + 24 + 1;

// Inputs of a point that carry derivatives in the tangent-linear and adjoint kernels
enum InId : int { IN_T, IN_QV, IN_QC, IN_NC, IN_QR, IN_NR, IN_QI, IN_NI, IN_QS, IN_QG, IN_NG, IN_QB, IN_N };
// Inputs of a point of phase C (final kernel) that carry derivatives
enum CInId : int {
  C_T1D, C_TTEN, C_QV, C_RHO, C_QC, C_NC, C_QR, C_NR, C_QI, C_NI, C_QS, C_QG, C_NG, C_QB,
  C_TQR, C_TNR, C_TQG, C_TNG, C_TQB, C_TQS, C_TQI, C_TNI, C_TQC, C_TNC, C_N
};
// Array outputs of a point
enum ArrId : int { A_T, A_QV, A_QC, A_NC, A_QR, A_NR, A_QI, A_NI, A_QS, A_QG, A_NG, A_QB, A_NWFA, A_NIFA, A_N };

template <class T, int N> struct Dual;

// Adjoint arguments (tempo_adjoint.cuh)
template <class T>
struct AdjArgs {
  T* lam[A_N];              // adjoint per ArrId (A_NWFA / A_NIFA unused), state layout
  T* lam_th;                // theta mode: adjoint of th
  T* lam_refl;              // tile 3-D, adjoint of refl10cm (dBZ); NULL = 0
  T* lam_precip[4];         // tile 2-D: rain, ice, snow, graupel; NULL = 0
  T* lam_sd;                // [SD_N][nz][ncol_pad]
  T* lam_sr;                // [SR_N][nz][ncol_pad]
  const Dual<T, 1>* psd;    // primal scratch (island fields) the phase reads
  const Dual<T, 1>* psr;    // primal fall-speed candidates (sedimentation adjoint)
  const Dual<T, 1>* psc;    // primal per-column sums
  const uint8_t* colflag;   // [ncol]: 1 = active column
};

// Point layout of the scratch planes (sd, sr, pmask, hgt and the adjoint's copies):
// each field plane holds nz * ncol_pad points; slots form tiles of kSlotTile consecutive
// slots, a tile stores its levels one after another, its slots fastest.  A warp over 32
// aligned slots of one level touches one contiguous segment (whole 32-byte sectors for
// every element size); a thread walking one slot's levels stays inside nz * kSlotTile
// entries (within one memory page), so a column's levels never spread over the whole
// plane.
constexpr int kSlotTile = 32;
// work rows of the semi-Lagrangian sweep per column (zi, wi, za, dza, qa, qmi, qpi, x0)
constexpr int kSlRows = 8;
// per-point record of phase C for the melting-layer reflectivity pass (F_MELT)
enum MeltVal : int { MV_ZER, MV_ZES, MV_ZEG, MV_RS, MV_SMOB, MV_SMOC, MV_RR, MV_RG, MV_NG, MV_ILAMG,
                     MV_IDX, kMeltN };
enum MeltBit : uint8_t { MB_WARMRAIN = 1, MB_QS = 2, MB_QG = 4 };
TG_HD inline long pt_base(long s, int nz) { return (s / kSlotTile) * (long)nz * kSlotTile + (s % kSlotTile); }
TG_HD inline long pt_off(long s, int k, int nz) { return pt_base(s, nz) + (long)k * kSlotTile; }

// Workspace rows (T, [row][slot]): working state of the 10 sedimenting fields, their
// filled fall speeds, checkpoints every 4 substeps, the pre-substep states of one block
// of 4 substeps, and one row of flux adjoints.
struct SedWork {
  int nck;      // checkpoints per field
  long rows;    // rows in total
  TG_HD long xw(int f, int k, int nz) const { return (long)f * nz + k; }
  TG_HD long vf(int f, int k, int nz) const { return 10L * nz + (long)f * nz + k; }
  TG_HD long ck(int f, int c, int k, int nz) const {
    return 20L * nz + ((long)f * nck + c) * nz + k;
  }
  TG_HD long bb(int fi, int n, int k, int nz) const {
    return 20L * nz + 10L * nck * nz + ((long)fi * 4 + n) * nz + k;
  }
  TG_HD long ls(int k, int nz) const { return 20L * nz + 10L * nck * nz + 12L * nz + k; }
  TG_HD static long rows_for(int nck, int nz) { return (20L + 10L * nck + 13L) * nz; }
};

}  // namespace tg
