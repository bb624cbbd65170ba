// tempo_types.h -- plain data structures shared by the host ABI layer and the kernels:
// the device table set, the launch arguments of the column step, option flags and
// the scratch field layout.  No device code here, so host C++ can include it.
#pragma once

#include <cstdint>

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
  F_DT_RIME = 1u << 16  // dt > timestep_conversion_rime_to_rain
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
// final (per active level: phase C).  Scratch is indexed by active-column slot s,
// [field][level][slot] with slot fastest.
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
  void* sd;           // Isl<R>[SD_N][nz][ncol_pad]
  void* sr;           // R[SR_N][nz][ncol_pad]
  void* sc;           // Isl<R>[SC_N][ncol_pad]
  void* hgt;          // Cst<R>[nz][ncol_pad]: level heights for the aerosol initial profiles
                      // (written only when nwfa or nifa is absent)
  int* act;           // [ncol_pad] column of each active slot
  unsigned int* nact; // active-slot counter (zero before prep)
  uint8_t* pmask;     // [nz][ncol_pad]
  uint8_t* cmask;     // [ncol_pad]
  unsigned long long* stats;  // [0] early exits, [1..5] max substeps
};

}  // namespace tg
