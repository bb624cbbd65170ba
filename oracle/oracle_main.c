/*
 * oracle_main.c -- CPU restatement (test infrastructure) of the TEMPO column step:
 * module_mp_tempo_main.F90 (tempo_main :73-864 and the routines it calls),
 * module_mp_tempo_aerosols.F90, module_mp_tempo_diags.F90 (non-melting parts) and
 * module_mp_tempo_driver.F90 tempo_run (:187-513).  Levels are 0-based here
 * (k0 = k-1); every comment cites the Fortran line it restates.
 */
#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle_common.h"
#include "tempo_oracle.h"

/* Rounding-tie detection (oracle-only instrumentation, no effect on results).
 * nint(x) and int(y) are discontinuous at half-integers and integers; where the
 * reference's arithmetic puts an argument there up to one rounding (e.g. the graupel
 * density class 10*rg/rb = 0.5 when rb sits at its clamp rg*1000/rho_g(1)), any
 * last-bit difference of a libm result moves the index.  The column is flagged so
 * that a comparison can tell such branch flips from real mismatches. */
static _Thread_local int t_tie;      /* flags of the current column */
static _Thread_local int t_tie_bit;  /* 1 before sedimentation, 2 in the final checks */
static int *g_tie_sink;
void oracle_set_tie_sink(int *flags) { g_tie_sink = flags; }
static inline int nint_tie(double x) {
  double f = x - floor(x);
  if (fabs(f - 0.5) <= 1e-12 * fmax2(1.0, fabs(x))) t_tie |= t_tie_bit;
  return nint(x);
}
/* Decision trace (oracle-only instrumentation, no effect on results): every table index
 * and branch decision of a step, per (tile column, level) point TRP ints and per column
 * TRC ints, in the layout the GPU library's test build records (TraceSlot and
 * TraceCheckBit in tempo_gb300/csrc/tempo_types.h), so a test compares them exactly. */
enum { TR_CHECK = 0, TR_RW = 5, TR_RS = 6, TR_RG = 7, TR_FZR = 8, TR_FZC = 9, TR_ICE = 10,
       TR_RIME = 11, TR_EVAP = 12, TR_LIMIT = 13, TRP = 16, TRC = 10 };
enum { TB_QC = 1, TB_QC_HIT = 2, TB_QR = 4, TB_QR_HIT = 8, TB_QI = 16, TB_QI_HIT = 32,
       TB_QS = 64, TB_QG = 128, TB_QG_HIT = 256 };
static int *g_trace;                 /* [ncol * nz * TRP] points, then [ncol * TRC] columns */
static _Thread_local int *t_trace;   /* the current column's point records (NULL = off) */
static _Thread_local int *t_trace_col;
static _Thread_local int t_tpass;    /* pass of the check routines */
void oracle_set_trace(int *buf) { g_trace = buf; }
#define TRACE(k, slot, bits)                                       \
  do {                                                             \
    if (t_trace) t_trace[(long)(k) * TRP + (slot)] |= (int)(bits); \
  } while (0)
#define TRACE_COL(j, v)                    \
  do {                                     \
    if (t_trace_col) t_trace_col[j] = (v); \
  } while (0)

static inline int int_tie(double y, int current_max) {
  if ((int)y + 1 >= current_max && fabs(y - nearbyint(y)) <= 1e-12 * fmax2(1.0, fabs(y)))
    t_tie |= 1;
  return (int)y;
}

/* ty_tend (main:47-64): 74 FP64 process-rate columns, in the tend_work order :167-266 */
enum {
  PRR_WAU, PNR_WAU, PNC_WAU, PRR_RCW, PNC_RCW, PNR_RCR,
  PRS_SCW, PNC_SCW, PNG_SCW, PBG_SCW, PRG_GCW, PNC_GCW, PBG_GCW, PRI_IHM, PNI_IHM, PRS_IHM, PRG_IHM, PRG_SCW,
  PRR_RCS, PNR_RCS, PRG_RCS, PNG_RCS, PRS_RCS, PBG_RCS,
  PRR_RCG, PNR_RCG, PRG_RCG, PNG_RCG, PBG_RCG,
  PRI_INU, PNI_INU, PRI_IHA, PNI_IHA,
  PRI_WFZ, PNI_WFZ,
  PRG_RFZ, PNG_RFZ, PNR_RFZ, PRI_RFZ, PNI_RFZ, PBG_RFZ,
  PRS_SDE, PRI_IDE, PNI_IDE, PRS_IDE, PRG_GDE, PNG_GDE,
  PNI_IAU, PRS_IAU,
  PRR_SML, PRR_GML, PBG_SML, PBG_GML, PNR_SML, PNR_GML,
  PRR_RCI, PNR_RCI, PRI_RCI, PNI_RCI, PRG_RCI, PNG_RCI, PBG_RCI,
  PNI_SCI, PRS_SCI,
  PRW_VCD, PNC_WCD, PRV_REV, PNR_REV,
  PNA_RCA, PNA_SCA, PNA_GCA, PND_RCD, PND_SCD, PND_GCD,
  NTEND
};
#define TD(name) tw[(long)(name) * nz + k]

/* per-column workspace (the local arrays of tempo_main :120-148) */
typedef struct {
  int nz;
  double *tten, *qvten, *qcten, *qiten, *qrten, *qsten, *qgten, *qbten, *niten, *nrten, *ncten,
      *ngten, *nwfaten, *nifaten;
  int *l_qc, *l_qi, *l_qr, *l_qs, *l_qg, *idx_bg;
  double *temp, *pres, *qv, *rho, *rhof, *rhof2, *qvs, *qvsi, *delqvs, *satw, *sati, *ssatw, *ssati,
      *diffu, *visco, *vsc2, *tcond, *lvap, *ocp, *lvt2;
  double *rc, *ri, *rr, *rs, *rg, *rb, *ni, *nr, *nc, *ng, *nwfa, *nifa;
  double *ilamc, *ilami, *ilamr, *ilamg, *mvd_r, *mvd_c, *mvd_g;
  double *smob, *smo2, *smo1, *smo0, *smoc, *smoe, *smof, *smog, *ns, *smoz;
  double *xrx, *xnx, *xncx, *xngx, *xqbx, *ncsave;
  double *vtrr, *vtnr, *vtrs, *vtri, *vtni, *vtrg, *vtng, *vtrc, *vtnc, *vtboost;
  double *tw, *t1_subl, *sed_r, *hgt;
  double *mhd, *refl, *re_c, *re_i, *re_s, *ze_r, *ze_s, *ze_g;
  void *block_d, *block_i;
} ws_t;

static ws_t *ws_new(int nz) {
  ws_t *w = (ws_t *)calloc(1, sizeof(ws_t));
  w->nz = nz;
  double **d[] = {&w->tten, &w->qvten, &w->qcten, &w->qiten, &w->qrten, &w->qsten, &w->qgten,
                  &w->qbten, &w->niten, &w->nrten, &w->ncten, &w->ngten, &w->nwfaten,
                  &w->nifaten, &w->temp, &w->pres, &w->qv, &w->rho, &w->rhof, &w->rhof2,
                  &w->qvs, &w->qvsi, &w->delqvs, &w->satw, &w->sati, &w->ssatw, &w->ssati,
                  &w->diffu, &w->visco, &w->vsc2, &w->tcond, &w->lvap, &w->ocp, &w->lvt2,
                  &w->rc, &w->ri, &w->rr, &w->rs, &w->rg, &w->rb, &w->ni, &w->nr, &w->nc,
                  &w->ng, &w->nwfa, &w->nifa, &w->ilamc, &w->ilami, &w->ilamr, &w->ilamg,
                  &w->mvd_r, &w->mvd_c, &w->mvd_g, &w->smob, &w->smo2, &w->smo1, &w->smo0,
                  &w->smoc, &w->smoe, &w->smof, &w->smog, &w->ns, &w->smoz, &w->xrx, &w->xnx,
                  &w->xncx, &w->xngx, &w->xqbx, &w->ncsave, &w->vtboost, &w->t1_subl,
                  &w->sed_r, &w->hgt, &w->mhd, &w->refl, &w->re_c, &w->re_i, &w->re_s,
                  &w->ze_r, &w->ze_s, &w->ze_g};
  double **dp1[] = {&w->vtrr, &w->vtnr, &w->vtrs, &w->vtri, &w->vtni,
                    &w->vtrg, &w->vtng, &w->vtrc, &w->vtnc};
  int nd = (int)(sizeof d / sizeof d[0]), nd1 = (int)(sizeof dp1 / sizeof dp1[0]);
  long total = (long)nd * nz + (long)nd1 * (nz + 1) + (long)NTEND * nz;
  double *blk = (double *)calloc((size_t)total, sizeof(double));
  long off = 0;
  for (int a = 0; a < nd; a++, off += nz) *d[a] = blk + off;
  for (int a = 0; a < nd1; a++, off += nz + 1) *dp1[a] = blk + off;
  w->tw = blk + off;
  int **ip[] = {&w->l_qc, &w->l_qi, &w->l_qr, &w->l_qs, &w->l_qg, &w->idx_bg};
  int *iblk = (int *)calloc((size_t)6 * nz, sizeof(int));
  for (int a = 0; a < 6; a++) *ip[a] = iblk + (long)a * nz;
  w->block_d = blk;
  w->block_i = iblk;
  return w;
}
static void ws_free(ws_t *w) {
  if (!w) return;
  free(w->block_d);
  free(w->block_i);
  free(w);
}

/* tempo_main_diags (main:29-45) */
typedef struct {
  double rain_precip, cloud_precip, ice_liquid_equiv_precip, snow_liquid_equiv_precip,
      graupel_liquid_equiv_precip, frozen_fraction, frz_rain_precip;
  int early_exit;
  int substeps[5];
} mdiag_t;

/* ------------------------------------------------------------------------------ */
/* aerosols.F90                                                                     */
/* ------------------------------------------------------------------------------ */
/* init_water_friendly_aerosols / init_ice_friendly_aerosols (aerosols:14-73) */
static void init_aerosols(int nz, const double *dz1d, double *x, double *hgt, double n0_,
                          double n1_) {
  hgt[0] = 0.0;
  for (int k = 1; k < nz; k++) hgt[k] = hgt[k - 1] + dz1d[k];
  double h_01;
  if (hgt[0] <= 1000.0)
    h_01 = 0.8;
  else if (hgt[0] >= 2500.0)
    h_01 = 0.01;
  else
    h_01 = 0.8 * cos(hgt[0] * 0.001 - 1.0);
  double n3 = -1.0 * log(n1_ / n0_) / h_01;
  x[0] = n1_ + n0_ * exp(-((hgt[1] - hgt[0]) / 1000.0) * n3);
  for (int k = 1; k < nz; k++) x[k] = n1_ + n0_ * exp(-((hgt[k] - hgt[0]) / 1000.0) * n3);
}

/* aerosol_collection_efficiency (aerosols:76-118) */
static double aerosol_collection_efficiency(double d, double da, double visc, double rhoa,
                                            double temp, char species) {
  const double boltzman = 1.3806503e-23, meanpath = 0.0256e-6;
  double vt = 1.0, rho_p = rho_w;
  if (species == 'r') {
    vt = -0.1021 + 4.932e3 * d - 0.9551e6 * d * d + 0.07934e9 * d * d * d -
         0.002362e12 * d * d * d * d;
    rho_p = rho_w;
  } else if (species == 's') {
    vt = av_s * pow(d, bv_s);
    rho_p = rho_s;
  } else if (species == 'g') {
    vt = AV_G(idx_bg1) * pow(d, BV_G(idx_bg1));
    rho_p = RHO_G(idx_bg1);
  }
  double cc = 1.0 + 2.0 * meanpath / da * (1.257 + 0.4 * exp(-0.55 * da / meanpath));
  double diff = boltzman * temp * cc / (3.0 * pi * visc * da);
  double re = 0.5 * rhoa * d * vt / visc;
  double scn = visc / (rhoa * diff);
  double st = (rho_p - rhoa) * da * da * vt * cc / (9.0 * visc * d);
  double aval = log(1.0 + re);
  double st2 = (1.2 + 1.0 / 12.0 * aval) / (1.0 + aval);
  double eff = 4.0 / (re * scn) * (1.0 + 0.4 * sqrt(re) * pow(scn, 0.3333) + 0.16 * sqrt(re) * sqrt(scn)) +
               4.0 * da / d * (0.02 + da / d * (1.0 + 2.0 * sqrt(re)));
  if (st > st2) eff = eff + pow((st - st2) / (st - st2 + 0.666667), 1.5);
  return fmax2(1.e-5, fmin2(eff, 1.0));
}

/* ------------------------------------------------------------------------------ */
/* check_and_update routines (main:867-1260)                                        */
/* ------------------------------------------------------------------------------ */
static void aerosol_check_and_update(int nz, const double *rho, const double *nwfa1d,
                                     const double *nifa1d, double *nwfa, double *nifa,
                                     const double *nwfaten, const double *nifaten, double dt) {
  for (int k = 0; k < nz; k++) {
    if (nwfa1d) nwfa[k] = (nwfa1d[k] + nwfaten[k] * dt) * rho[k];
    if (nifa1d) nifa[k] = (nifa1d[k] + nifaten[k] * dt) * rho[k];
    nwfa[k] = fmax2(nwfa_default * rho[k], fmin2(aero_max * rho[k], nwfa[k]));
    nifa[k] = fmax2(nifa_default * rho[k], fmin2(aero_max * rho[k], nifa[k]));
  }
}

/* cloud_check_and_update (main:891-973) */
static void cloud_check_and_update(int nz, const double *rho, int *l_qc, double *qc1d, double *nc1d,
                                   const double *ncsave, double *rc, double *nc, double *qcten,
                                   double *ncten, double *ilamc, double *mvd_c, double dt,
                                   double odt) {
  for (int k = 0; k < nz; k++) {
    int hit_limit = 0, nu_c;
    double lamc, xdc;
    if (qc1d[k] + qcten[k] * dt > r1) {
      l_qc[k] = 1;
      rc[k] = (qc1d[k] + qcten[k] * dt) * rho[k];
      qc1d[k] = qc1d[k] + qcten[k] * dt;
      if (nc1d) {
        nc[k] = fmax2(nt_c_min, (nc1d[k] + ncten[k] * dt) * rho[k]);
        if (nc[k] <= nt_c_min) {
          hit_limit = 1;
          nc[k] = nt_c_min;
        }
        if (nc[k] > nt_c_max) {
          hit_limit = 1;
          nc[k] = nt_c_max;
        }
        nu_c = o_get_nuc(nc[k]);
        lamc = pow(nc[k] * am_r * CCG(2, nu_c) * OCG1(nu_c) / rc[k], obmr);
        xdc = (bm_r + nu_c + 1.0) / lamc;
        if (xdc < d0c) {
          lamc = CCE(2, nu_c) / d0c;
          hit_limit = 1;
        } else if (xdc > d0r * 2.0) {
          lamc = CCE(2, nu_c) / (d0r * 2.0);
          hit_limit = 1;
        }
        nc[k] = CCG(1, nu_c) * OCG2(nu_c) * rc[k] / am_r * pow(lamc, bm_r);
        if (hit_limit) ncten[k] = (nc[k] / rho[k] - nc1d[k]) * odt;
        nc1d[k] = fmax2(nt_c_min / rho[k],
                        fmin2(CCG(1, nu_c) * OCG2(nu_c) * qc1d[k] / am_r * pow(lamc, bm_r),
                              nt_c_max / rho[k]));
      } else {
        nc[k] = ncsave ? ncsave[k] : nt_c_l;
      }
      nu_c = o_get_nuc(nc[k]);
      lamc = pow(nc[k] * am_r * CCG(2, nu_c) * OCG1(nu_c) / rc[k], obmr);
      ilamc[k] = 1.0 / lamc;
      mvd_c[k] = fmax2(fmin2((3.0 + nu_c + 0.672) * ilamc[k], d0r), d0c);
      TRACE(k, TR_CHECK + t_tpass, TB_QC | (hit_limit ? TB_QC_HIT : 0) | (nu_c << 16));
    } else {
      l_qc[k] = 0;
      rc[k] = r1;
      nc[k] = nt_c_min;
      mvd_c[k] = d0c;
      ilamc[k] = 0.0;
      qcten[k] = -qc1d[k] * odt;
      qc1d[k] = 0.0;
      if (nc1d) {
        ncten[k] = -nc1d[k] * odt;
        nc1d[k] = 0.0;
      }
    }
  }
}

/* rain_check_and_update (main:976-1042) */
static void rain_check_and_update(int nz, const double *rho, int *l_qr, double *qr1d, double *nr1d,
                                  double *rr, double *nr, double *qrten, double *nrten,
                                  double *ilamr, double *mvd_r, double dt, double odt) {
  for (int k = 0; k < nz; k++) {
    int hit_limit = 0;
    double lamr;
    if (qr1d[k] + qrten[k] * dt > r1) {
      l_qr[k] = 1;
      rr[k] = (qr1d[k] + qrten[k] * dt) * rho[k];
      qr1d[k] = qr1d[k] + qrten[k] * dt;
      nr[k] = fmax2(r2, (nr1d[k] + nrten[k] * dt) * rho[k]);
      if (nr[k] <= r2) {
        hit_limit = 1;
        mvd_r[k] = 1.0e-3;
        lamr = (3.0 + mu_r + 0.672) / mvd_r[k];
        nr[k] = CRG(2) * org3 * rr[k] * pow(lamr, bm_r) / am_r;
      }
      lamr = pow(am_r * CRG(3) * org2 * nr[k] / rr[k], obmr);
      mvd_r[k] = (3.0 + mu_r + 0.672) / lamr;
      if (mvd_r[k] > d0r_max) {
        hit_limit = 1;
        mvd_r[k] = d0r_max;
        lamr = (3.0 + mu_r + 0.672) / mvd_r[k];
        nr[k] = CRG(2) * org3 * rr[k] * pow(lamr, bm_r) / am_r;
      } else if (mvd_r[k] < d0r * 0.75) {
        hit_limit = 1;
        mvd_r[k] = d0r * 0.75;
        lamr = (3.0 + mu_r + 0.672) / mvd_r[k];
        nr[k] = CRG(2) * org3 * rr[k] * pow(lamr, bm_r) / am_r;
      }
      if (hit_limit) nrten[k] = (nr[k] / rho[k] - nr1d[k]) * odt;
      nr1d[k] = CRG(2) * org3 * qr1d[k] * pow(lamr, bm_r) / am_r;
      ilamr[k] = 1.0 / lamr;
      TRACE(k, TR_CHECK + t_tpass, TB_QR | (hit_limit ? TB_QR_HIT : 0));
    } else {
      l_qr[k] = 0;
      rr[k] = r1;
      nr[k] = r2;
      mvd_r[k] = d0r;
      ilamr[k] = 0.0;
      qrten[k] = -qr1d[k] * odt;
      nrten[k] = -nr1d[k] * odt;
      qr1d[k] = 0.0;
      nr1d[k] = 0.0;
    }
  }
}

/* ice_check_and_update (main:1045-1107) */
static void ice_check_and_update(int nz, const double *rho, int *l_qi, double *qi1d, double *ni1d,
                                 double *ri, double *ni, double *qiten, double *niten,
                                 double *ilami, double dt, double odt) {
  for (int k = 0; k < nz; k++) {
    int hit_limit = 0;
    double lami, xdi;
    if (qi1d[k] + qiten[k] * dt > r1) {
      l_qi[k] = 1;
      ri[k] = (qi1d[k] + qiten[k] * dt) * rho[k];
      qi1d[k] = qi1d[k] + qiten[k] * dt;
      ni[k] = fmax2(r2, (ni1d[k] + niten[k] * dt) * rho[k]);
      if (ni[k] <= r2) {
        hit_limit = 1;
        lami = CIE(2) / 5.e-6;
        ni[k] = fmin2(max_ni, CIG(1) * oig2 * ri[k] / am_i * pow(lami, bm_i));
      }
      lami = pow(am_i * CIG(2) * oig1 * ni[k] / ri[k], obmi);
      xdi = (bm_i + mu_i + 1.0) / lami;
      if (xdi < 5.e-6) {
        hit_limit = 1;
        lami = CIE(2) / 5.e-6;
        ni[k] = fmin2(max_ni, CIG(1) * oig2 * ri[k] / am_i * pow(lami, bm_i));
      } else if (xdi > d0s) {
        hit_limit = 1;
        lami = CIE(2) / d0s;
        ni[k] = CIG(1) * oig2 * ri[k] / am_i * pow(lami, bm_i);
      }
      if (hit_limit) niten[k] = (ni[k] / rho[k] - ni1d[k]) * odt;
      ni1d[k] = fmax2(r2 / rho[k], fmin2(CIG(1) * oig2 * qi1d[k] / am_i * pow(lami, bm_i),
                                         max_ni / rho[k]));
      ilami[k] = 1.0 / lami;
      TRACE(k, TR_CHECK + t_tpass, TB_QI | (hit_limit ? TB_QI_HIT : 0));
    } else {
      l_qi[k] = 0;
      ri[k] = r1;
      ni[k] = r2;
      ilami[k] = 0.0;
      qiten[k] = -qi1d[k] * odt;
      niten[k] = -ni1d[k] * odt;
      qi1d[k] = 0.0;
      ni1d[k] = 0.0;
    }
  }
}

/* snow_check_and_update (main:1110-1134) */
static void snow_check_and_update(int nz, const double *rho, int *l_qs, double *qs1d, double *rs,
                                  double *qsten, double dt, double odt) {
  for (int k = 0; k < nz; k++) {
    if (qs1d[k] + qsten[k] * dt > r1) {
      l_qs[k] = 1;
      rs[k] = (qs1d[k] + qsten[k] * dt) * rho[k];
      qs1d[k] = qs1d[k] + qsten[k] * dt;
      TRACE(k, TR_CHECK + t_tpass, TB_QS);
    } else {
      l_qs[k] = 0;
      rs[k] = r1;
      qsten[k] = -qs1d[k] * odt;
      qs1d[k] = 0.0;
    }
  }
}

/* graupel_check_and_update (main:1137-1231); ng1d/qb1d both non-NULL = hail-aware */
static void graupel_check_and_update(int nz, const double *rho, int *l_qg, double *qg1d,
                                     double *ng1d, double *qb1d, double *rg, double *ng,
                                     double *rb, int *idx, double *qgten, double *ngten,
                                     double *qbten, double *ilamg, double *mvd_g, double dt,
                                     double odt) {
  for (int k = 0; k < nz; k++) {
    int hit_limit = 0;
    double lamg;
    if (qg1d[k] + qgten[k] * dt > r1) {
      l_qg[k] = 1;
      rg[k] = (qg1d[k] + qgten[k] * dt) * rho[k];
      qg1d[k] = qg1d[k] + qgten[k] * dt;
      if (ng1d && qb1d) {
        ng[k] = fmax2(r2, (ng1d[k] + ngten[k] * dt) * rho[k]);
        rb[k] = fmin2(fmax2(rg[k] * meters3_to_liters / RHO_G(nrhg), (qb1d[k] + qbten[k] * dt) * rho[k]),
                      rg[k] * meters3_to_liters / RHO_G(1));
        idx[k] = imax(1, imin(nint_tie(10.0 * rg[k] / rb[k]) + 1, nrhg));
        if (ng[k] <= r2) {
          hit_limit = 1;
          mvd_g[k] = 1.5e-3;
          lamg = (3.0 + mu_g + 0.672) / mvd_g[k];
          ng[k] = CGG(2, 1) * ogg3 * rg[k] * pow(lamg, bm_g) / AM_G(idx[k]);
        }
        lamg = pow(AM_G(idx[k]) * CGG(3, 1) * ogg2 * ng[k] / rg[k], obmg);
        mvd_g[k] = (3.0 + mu_g + 0.672) / lamg;
        if (mvd_g[k] > 25.4e-3) {
          hit_limit = 1;
          mvd_g[k] = 25.4e-3;
          lamg = (3.0 + mu_g + 0.672) / mvd_g[k];
          ng[k] = CGG(2, 1) * ogg3 * rg[k] * pow(lamg, bm_g) / AM_G(idx[k]);
        } else if (mvd_g[k] < d0r) {
          hit_limit = 1;
          mvd_g[k] = d0r;
          lamg = (3.0 + mu_g + 0.672) / mvd_g[k];
          ng[k] = CGG(2, 1) * ogg3 * rg[k] * pow(lamg, bm_g) / AM_G(idx[k]);
        }
        if (hit_limit) ngten[k] = (ng[k] / rho[k] - ng1d[k]) * odt;
        ng1d[k] = CGG(2, 1) * ogg3 * qg1d[k] * pow(lamg, bm_g) / AM_G(idx[k]);
        qb1d[k] = fmin2(fmax2(qg1d[k] * meters3_to_liters / RHO_G(nrhg), qb1d[k] + qbten[k] * dt),
                        meters3_to_liters * qg1d[k] / RHO_G(1));
        idx[k] = imax(1, imin(nint_tie(10.0 * qg1d[k] / qb1d[k]) + 1, nrhg));
      } else {
        idx[k] = idx_bg1;
        double ygra1 = log10(fmax2(1.e-9, rg[k]));
        double zans1 = 3.4 + 2.0 / 7.0 * (ygra1 + 8.0);
        double n0_exp = fmax2(gonv_min, fmin2(pow(10.0, zans1), gonv_max));
        double lam_exp = pow(n0_exp * AM_G(idx[k]) * CGG(1, 1) / rg[k], oge1);
        lamg = lam_exp * pow(CGG(3, 1) * ogg2 * ogg1, obmg);
        ng[k] = CGG(2, 1) * ogg3 * rg[k] * pow(lamg, bm_g) / AM_G(idx[k]);
        rb[k] = meters3_to_liters * rg[k] / RHO_G(idx[k]);
      }
      ilamg[k] = 1.0 / lamg;
      mvd_g[k] = (3.0 + mu_g + 0.672) * ilamg[k];
      TRACE(k, TR_CHECK + t_tpass, TB_QG | (hit_limit ? TB_QG_HIT : 0) | (idx[k] << 12));
    } else {
      l_qg[k] = 0;
      rg[k] = r1;
      ng[k] = r2;
      mvd_g[k] = d0g;
      ilamg[k] = 0.0;
      idx[k] = idx_bg1;
      rb[k] = meters3_to_liters * r1 / RHO_G(idx[k]);
      qgten[k] = -qg1d[k] * odt;
      qg1d[k] = 0.0;
      if (ng1d && qb1d) {
        ngten[k] = -ng1d[k] * odt;
        qbten[k] = -qb1d[k] * odt;
        ng1d[k] = 0.0;
        qb1d[k] = 0.0;
      }
    }
  }
}

/* graupel_init (main:1234-1260) */
static void graupel_init(int nz, const double *rho, const double *qg1d, double *ng1d, double *qb1d) {
  for (int k = 0; k < nz; k++) {
    if (qg1d[k] > r1) {
      double rg = qg1d[k] * rho[k];
      double rb = rg * meters3_to_liters / RHO_G(idx_bg1);
      int idx = imax(1, imin(nint_tie(10.0 * rg / rb) + 1, nrhg));
      double mvd_g = 5.e-3;
      double lamg = (3.0 + mu_g + 0.672) / mvd_g;
      double ng = CGG(2, 1) * ogg3 * rg * pow(lamg, bm_g) / AM_G(idx);
      ng1d[k] = ng / rho[k];
      qb1d[k] = rb / rho[k];
    }
  }
}

/* thermo_vars (main:1263-1310) */
static void thermo_vars(ws_t *w, int *supersaturated) {
  int nz = w->nz;
  *supersaturated = 0;
  for (int k = 0; k < nz; k++) {
    double otemp = 1.0 / w->temp[k];
    double tempc = w->temp[k] - t0;
    w->rhof[k] = sqrt(rho_not / w->rho[k]);
    w->rhof2[k] = sqrt(w->rhof[k]);
    w->qvs[k] = o_calc_rslf(w->pres[k], w->temp[k]);
    w->delqvs[k] = fmax2(0.0, o_calc_rslf(w->pres[k], t0) - w->qv[k]);
    if (tempc <= 0.0)
      w->qvsi[k] = o_calc_rsif(w->pres[k], w->temp[k]);
    else
      w->qvsi[k] = w->qvs[k];
    w->satw[k] = w->qv[k] / w->qvs[k];
    w->sati[k] = w->qv[k] / w->qvsi[k];
    w->ssatw[k] = w->satw[k] - 1.0;
    w->ssati[k] = w->sati[k] - 1.0;
    if (fabs(w->ssatw[k]) < eps) w->ssatw[k] = 0.0;
    if (fabs(w->ssati[k]) < eps) w->ssati[k] = 0.0;
    if (w->ssati[k] > 0.0) *supersaturated = 1;
    w->diffu[k] = 2.11e-5 * pow(w->temp[k] / t0, 1.94) * (101325.0 / w->pres[k]);
    if (tempc >= 0.0)
      w->visco[k] = (1.718 + 0.0049 * tempc) * 1.0e-5;
    else
      w->visco[k] = (1.718 + 0.0049 * tempc - 1.2e-5 * tempc * tempc) * 1.0e-5;
    w->ocp[k] = 1.0 / (cp * (1.0 + 0.887 * w->qv[k]));
    w->vsc2[k] = sqrt(w->rho[k] / w->visco[k]);
    w->lvap[k] = lvap0 + (2106.0 - 4218.0) * tempc;
    w->tcond[k] = (5.69 + 0.0168 * tempc) * 1.0e-5 * 418.936;
    w->lvt2[k] = w->lvap[k] * w->lvap[k] * w->ocp[k] * orv * otemp * otemp;
  }
}

/* check_over_depletion (main:1313-1438) */
static void check_over_depletion(ws_t *w, double odt) {
  int nz = w->nz;
  double *tw = w->tw;
  for (int k = 0; k < nz; k++) {
    double sump, rate_max, ratio;
    sump = TD(PRI_INU) + TD(PRI_IDE) + TD(PRS_IDE) + TD(PRS_SDE) + TD(PRG_GDE) + TD(PRI_IHA);
    rate_max = (w->qv[k] - w->qvsi[k]) * w->rho[k] * odt * 0.999;
    if ((sump > eps && sump > rate_max) || (sump < -eps && sump < rate_max)) {
      TRACE(k, TR_LIMIT, 1 << 0);
      ratio = rate_max / sump;
      TD(PRI_INU) = TD(PRI_INU) * ratio;
      TD(PRI_IDE) = TD(PRI_IDE) * ratio;
      TD(PNI_IDE) = TD(PNI_IDE) * ratio;
      TD(PRS_IDE) = TD(PRS_IDE) * ratio;
      TD(PRS_SDE) = TD(PRS_SDE) * ratio;
      TD(PRG_GDE) = TD(PRG_GDE) * ratio;
      TD(PRI_IHA) = TD(PRI_IHA) * ratio;
    }
    sump = -TD(PRR_WAU) - TD(PRI_WFZ) - TD(PRR_RCW) - TD(PRS_SCW) - TD(PRG_SCW) - TD(PRG_GCW);
    rate_max = -w->rc[k] * odt;
    if (w->l_qc[k]) {
      if (sump < rate_max) {
        TRACE(k, TR_LIMIT, 1 << 1);
        ratio = rate_max / sump;
        TD(PRR_WAU) = TD(PRR_WAU) * ratio;
        TD(PRI_WFZ) = TD(PRI_WFZ) * ratio;
        TD(PRR_RCW) = TD(PRR_RCW) * ratio;
        TD(PRS_SCW) = TD(PRS_SCW) * ratio;
        TD(PRG_SCW) = TD(PRG_SCW) * ratio;
        TD(PRG_GCW) = TD(PRG_GCW) * ratio;
      }
    }
    sump = TD(PRI_IDE) - TD(PRS_IAU) - TD(PRS_SCI) - TD(PRI_RCI);
    rate_max = -w->ri[k] * odt;
    if (w->l_qi[k]) {
      if (sump < rate_max) {
        TRACE(k, TR_LIMIT, 1 << 2);
        ratio = rate_max / sump;
        TD(PRI_IDE) = TD(PRI_IDE) * ratio;
        TD(PRS_IAU) = TD(PRS_IAU) * ratio;
        TD(PRS_SCI) = TD(PRS_SCI) * ratio;
        TD(PRI_RCI) = TD(PRI_RCI) * ratio;
      }
    }
    sump = -TD(PRG_RFZ) - TD(PRI_RFZ) - TD(PRR_RCI) + TD(PRR_RCS) + TD(PRR_RCG);
    rate_max = -w->rr[k] * odt;
    if (w->l_qr[k]) {
      if (sump < rate_max) {
        TRACE(k, TR_LIMIT, 1 << 3);
        ratio = rate_max / sump;
        TD(PRG_RFZ) = TD(PRG_RFZ) * ratio;
        TD(PBG_RFZ) = TD(PBG_RFZ) * ratio;
        TD(PRI_RFZ) = TD(PRI_RFZ) * ratio;
        TD(PRR_RCI) = TD(PRR_RCI) * ratio;
        TD(PRR_RCS) = TD(PRR_RCS) * ratio;
        TD(PRR_RCG) = TD(PRR_RCG) * ratio;
      }
    }
    sump = TD(PRS_SDE) - TD(PRS_IHM) - TD(PRR_SML) + TD(PRS_RCS);
    rate_max = -w->rs[k] * odt;
    if (w->l_qs[k]) {
      if (sump < rate_max) {
        TRACE(k, TR_LIMIT, 1 << 4);
        ratio = rate_max / sump;
        TD(PRS_SDE) = TD(PRS_SDE) * ratio;
        TD(PRS_IHM) = TD(PRS_IHM) * ratio;
        TD(PRR_SML) = TD(PRR_SML) * ratio;
        TD(PRS_RCS) = TD(PRS_RCS) * ratio;
      }
    }
    sump = TD(PRG_GDE) - TD(PRG_IHM) - TD(PRR_GML) + TD(PRG_RCG);
    rate_max = -w->rg[k] * odt;
    if (w->l_qg[k]) {
      if (sump < rate_max) {
        TRACE(k, TR_LIMIT, 1 << 5);
        ratio = rate_max / sump;
        TD(PRG_GDE) = TD(PRG_GDE) * ratio;
        TD(PRG_IHM) = TD(PRG_IHM) * ratio;
        TD(PRR_GML) = TD(PRR_GML) * ratio;
        TD(PRG_RCG) = TD(PRG_RCG) * ratio;
        TD(PBG_RCG) = TD(PBG_RCG) * ratio;
      }
    }
    TD(PRI_IHM) = TD(PRS_IHM) + TD(PRG_IHM);
    ratio = fmin2(fabs(TD(PRR_RCG)), fabs(TD(PRG_RCG)));
    TD(PRR_RCG) = ratio * copysign(1.0, TD(PRR_RCG));
    TD(PRG_RCG) = -TD(PRR_RCG);
    TD(PBG_RCG) = meters3_to_liters * TD(PRG_RCG) / rho_i;
    if (w->temp[k] > t0) {
      ratio = fmin2(fabs(TD(PRR_RCS)), fabs(TD(PRS_RCS)));
      TD(PRR_RCS) = ratio * copysign(1.0, TD(PRR_RCS));
      TD(PRS_RCS) = -TD(PRR_RCS);
    }
  }
}

/* sum_tendencies (main:1441-1513) */
static void sum_tendencies(ws_t *w) {
  int nz = w->nz;
  double *tw = w->tw;
  for (int k = 0; k < nz; k++) {
    double orho = 1. / w->rho[k];
    double lfus2 = lsub - w->lvap[k];
    w->qvten[k] = w->qvten[k] + (-TD(PRI_INU) - TD(PRI_IHA) - TD(PRI_IDE) - TD(PRS_IDE) -
                                 TD(PRS_SDE) - TD(PRG_GDE)) * orho;
    w->qcten[k] = w->qcten[k] + (-TD(PRR_WAU) - TD(PRI_WFZ) - TD(PRR_RCW) - TD(PRS_SCW) -
                                 TD(PRG_SCW) - TD(PRG_GCW)) * orho;
    w->ncten[k] = w->ncten[k] + (-TD(PNC_WAU) - TD(PNC_RCW) - TD(PNI_WFZ) - TD(PNC_SCW) -
                                 TD(PNC_GCW)) * orho;
    w->qiten[k] = w->qiten[k] + (TD(PRI_INU) + TD(PRI_IHA) + TD(PRI_IHM) + TD(PRI_WFZ) +
                                 TD(PRI_RFZ) + TD(PRI_IDE) - TD(PRS_IAU) - TD(PRS_SCI) -
                                 TD(PRI_RCI)) * orho;
    w->niten[k] = w->niten[k] + (TD(PNI_INU) + TD(PNI_IHA) + TD(PNI_IHM) + TD(PNI_WFZ) +
                                 TD(PNI_RFZ) + TD(PNI_IDE) - TD(PNI_IAU) - TD(PNI_SCI) -
                                 TD(PNI_RCI)) * orho;
    w->qrten[k] = w->qrten[k] + (TD(PRR_WAU) + TD(PRR_RCW) + TD(PRR_SML) + TD(PRR_GML) +
                                 TD(PRR_RCS) + TD(PRR_RCG) - TD(PRG_RFZ) - TD(PRI_RFZ) -
                                 TD(PRR_RCI)) * orho;
    w->nrten[k] = w->nrten[k] + (TD(PNR_WAU) + TD(PNR_SML) + TD(PNR_GML) -
                                 (TD(PNR_RFZ) + TD(PNR_RCR) + TD(PNR_RCG) + TD(PNR_RCS) +
                                  TD(PNR_RCI) + TD(PNI_RFZ))) * orho;
    w->qsten[k] = w->qsten[k] + (TD(PRS_IAU) + TD(PRS_SDE) + TD(PRS_SCI) + TD(PRS_SCW) +
                                 TD(PRS_RCS) + TD(PRS_IDE) - TD(PRS_IHM) - TD(PRR_SML)) * orho;
    w->qgten[k] = w->qgten[k] + (TD(PRG_SCW) + TD(PRG_RFZ) + TD(PRG_GDE) + TD(PRG_RCG) +
                                 TD(PRG_GCW) + TD(PRG_RCI) + TD(PRG_RCS) - TD(PRG_IHM) -
                                 TD(PRR_GML)) * orho;
    w->ngten[k] = w->ngten[k] + (TD(PNG_SCW) + TD(PNG_RFZ) - TD(PNG_RCG) + TD(PNG_RCI) +
                                 TD(PNG_RCS) + TD(PNG_GDE) - TD(PNR_GML)) * orho;
    w->qbten[k] = w->qbten[k] + (TD(PBG_SCW) + TD(PBG_RFZ) + TD(PBG_GCW) + TD(PBG_RCI) +
                                 TD(PBG_RCS) + TD(PBG_RCG) + TD(PBG_SML) - TD(PBG_GML) +
                                 meters3_to_liters * (TD(PRG_GDE) - TD(PRG_IHM)) /
                                     RHO_G(w->idx_bg[k])) * orho;
    if (w->temp[k] < t0) {
      w->tten[k] = w->tten[k] +
                   (lsub * w->ocp[k] * (TD(PRI_INU) + TD(PRI_IDE) + TD(PRS_IDE) + TD(PRS_SDE) +
                                        TD(PRG_GDE) + TD(PRI_IHA)) +
                    lfus2 * w->ocp[k] * (TD(PRI_WFZ) + TD(PRI_RFZ) + TD(PRG_RFZ) + TD(PRS_SCW) +
                                         TD(PRG_SCW) + TD(PRG_GCW) + TD(PRG_RCS) + TD(PRS_RCS) +
                                         TD(PRR_RCI) + TD(PRG_RCG))) * orho;
    } else {
      w->tten[k] = w->tten[k] +
                   (lfus * w->ocp[k] * (-TD(PRR_SML) - TD(PRR_GML) - TD(PRR_RCG) - TD(PRR_RCS)) +
                    lsub * w->ocp[k] * (TD(PRS_SDE) + TD(PRG_GDE))) * orho;
    }
  }
}

/* sedimentation (main:1516-1559); ktop is the 1-based ktop_sedi */
static void sedimentation(int nz, double *xr, const double *vt, const double *dz1d,
                          const double *rho, double *xten, double limit, int steps, int ktop,
                          double *precip, double dt, double *sed_r) {
  for (int k = nz - 1; k >= 0; k--) sed_r[k] = vt[k] * xr[k];
  int k = nz - 1;
  double odz = 1.0 / dz1d[k], orho = 1.0 / rho[k];
  xten[k] = xten[k] - sed_r[k] * odz * (1.0 / (double)steps) * orho;
  xr[k] = fmax2(limit, xr[k] - sed_r[k] * odz * dt * (1.0 / (double)steps));
  for (k = ktop - 1; k >= 0; k--) {
    odz = 1.0 / dz1d[k];
    orho = 1.0 / rho[k];
    xten[k] = xten[k] + (sed_r[k + 1] - sed_r[k]) * odz * (1.0 / (double)steps) * orho;
    xr[k] = fmax2(limit, xr[k] + (sed_r[k + 1] - sed_r[k]) * odz * dt * (1.0 / (double)steps));
  }
  if (precip)
    if (xr[0] > low_limit_mass_for_precip) *precip = *precip + sed_r[0] * dt * (1.0 / (double)steps);
}

/* substep reduction of the semi-Lagrangian path (main:595, 636) */
static const double semi_sedi_factor = 10.0;

/* semilagrangian_sedimentation (main:1562-1749): the semi-Lagrangian scheme of Juang and
 * Hong (2010), Mon. Wea. Rev. 138, 1778-1791.  vt holds nz + 1 speeds (vt[nz] = 0).
 * Arrays below keep the reference's 1-based indices through the macros. */
static void semilagrangian_sedimentation(int nz, const double *dz1d, const double *rho, double *xr,
                                         double *xten, const double *vt, int steps, double limit,
                                         double *precip, double dt, double odt) {
  double zi_[nz + 1], wi_[nz + 1], dza_[nz + 1], za_[nz + 2], qa_[nz + 1], qmi_[nz + 1],
      qpi_[nz + 1], rr_save_[nz];
#define ZI(i) zi_[(i) - 1]
#define WI(i) wi_[(i) - 1]
#define DZA(i) dza_[(i) - 1]
#define ZA(i) za_[(i) - 1]
#define QA(i) qa_[(i) - 1]
#define QMI(i) qmi_[(i) - 1]
#define QPI(i) qpi_[(i) - 1]
#define VT(i) vt[(i) - 1]
#define DZ(i) dz1d[(i) - 1]
#define XR(i) xr[(i) - 1]
  const double osteps = 1.0 / (double)steps;
  for (int k = 1; k <= nz + 1; k++) ZI(k) = WI(k) = DZA(k) = QA(k) = QMI(k) = QPI(k) = 0.0;
  for (int k = 1; k <= nz + 2; k++) ZA(k) = 0.0;
  for (int k = 0; k < nz; k++) rr_save_[k] = xr[k];
  ZI(1) = 0.0;
  for (int k = 1; k <= nz; k++) ZI(k + 1) = ZI(k) + DZ(k);
  /* 3rd-order interpolation of the interface speeds (:1599-1611) */
  const double fa1 = 9.0 / 16.0, fa2 = 1.0 / 16.0;
  WI(1) = VT(1);
  WI(2) = 0.5 * (VT(2) + VT(1));
  for (int k = 3; k <= nz - 1; k++) WI(k) = fa1 * (VT(k) + VT(k - 1)) - fa2 * (VT(k + 1) + VT(k - 2));
  WI(nz) = 0.5 * (VT(nz) + VT(nz - 1));
  WI(nz + 1) = VT(nz + 1);
  for (int k = 2; k <= nz; k++)
    if (VT(k) == 0.0) WI(k) = VT(k - 1);
  /* limit of the speed's divergence per substep (:1613-1621) */
  const double con1 = 0.05;
  for (int k = nz; k >= 1; k--) {
    double decfl = (WI(k + 1) - WI(k)) * dt * osteps / DZ(k);
    if (decfl > con1) WI(k) = WI(k + 1) - con1 * DZ(k) * odt * (double)steps;
  }
  /* departure heights of the interfaces and the deformed cells (:1623-1636) */
  for (int k = 1; k <= nz + 1; k++) ZA(k) = ZI(k) - WI(k) * dt * osteps;
  ZA(nz + 2) = ZI(nz + 1);
  for (int k = 1; k <= nz + 1; k++) DZA(k) = ZA(k + 1) - ZA(k);
  for (int k = 1; k <= nz; k++) QA(k) = XR(k) * DZ(k) / DZA(k);
  QA(nz + 1) = 0.0;
  /* interface values with the reference's monotonicity test (:1638-1659) */
  for (int k = 2; k <= nz; k++) {
    double dip = (QA(k + 1) - QA(k)) / (DZA(k + 1) + DZA(k));
    double dim = (QA(k) - QA(k - 1)) / (DZA(k - 1) + DZA(k));
    if (dip * dim <= 0.0) {
      QMI(k) = QA(k);
      QPI(k) = QA(k);
    } else {
      QPI(k) = QA(k) + 0.5 * (dip + dim) * DZA(k);
      QMI(k) = 2.0 * QA(k) - QPI(k);
      if (QPI(k) > 0.0 || QMI(k) < 0.0) {
        QPI(k) = QA(k);
        QMI(k) = QA(k);
      }
    }
  }
  QPI(1) = QA(1);
  QMI(1) = QA(1);
  QMI(nz + 1) = QA(nz + 1);
  QPI(nz + 1) = QA(nz + 1);
  /* remap onto the regular cells (:1661-1723) */
  int kb = 1, kt = 1;
  for (int k = 1; k <= nz; k++) {
    kb = imax(kb - 1, 1);
    kt = imax(kt - 1, 1);
    if (ZI(k) >= ZA(nz + 1)) break;
    for (int kk = kb; kk <= nz; kk++)
      if (ZI(k) <= ZA(kk + 1)) {
        kb = kk;
        break;
      }
    for (int kk = kt; kk <= nz + 2; kk++)
      if (ZI(k + 1) <= ZA(kk)) {
        kt = kk;
        break;
      }
    kt = kt - 1;
    if (kt == kb) {
      double tl = (ZI(k) - ZA(kb)) / DZA(kb);
      double th = (ZI(k + 1) - ZA(kb)) / DZA(kb);
      double tl2 = tl * tl, th2 = th * th;
      double qqd = 0.5 * (QPI(kb) - QMI(kb));
      double qqh = qqd * th2 + QMI(kb) * th;
      double qql = qqd * tl2 + QMI(kb) * tl;
      XR(k) = (qqh - qql) / (th - tl);
    } else if (kt > kb) {
      double tl = (ZI(k) - ZA(kb)) / DZA(kb);
      double tl2 = tl * tl;
      double qqd = 0.5 * (QPI(kb) - QMI(kb));
      double qql = qqd * tl2 + QMI(kb) * tl;
      double dql = QA(kb) - qql;
      double zsum = (1.0 - tl) * DZA(kb);
      double qsum = dql * DZA(kb);
      if (kt - kb > 1)
        for (int m = kb + 1; m <= kt - 1; m++) {
          zsum = zsum + DZA(m);
          qsum = qsum + QA(m) * DZA(m);
        }
      double th = (ZI(k + 1) - ZA(kt)) / DZA(kt);
      double th2 = th * th;
      qqd = 0.5 * (QPI(kt) - QMI(kt));
      double dqh = qqd * th2 + QMI(kt) * th;
      zsum = zsum + th * DZA(kt);
      qsum = qsum + dqh * DZA(kt);
      XR(k) = qsum / zsum;
    }
    double orho = 1.0 / rho[k - 1];
    XR(k) = fmax2(XR(k), limit);
    xten[k - 1] = xten[k - 1] + (XR(k) - rr_save_[k - 1]) * orho * odt;
  }
  /* mass through the surface (:1725-1739) */
  for (int k = 1; k <= nz; k++) {
    if (ZA(k) < 0.0 && ZA(k + 1) <= 0.0) {
      if (precip) *precip = *precip + QA(k) * DZA(k);
    } else if (ZA(k) < 0.0 && ZA(k + 1) > 0.0) {
      double th = (0.0 - ZA(k)) / DZA(k);
      double th2 = th * th;
      double qqd = 0.5 * (QPI(k) - QMI(k));
      double qqh = qqd * th2 + QMI(k) * th;
      if (precip) *precip = *precip + qqh * DZA(k);
      break;
    }
  }
#undef ZI
#undef WI
#undef DZA
#undef ZA
#undef QA
#undef QMI
#undef QPI
#undef VT
#undef DZ
#undef XR
}

/* rain_fallspeed (main:1752-1790); substeps and ktop optional (NULL = absent) */
static void rain_fallspeed(int nz, const double *rhof, const double *rr, const double *ilamr,
                           const double *dz1d, double *vt, double *vtn, int *substeps, int *ktop,
                           double dt) {
  if (ktop) *ktop = 1;
  if (substeps) *substeps = 1;
  for (int k = nz - 1; k >= 0; k--) {
    if (rr[k] > r1) {
      double lamr = 1.0 / ilamr[k];
      vt[k] = rhof[k] * av_r * CRG(6) * org3 * pow(lamr, CRE(3)) * pow(lamr + fv_r, -CRE(6));
      vtn[k] = rhof[k] * av_r * CRG(7) / CRG(12) * pow(lamr, CRE(12)) * pow(lamr + fv_r, -CRE(7));
    } else {
      vt[k] = vt[k + 1];
      vtn[k] = vtn[k + 1];
    }
    if (fmax2(vt[k], vtn[k]) > 1.e-3) {
      if (ktop) *ktop = imax(*ktop, k + 1);
      double dz_by_vt = dz1d[k] / fmax2(vt[k], vtn[k]);
      if (substeps) *substeps = imax(*substeps, int_tie(dt / dz_by_vt + 1.0, *substeps));
    }
  }
  if (ktop && *ktop == nz) *ktop = nz - 1;
}

/* graupel_fallspeed (main:1793-1848); hail_vol = present(qb1d); substeps and ktop optional */
static void graupel_fallspeed(int nz, const double *rhof, const double *rho, const double *visco,
                              const double *rg, const double *rb, int hail_vol, const int *idx,
                              const double *ilamg, const double *dz1d, double *vt, double *vtn,
                              int *substeps, int *ktop, double dt) {
  if (ktop) *ktop = 1;
  if (substeps) *substeps = 1;
  for (int k = nz - 1; k >= 0; k--) {
    if (rg[k] > r1) {
      double afall, bfall;
      if (hail_vol) {
        double dens_g = fmax2(RHO_G(1), fmin2(meters3_to_liters * rg[k] / rb[k], RHO_G(nrhg)));
        afall = a_coeff * pow((4.0 * dens_g * earth_gravity) / (3.0 * rho[k]), b_coeff);
        afall = afall * pow(visco[k], 1.0 - 2.0 * b_coeff);
        bfall = 3.0 * b_coeff - 1.0;
      } else {
        afall = av_g_old;
        bfall = bv_g_old;
      }
      vt[k] = rhof[k] * afall * CGG(6, idx[k]) * ogg3 * pow(ilamg[k], bfall);
      vtn[k] = rhof[k] * afall * CGG(7, idx[k]) / CGG(12, idx[k]) * pow(ilamg[k], bfall);
    } else {
      vt[k] = vt[k + 1];
      vtn[k] = vtn[k + 1];
    }
    if (vt[k] > 1.e-3) {
      if (ktop) *ktop = imax(*ktop, k + 1);
      double dz_by_vt = dz1d[k] / vt[k];
      if (substeps) *substeps = imax(*substeps, int_tie(dt / dz_by_vt + 1.0, *substeps));
    }
  }
  if (ktop && *ktop == nz) *ktop = nz - 1;
}

/* snow_fallspeed (main:1851-1906) */
static void snow_fallspeed(int nz, const double *rhof, const double *rs, const double *prr_sml,
                           const double *smob, const double *smoc, const double *rr,
                           const double *vtrr, const double *dz1d, double *vt,
                           const double *vtboost, int *substeps, int *ktop, double dt) {
  *ktop = 1;
  *substeps = 1;
  for (int k = nz - 1; k >= 0; k--) {
    if (rs[k] > r1) {
      double xds = smoc[k] / smob[k];
      double mrat = 1.0 / xds;
      double ils1 = 1.0 / (mrat * lam0 + fv_s);
      double ils2 = 1.0 / (mrat * lam1 + fv_s);
      double t1_vts = kap0 * CSG(4) * pow(ils1, CSE(4));
      double t2_vts = kap1 * pow(mrat, mu_s) * CSG(10) * pow(ils2, CSE(10));
      ils1 = 1.0 / (mrat * lam0);
      ils2 = 1.0 / (mrat * lam1);
      double t3_vts = kap0 * CSG(1) * pow(ils1, CSE(1));
      double t4_vts = kap1 * pow(mrat, mu_s) * CSG(7) * pow(ils2, CSE(7));
      double vts = rhof[k] * av_s * (t1_vts + t2_vts) / (t3_vts + t4_vts);
      if (prr_sml[k] > 0.0) {
        double sr = rs[k] / (rs[k] + rr[k]);
        vt[k] = vts * sr + (1.0 - sr) * vtrr[k];
      } else {
        vt[k] = vts * vtboost[k];
      }
    } else {
      vt[k] = vt[k + 1];
    }
    if (vt[k] > 1.e-3) {
      *ktop = imax(*ktop, k + 1);
      double dz_by_vt = dz1d[k] / vt[k];
      *substeps = imax(*substeps, int_tie(dt / dz_by_vt + 1.0, *substeps));
    }
  }
  if (*ktop == nz) *ktop = nz - 1;
}

/* ice_fallspeed (main:1909-1942) */
static void ice_fallspeed(int nz, const double *rhof, const double *ri, const double *ilami,
                          const double *dz1d, double *vt, double *vtn, int *substeps, int *ktop,
                          double dt) {
  *ktop = 1;
  *substeps = 1;
  for (int k = nz - 1; k >= 0; k--) {
    if (ri[k] > r1) {
      vt[k] = rhof[k] * av_i * CIG(3) * oig2 * pow(ilami[k], bv_i);
      vtn[k] = rhof[k] * av_i * CIG(6) / CIG(7) * pow(ilami[k], bv_i);
    } else {
      vt[k] = vt[k + 1];
      vtn[k] = vtn[k + 1];
    }
    if (vt[k] > 1.e-3) {
      *ktop = imax(*ktop, k + 1);
      double dz_by_vt = dz1d[k] / vt[k];
      *substeps = imax(*substeps, int_tie(dt / dz_by_vt + 1.0, *substeps));
    }
  }
  if (*ktop == nz) *ktop = nz - 1;
}

/* cloud_fallspeed (main:1945-1977) */
static void cloud_fallspeed(int nz, const double *rhof, const double *w1d, const double *rc,
                            const double *nc, const double *ilamc, const double *dz1d, double *vt,
                            double *vtn, int *ktop) {
  *ktop = 1;
  double hgt = 0.0;
  for (int k = 1; k <= nz - 1; k++) {
    if (rc[k - 1] > r2) *ktop = k;
    hgt = hgt + dz1d[k - 1];
    if (hgt > 500.0) break;
  }
  for (int k = *ktop; k >= 1; k--) {
    int k0 = k - 1;
    if (rc[k0] > r1 && w1d[k0] < 0.1) {
      int nu_c = o_get_nuc(nc[k0]);
      vt[k0] = rhof[k0] * av_c * CCG(5, nu_c) * OCG2(nu_c) * pow(ilamc[k0], bv_c);
      vtn[k0] = rhof[k0] * av_c * CCG(4, nu_c) * OCG1(nu_c) * pow(ilamc[k0], bv_c);
    }
  }
}

/* ------------------------------------------------------------------------------ */
/* table indices (main:2493-2635, 2839-2858)                                        */
/* ------------------------------------------------------------------------------ */
/* decade search shared by the get_*_table_index routines: finds n with
 * 1 <= x/10**n < 10 among nint(log10(x)) + {-1,0,+1}, then the linear bin index. */
static int decade_index(double x, int n2, int nmax) {
  int nx = nint(log10(x)), n = 0;
  for (int nn = nx - 1; nn <= nx + 1; nn++) {
    n = nn;
    if ((x / ipow(10.0, nn)) >= 1.0 && (x / ipow(10.0, nn)) < 10.0) break;
  }
  int idx = (int)(x / ipow(10.0, n)) + 10 * (n - n2) - (n - n2);
  return imax(1, imin(idx, nmax));
}
static void get_snow_table_index(double rs, int *idx_s) { *idx_s = decade_index(rs, nis2, ntb_s); }
static void get_temperature_table_index(double tempk, int *idx_t) {
  double tempc = tempk - t0;
  int it = (int)((tempc - 2.5) / 5.0) - 1;
  it = imax(1, -it);
  *idx_t = imin(it, ntb_t);
}
static void get_rain_table_index(double rr, double ilamr, int *idx_r, int *idx_r1) {
  *idx_r = decade_index(rr, nir2, ntb_r);
  double lamr = 1. / ilamr;
  double lam_exp = lamr * pow(CRG(3) * org2 * org1, bm_r);
  double n0_exp = org1 * rr / am_r * pow(lam_exp, CRE(1));
  *idx_r1 = decade_index(n0_exp, nir3, ntb_r1);
}
static void get_graupel_table_index(double rg, double ilamg, int idx, int *idx_g, int *idx_g1) {
  *idx_g = decade_index(rg, nig2, ntb_g);
  double lamg = 1. / ilamg;
  double lam_exp = lamg * pow(CGG(3, 1) * ogg2 * ogg1, bm_g);
  double n0_exp = ogg1 * rg / AM_G(idx) * pow(lam_exp, CGE(1, 1));
  *idx_g1 = decade_index(n0_exp, nig3, ntb_g1);
}
static void get_cloud_table_index(double rc, double nc, int *idx_c, int *idx_n) {
  *idx_c = decade_index(rc, nic2, ntb_c);
  int in = nint(1.0 + (double)nbc * log(nc / t_nc[0]) / nic1);
  *idx_n = imax(1, imin(in, nbc));
}
static void get_ice_table_index(double ri, double ni, int *idx_i, int *idx_i1) {
  *idx_i = decade_index(ri, nii2, ntb_i);
  *idx_i1 = decade_index(ni, nii3, ntb_i1);
}
static void get_in_table_index(double xni, int *idx_in) {
  if (xni > nt_in[0])
    *idx_in = decade_index(xni, niin2, ntb_in);
  else
    *idx_in = 1;
}

/* ------------------------------------------------------------------------------ */
/* process rates                                                                    */
/* ------------------------------------------------------------------------------ */
/* koop_nucleation (main:2168-2195) */
static double koop_nucleation(double temp, double satw, double naero, double dt) {
  double xni = 0.0;
  double mu_diff = 210368.0 + (131.438 * temp) - (3.32373e6 / temp) - (41729.1 * log(temp));
  double a_w_i = exp(mu_diff / (r_uni * temp));
  double delta_aw = satw - a_w_i;
  double log_j_rate = -906.7 + (8502.0 * delta_aw) - (26924.0 * delta_aw * delta_aw) +
                      (29180.0 * delta_aw * delta_aw * delta_aw);
  log_j_rate = fmin2(20.0, log_j_rate);
  double j_rate = pow(10.0, log_j_rate);
  double prob_h = fmin2(1.0 - exp(-j_rate * ar_volume * dt), 1.0);
  if (prob_h > 0.0) xni = fmin2(prob_h * naero, 1000.e3);
  return fmax2(0.0, xni);
}

/* activate_cloud_number (main:2198-2276), land absent */
static double activate_cloud_number(double temp, double w1d, double nwfa) {
  double n_local = nwfa * 1.e-6;
  if (n_local >= ta_na[ntb_arc - 1])
    n_local = ta_na[ntb_arc - 1] - 1.0;
  else if (n_local <= ta_na[0])
    n_local = ta_na[0] + 1.0;
  int n;
  for (n = 2; n <= ntb_arc; n++)
    if (n_local >= ta_na[n - 2] && n_local < ta_na[n - 1]) break;
  int i = n;
  double x1 = log(ta_na[i - 2]), x2 = log(ta_na[i - 1]);
  double w_local = w1d;
  if (w_local >= ta_ww[ntb_arw - 1])
    w_local = ta_ww[ntb_arw - 1] - 1.0;
  else if (w_local <= ta_ww[0])
    w_local = ta_ww[0] + 0.001;
  for (n = 2; n <= ntb_arw; n++)
    if (w_local >= ta_ww[n - 2] && w_local < ta_ww[n - 1]) break;
  int j = n;
  double y1 = log(ta_ww[j - 2]), y2 = log(ta_ww[j - 1]);
  int k = imax(1, imin(nint((temp - ta_tk[0]) * 0.1) + 1, ntb_art));
  int l = 3, m = 2;
  double lower_lim_nuc_frac = 0.;
  double a = TNCCN(i - 1, j - 1, k, l, m);
  double b = TNCCN(i, j - 1, k, l, m);
  double c = TNCCN(i, j, k, l, m);
  double d = TNCCN(i - 1, j, k, l, m);
  double nx = log(n_local), wy = log(w_local);
  double t = (nx - x1) / (x2 - x1), u = (wy - y1) / (y2 - y1);
  double fraction = (1.0 - t) * (1.0 - u) * a + t * (1.0 - u) * b + t * u * c + (1.0 - t) * u * d;
  fraction = fmax2(fraction, lower_lim_nuc_frac);
  return nwfa * fraction;
}

/* warm_rain (main:2279-2355) */
static void warm_rain(ws_t *w, double odt) {
  int nz = w->nz;
  double *tw = w->tw;
  for (int k = 0; k < nz; k++) {
    if (w->l_qr[k]) {
      if (w->mvd_r[k] > d0r) {
        TRACE(k, TR_RW, 1 << 16);
        double ef_rr = fmax2(-0.1, 1.0 - exp(2300.0 * (w->mvd_r[k] - 1950.0e-6)));
        TD(PNR_RCR) = ef_rr * 2.0 * w->nr[k] * w->rr[k];
      }
    }
    if (w->l_qc[k]) {
      if (w->rc[k] > 0.01e-3) {
        TRACE(k, TR_RW, 1 << 17);
        int nu_c = o_get_nuc(w->nc[k]);
        double lamc = 1.0 / w->ilamc[k];
        double xdc = fmax2(d0c * 1.e6, (pow(w->rc[k] / (am_r * w->nc[k]), obmr)) * 1.e6);
        double dc_g = (pow(CCG(3, nu_c) * OCG2(nu_c), obmr) / lamc) * 1.e6;
        double dc_b = pow(xdc * xdc * xdc * dc_g * dc_g * dc_g - xdc * xdc * xdc * xdc * xdc * xdc,
                          1.0 / 6.0);
        double zeta1 = 0.5 * ((6.25e-6 * xdc * dc_b * dc_b * dc_b - 0.4) +
                              fabs(6.25e-6 * xdc * dc_b * dc_b * dc_b - 0.4));
        double zeta = 0.027 * w->rc[k] * zeta1;
        double taud = 0.5 * ((0.5 * dc_b - 7.5) + fabs(0.5 * dc_b - 7.5)) + r1;
        double tau = 3.72 / (w->rc[k] * taud);
        TD(PRR_WAU) = zeta / tau;
        TD(PRR_WAU) = fmin2(w->rc[k] * odt, TD(PRR_WAU));
        TD(PNR_WAU) = TD(PRR_WAU) / (am_r * nu_c * autocon_nr_factor * d0r * d0r * d0r);
        TD(PNC_WAU) = fmin2(w->nc[k] * odt, TD(PRR_WAU) / (am_r * w->mvd_c[k] * w->mvd_c[k] * w->mvd_c[k]));
      }
    }
    if (w->l_qr[k] && w->l_qc[k]) {
      if (w->mvd_r[k] > d0r && w->mvd_c[k] > d0c) {
        double lamr = (3.0 + mu_r + 0.672) / w->mvd_r[k];
        int idx = 1 + (int)(nbr * log(w->mvd_r[k] / dr[0]) / log(dr[nbr - 1] / dr[0]));
        idx = imin(idx, nbr);
        TRACE(k, TR_RW, idx | ((int)(w->mvd_c[k] * 1.e6) << 8) | (1 << 18));
        double ef_rw = T_EFRW(idx, (int)(w->mvd_c[k] * 1.e6));
        double n0_r = w->nr[k] * org2 * pow(lamr, CRE(2));
        TD(PRR_RCW) = w->rhof[k] * t1_qr_qc * ef_rw * w->rc[k] * n0_r * pow(lamr + fv_r, -CRE(9));
        TD(PRR_RCW) = fmin2(w->rc[k] * odt, TD(PRR_RCW));
        TD(PNC_RCW) = w->rhof[k] * t1_qr_qc * ef_rw * w->nc[k] * n0_r * pow(lamr + fv_r, -CRE(9));
        TD(PNC_RCW) = fmin2(w->nc[k] * odt, TD(PNC_RCW));
      }
    }
  }
}

/* riming (main:2358-2490) */
static void riming(ws_t *w, double odt) {
  int nz = w->nz;
  double *tw = w->tw;
  for (int k = 0; k < nz; k++) {
    double tempc = w->temp[k] - t0;
    w->vtboost[k] = 1.0;
    if (w->l_qc[k] && w->l_qs[k]) {
      double xds = w->smoc[k] / w->smob[k];
      if ((w->mvd_c[k] > d0c) && (xds > d0s)) {
        int idxs = 1 + (int)(nbs * log(xds / ds[0]) / log(ds[nbs - 1] / ds[0]));
        idxs = imin(idxs, nbs);
        TRACE(k, TR_RIME, idxs | ((int)(w->mvd_c[k] * 1.e6) << 8) | (1 << 16));
        double ef_sw = T_EFSW(idxs, (int)(w->mvd_c[k] * 1.e6));
        TD(PRS_SCW) = w->rhof[k] * t1_qs_qc * ef_sw * w->rc[k] * w->smoe[k];
        TD(PRS_SCW) = fmin2(w->rc[k] * odt, TD(PRS_SCW));
        TD(PNC_SCW) = w->rhof[k] * t1_qs_qc * ef_sw * w->nc[k] * w->smoe[k];
        TD(PNC_SCW) = fmin2(w->nc[k] * odt, TD(PNC_SCW));
        if (w->temp[k] < t0) {
          if (TD(PRS_SCW) > rime_threshold * TD(PRS_SDE) && TD(PRS_SDE) > eps) {
            double r_frac = fmin2(30.0, TD(PRS_SCW) / TD(PRS_SDE));
            double g_frac = fmin2(rime_conversion, 0.15 + (r_frac - 2.0) * .028);
            w->vtboost[k] = fmin2(1.5, 1.1 + (r_frac - 2.) * .014);
            TD(PRG_SCW) = g_frac * TD(PRS_SCW);
            TD(PNG_SCW) = TD(PRG_SCW) * w->smo0[k] / w->rs[k];
            double vts = av_s * pow(xds, bv_s) * exp(-fv_s * xds);
            double const_ri = -1.0 * (w->mvd_c[k] * 0.5e6) * vts / fmin2(-0.1, tempc);
            const_ri = fmax2(0.1, fmin2(const_ri, 10.0));
            double rime_dens = (0.051 + 0.114 * const_ri - 0.0055 * const_ri * const_ri) * 1000.0;
            if (rime_dens < 150.0) {
              g_frac = 0.0;
              TD(PRG_SCW) = 0.0;
              TD(PNG_SCW) = 0.0;
            }
            double snow_dens_frac =
                fmin2(1.0, fmax2(0.0, w->rs[k] * odt / (w->rs[k] * odt + TD(PRG_SCW))));
            TD(PBG_SCW) = meters3_to_liters * TD(PRG_SCW) /
                          (rho_s * snow_dens_frac + rime_dens * (1.0 - snow_dens_frac));
            TD(PRS_SCW) = (1.0 - g_frac) * TD(PRS_SCW);
          }
        }
      }
    }
    if (w->l_qc[k] && w->l_qg[k]) {
      if (w->rg[k] >= r_g[0] && w->mvd_c[k] > d0c) {
        int ig = w->idx_bg[k];
        double xdg = (bm_g + mu_g + 1.0) * w->ilamg[k];
        double vtg = w->rhof[k] * AV_G(ig) * CGG(6, ig) * ogg3 * pow(w->ilamg[k], BV_G(ig));
        double stoke_g = w->mvd_c[k] * w->mvd_c[k] * vtg * rho_w / (9.0 * w->visco[k] * xdg);
        double const_ri = -1.0 * (w->mvd_c[k] * 0.5e6) * vtg / fmin2(-0.1, tempc);
        const_ri = fmax2(0.1, fmin2(const_ri, 10.0));
        double rime_dens = (0.051 + 0.114 * const_ri - 0.0055 * const_ri * const_ri) * 1000.0;
        if (xdg > d0g) {
          double ef_gw = 0.0;
          if (stoke_g >= 0.4 && stoke_g <= 10.0)
            ef_gw = 0.55 * log10(2.51 * stoke_g);
          else if (stoke_g < 0.4)
            ef_gw = 0.0;
          else if (stoke_g > 10.0)
            ef_gw = 0.77;
          if (w->temp[k] > t0) ef_gw = ef_gw * 0.1;
          double t1_qg_qc = pi * .25 * AV_G(ig) * CGG(9, ig);
          double n0_g = w->ng[k] * ogg2 * pow(1.0 / w->ilamg[k], CGE(2, 1));
          TD(PRG_GCW) = w->rhof[k] * t1_qg_qc * ef_gw * w->rc[k] * n0_g * pow(w->ilamg[k], CGE(9, ig));
          TD(PNC_GCW) = w->rhof[k] * t1_qg_qc * ef_gw * w->nc[k] * n0_g * pow(w->ilamg[k], CGE(9, ig));
          TD(PNC_GCW) = fmin2(w->nc[k] * odt, TD(PNC_GCW));
          if (w->temp[k] < t0) TD(PBG_GCW) = meters3_to_liters * TD(PRG_GCW) / rime_dens;
          if (w->temp[k] < t0) {
            if (TD(PRG_GCW) > eps && tempc > -8.0) {
              double tf = 0.0;
              if (tempc >= -5.0 && tempc < -3.0)
                tf = 0.5 * (-3.0 - tempc);
              else if (tempc > -8.0 && tempc < -5.0)
                tf = 0.33333333 * (8.0 + tempc);
              TD(PNI_IHM) = 3.5e8 * tf * TD(PRG_GCW);
              TD(PRI_IHM) = xm0i * TD(PNI_IHM);
              TD(PRS_IHM) = TD(PRS_SCW) / (TD(PRS_SCW) + TD(PRG_GCW)) * TD(PRI_IHM);
              TD(PRG_IHM) = TD(PRG_GCW) / (TD(PRS_SCW) + TD(PRG_GCW)) * TD(PRI_IHM);
            }
          }
        }
      }
    }
  }
}

/* rain_snow_rain_graupel (main:2638-2727) */
static void rain_snow_rain_graupel(ws_t *w, double odt) {
  int nz = w->nz;
  double *tw = w->tw;
  for (int k = 0; k < nz; k++) {
    int idx_r, idx_r1, idx_s, idx_t, idx_g, idx_g1;
    if (w->l_qr[k] && w->l_qs[k]) {
      if (w->rr[k] >= r_r[0] && w->rs[k] >= r_s[0]) {
        get_temperature_table_index(w->temp[k], &idx_t);
        get_rain_table_index(w->rr[k], w->ilamr[k], &idx_r, &idx_r1);
        get_snow_table_index(w->rs[k], &idx_s);
        TRACE(k, TR_RS, idx_s | (idx_t << 6) | (idx_r1 << 12) | (idx_r << 18) | (1 << 24));
#define QSV(a) QS4(a, idx_s, idx_t, idx_r1, idx_r)
        if (w->temp[k] < t0) {
          TD(PRR_RCS) = -(QSV(tmr_racs2) + QSV(tcr_sacr2) + QSV(tmr_racs1) + QSV(tcr_sacr1));
          TD(PRS_RCS) = QSV(tmr_racs2) + QSV(tcr_sacr2) - QSV(tcs_racs1) - QSV(tms_sacr1);
          TD(PRG_RCS) = QSV(tmr_racs1) + QSV(tcr_sacr1) + QSV(tcs_racs1) + QSV(tms_sacr1);
          TD(PRR_RCS) = fmax2(-w->rr[k] * odt, TD(PRR_RCS));
          TD(PRS_RCS) = fmax2(-w->rs[k] * odt, TD(PRS_RCS));
          TD(PRG_RCS) = fmin2((w->rr[k] + w->rs[k]) * odt, TD(PRG_RCS));
          TD(PNR_RCS) = QSV(tnr_racs1) + QSV(tnr_racs2) + QSV(tnr_sacr1) + QSV(tnr_sacr2);
          TD(PNR_RCS) = fmin2(w->nr[k] * odt, TD(PNR_RCS));
          TD(PNG_RCS) = TD(PNR_RCS);
          TD(PBG_RCS) = meters3_to_liters * TD(PRG_RCS) / rho_i;
        } else {
          TD(PRS_RCS) = -QSV(tcs_racs1) - QSV(tms_sacr1) + QSV(tmr_racs2) + QSV(tcr_sacr2);
          TD(PRS_RCS) = fmax2(-w->rs[k] * odt, TD(PRS_RCS));
          TD(PRR_RCS) = -TD(PRS_RCS);
        }
#undef QSV
      }
    }
    if (w->l_qr[k] && w->l_qg[k]) {
      if (w->rr[k] >= r_r[0] && w->rg[k] >= r_g[0]) {
        int ig = w->idx_bg[k];
        get_temperature_table_index(w->temp[k], &idx_t);
        get_rain_table_index(w->rr[k], w->ilamr[k], &idx_r, &idx_r1);
        get_graupel_table_index(w->rg[k], w->ilamg[k], ig, &idx_g, &idx_g1);
        TRACE(k, TR_RG, idx_g1 | (idx_g << 6) | (idx_r1 << 12) | (idx_r << 18) | (1 << 24));
#define QGV(a) QG5(a, idx_g1, idx_g, ig, idx_r1, idx_r)
        if (w->temp[k] < t0) {
          TD(PRG_RCG) = QGV(tmr_racg) + QGV(tcr_gacr);
          TD(PRG_RCG) = fmin2(w->rr[k] * odt, TD(PRG_RCG));
          TD(PRR_RCG) = -TD(PRG_RCG);
          TD(PNR_RCG) = QGV(tnr_racg) + QGV(tnr_gacr);
          TD(PNR_RCG) = fmin2(w->nr[k] * odt, TD(PNR_RCG));
          TD(PBG_RCG) = meters3_to_liters * TD(PRG_RCG) / rho_i;
        } else {
          TD(PRR_RCG) = QGV(tcg_racg);
          TD(PRR_RCG) = fmin2(w->rg[k] * odt, TD(PRR_RCG));
          TD(PRG_RCG) = -TD(PRR_RCG);
          TD(PNG_RCG) = QGV(tnr_racg);
          TD(PNG_RCG) = fmin2(w->ng[k] * odt, TD(PNG_RCG));
          TD(PBG_RCG) = meters3_to_liters * TD(PRG_RCG) / RHO_G(ig);
          TD(PNR_RCG) = -1.5 * QGV(tnr_gacr);
        }
#undef QGV
      }
    }
  }
}

/* demott_nucleation (main:2823-2836) */
static double demott_nucleation(double tempc, double rho, double nifa) {
  double nifa_cc = fmax2(0.5, nifa * rho_not0 * 1.e-6 / rho);
  double xni = (5.94e-5 * pow(-tempc, 3.33)) * (pow(nifa_cc, (-0.0264 * (tempc)) + 0.0033));
  xni = xni * rho / rho_not0 * 1000.0;
  return fmax2(0.0, xni);
}

/* ice_nucleation (main:2730-2820) */
static void ice_nucleation(ws_t *w, const double *w1d, const double *nwfa1d, const double *nifa1d,
                           double dt, double odt) {
  int nz = w->nz;
  double *tw = w->tw;
  for (int k = 0; k < nz; k++) {
    if (w->temp[k] < t0) {
      double tempc = w->temp[k] - t0;
      int idx_tc = imax(1, imin(nint(-tempc), 45));
      double rate_max = (w->qv[k] - w->qvsi[k]) * w->rho[k] * odt * 0.999;
      double xni, xnc;
      int idx_in, idx_r, idx_r1, idx_c, idx_n;
      if (nifa1d)
        xni = demott_nucleation(tempc, w->rho[k], w->nifa[k]);
      else
        xni = 1.0 * 1000.0;
      get_in_table_index(xni, &idx_in);
      if (w->rr[k] > r_r[0]) {
        get_rain_table_index(w->rr[k], w->ilamr[k], &idx_r, &idx_r1);
        TRACE(k, TR_FZR, idx_r | (idx_r1 << 6) | (idx_tc << 12) | (idx_in << 18) | (1 << 24));
        TD(PRG_RFZ) = QRFZ(tpg_qrfz, idx_r, idx_r1, idx_tc, idx_in) * odt;
        TD(PRI_RFZ) = QRFZ(tpi_qrfz, idx_r, idx_r1, idx_tc, idx_in) * odt;
        TD(PNI_RFZ) = QRFZ(tni_qrfz, idx_r, idx_r1, idx_tc, idx_in) * odt;
        TD(PNR_RFZ) = QRFZ(tnr_qrfz, idx_r, idx_r1, idx_tc, idx_in) * odt;
        TD(PRG_RFZ) = fmin2(w->rr[k] * odt, TD(PRG_RFZ));
        TD(PNR_RFZ) = fmin2(w->nr[k] * odt, TD(PNR_RFZ));
        TD(PNG_RFZ) = TD(PNR_RFZ) * fmax2(fmin2((pow(10.0, -0.1 * w1d[k]) + 0.1), 1.0), 0.1);
      } else if (w->rr[k] > r1 && w->temp[k] < hgfrz) {
        TRACE(k, TR_FZR, 1 << 25);
        TD(PRI_RFZ) = w->rr[k] * odt;
        TD(PNI_RFZ) = w->nr[k] * odt;
      }
      TD(PBG_RFZ) = meters3_to_liters * TD(PRG_RFZ) / rho_i;
      if (w->rc[k] > r_c[0]) {
        get_cloud_table_index(w->rc[k], w->nc[k], &idx_c, &idx_n);
        TRACE(k, TR_FZC, idx_c | (idx_n << 8) | (1 << 16));
        TD(PRI_WFZ) = QCFZ(tpi_qcfz, idx_c, idx_n, idx_tc, idx_in) * odt;
        TD(PRI_WFZ) = fmin2(w->rc[k] * odt, TD(PRI_WFZ));
        TD(PNI_WFZ) = QCFZ(tni_qcfz, idx_c, idx_n, idx_tc, idx_in) * odt;
        TD(PNI_WFZ) = fmin3(w->nc[k] * odt, TD(PRI_WFZ) / (2.0 * xm0i), TD(PNI_WFZ));
      } else if (w->rc[k] > r1 && w->temp[k] < hgfrz) {
        TRACE(k, TR_FZC, 1 << 17);
        TD(PRI_WFZ) = w->rc[k] * odt;
        TD(PNI_WFZ) = w->nc[k] * odt;
      }
      if ((w->ssati[k] >= demott_nuc_ssati) || (w->ssatw[k] > eps && tempc < demott_nuc_tempc)) {
        if (nifa1d)
          xnc = demott_nucleation(tempc, w->rho[k], w->nifa[k]);
        else
          xnc = fmin2(icenuc_max, tno * exp(ato * (t0 - w->temp[k])));
        xni = w->ni[k] + (TD(PNI_RFZ) + TD(PNI_WFZ)) * dt;
        TD(PNI_INU) = 0.5 * (xnc - xni + fabs(xnc - xni)) * odt;
        TD(PRI_INU) = fmin2(rate_max, xm0i * TD(PNI_INU));
        TD(PNI_INU) = TD(PRI_INU) / xm0i;
      }
      xni = w->smo0[k] + w->ni[k] + (TD(PNI_RFZ) + TD(PNI_WFZ) + TD(PNI_INU)) * dt;
      if (nwfa1d) {
        if ((xni <= max_ni) && (w->temp[k] < 238.0) && (w->ssati[k] >= 0.4)) {
          xnc = koop_nucleation(w->temp[k], w->ssatw[k], w->nwfa[k], dt);
          TD(PNI_IHA) = xnc * odt;
          TD(PRI_IHA) = fmin2(rate_max, xm0i * 0.1 * TD(PNI_IHA));
          TD(PNI_IHA) = TD(PRI_IHA) / (xm0i * 0.1);
        }
      }
    }
  }
}

/* get_t1_subl (main:2861-2888) */
static void get_t1_subl(ws_t *w) {
  int nz = w->nz;
  for (int k = 0; k < nz; k++) {
    double otemp = 1.0 / w->temp[k];
    double rvs = w->rho[k] * w->qvsi[k];
    double rvs_p = rvs * otemp * (lsub * otemp * orv - 1.0);
    double rvs_pp = rvs * (otemp * (lsub * otemp * orv - 1.0) * otemp * (lsub * otemp * orv - 1.0) +
                           (-2. * lsub * otemp * otemp * otemp * orv) + otemp * otemp);
    double gamsc = lsub * w->diffu[k] / w->tcond[k] * rvs_p;
    double alphsc = 0.5 * (gamsc / (1.0 + gamsc)) * (gamsc / (1.0 + gamsc)) * rvs_pp / rvs_p * rvs / rvs_p;
    alphsc = fmax2(1.e-9, alphsc);
    double xsat = w->ssati[k];
    if (fabs(xsat) < 1.e-9) xsat = 0.0;
    w->t1_subl[k] = 4.0 * pi *
                    (1.0 - alphsc * xsat + 2.0 * alphsc * alphsc * xsat * xsat -
                     5.0 * alphsc * alphsc * alphsc * xsat * xsat * xsat) /
                    (1.0 + gamsc);
  }
}

/* ice_processes (main:2891-3018) */
static void ice_processes(ws_t *w, const double *w1d, double odt) {
  int nz = w->nz;
  double *tw = w->tw;
  get_t1_subl(w);
  for (int k = 0; k < nz; k++) {
    double rvs = w->rho[k] * w->qvsi[k];
    double rate_max = (w->qv[k] - w->qvsi[k]) * w->rho[k] * odt * 0.999;
    if (w->temp[k] < t0) {
      if (w->l_qi[k]) {
        int idx_i, idx_i1;
        get_ice_table_index(w->ri[k], w->ni[k], &idx_i, &idx_i1);
        TRACE(k, TR_ICE, idx_i | (idx_i1 << 8) | (1 << 16));
        double xdi = fmax2(d0i, (bm_i + mu_i + 1.) * w->ilami[k]);
        double xmi = am_i * pow(xdi, bm_i);
        double oxmi = 1.0 / xmi;
        TD(PRI_IDE) = c_cube * w->t1_subl[k] * w->diffu[k] * w->ssati[k] * rvs * oig1 * CIG(5) *
                      w->ni[k] * w->ilami[k];
        if (TD(PRI_IDE) < 0.0) {
          TD(PRI_IDE) = fmax3(-w->ri[k] * odt, TD(PRI_IDE), rate_max);
          TD(PNI_IDE) = TD(PRI_IDE) * oxmi;
          TD(PNI_IDE) = fmax2(-w->ni[k] * odt, TD(PNI_IDE));
        } else {
          TD(PRI_IDE) = fmin2(TD(PRI_IDE), rate_max);
          TD(PRS_IDE) = (1.0 - IAUS(tpi_ide, idx_i, idx_i1)) * TD(PRI_IDE);
          TD(PRI_IDE) = IAUS(tpi_ide, idx_i, idx_i1) * TD(PRI_IDE);
        }
        if ((idx_i == ntb_i) || (xdi > 5.0 * d0s)) {
          TD(PRS_IAU) = w->ri[k] * .99 * odt;
          TD(PNI_IAU) = w->ni[k] * .95 * odt;
        } else if (xdi < 0.1 * d0s) {
          TD(PRS_IAU) = 0.0;
          TD(PNI_IAU) = 0.0;
        } else {
          TD(PRS_IAU) = IAUS(tps_iaus, idx_i, idx_i1) * odt;
          TD(PRS_IAU) = fmin2(w->ri[k] * .99 * odt, TD(PRS_IAU));
          TD(PNI_IAU) = IAUS(tni_iaus, idx_i, idx_i1) * odt;
          TD(PNI_IAU) = fmin2(w->ni[k] * .95 * odt, TD(PNI_IAU));
        }
        double lami = pow(am_i * CIG(2) * oig1 * w->ni[k] / w->ri[k], obmi);
        (void)lami;
        xdi = fmax2(d0i, (bm_i + mu_i + 1.) * w->ilami[k]);
        xmi = am_i * pow(xdi, bm_i);
        oxmi = 1. / xmi;
        if (w->rs[k] >= r_s[0]) {
          TD(PRS_SCI) = t1_qs_qi * w->rhof[k] * ef_si * w->ri[k] * w->smoe[k];
          TD(PNI_SCI) = TD(PRS_SCI) * oxmi;
        }
        if (w->rr[k] >= r_r[0] && w->mvd_r[k] > 4.0 * xdi) {
          double lamr = 1.0 / w->ilamr[k];
          double n0_r = w->nr[k] * org2 * pow(lamr, CRE(2));
          TD(PRI_RCI) = w->rhof[k] * t1_qr_qi * ef_ri * w->ri[k] * n0_r * pow(lamr + fv_r, -CRE(9));
          TD(PNR_RCI) = w->rhof[k] * t1_qr_qi * ef_ri * w->ni[k] * n0_r * pow(lamr + fv_r, -CRE(9));
          TD(PNR_RCI) = fmin2(w->nr[k] * odt, TD(PNR_RCI));
          TD(PNG_RCI) = TD(PNR_RCI) * fmax2(fmin2((pow(10.0, -0.1 * w1d[k]) + 0.1), 1.0), 0.1);
          TD(PNI_RCI) = TD(PRI_RCI) * oxmi;
          TD(PRR_RCI) = w->rhof[k] * t2_qr_qi * ef_ri * w->ni[k] * n0_r * pow(lamr + fv_r, -CRE(8));
          TD(PRR_RCI) = fmin2(w->rr[k] * odt, TD(PRR_RCI));
          TD(PRG_RCI) = TD(PRI_RCI) + TD(PRR_RCI);
          TD(PBG_RCI) = TD(PRG_RCI) / rho_i;
        }
      }
      if (w->l_qs[k]) {
        double c_snow = c_sqrd + (w->temp[k] - t0 + 1.5) * (c_cube - c_sqrd) / (-30.0 + 1.5);
        c_snow = fmax2(c_sqrd, fmin2(c_snow, c_cube));
        TD(PRS_SDE) = c_snow * w->t1_subl[k] * w->diffu[k] * w->ssati[k] * rvs *
                      (t1_qs_sd * w->smo1[k] + t2_qs_sd * w->rhof2[k] * w->vsc2[k] * w->smof[k]);
        if (TD(PRS_SDE) < 0.0)
          TD(PRS_SDE) = fmax3(-w->rs[k] * odt, TD(PRS_SDE), rate_max);
        else
          TD(PRS_SDE) = fmin2(TD(PRS_SDE), rate_max);
      }
      if (w->l_qg[k]) {
        if (w->ssati[k] < -eps) {
          int ig = w->idx_bg[k];
          double n0_g = w->ng[k] * ogg2 * pow(1.0 / w->ilamg[k], CGE(2, 1));
          double t2_qg_sd = 0.28 * sc3 * sqrt(AV_G(ig)) * CGG(11, ig);
          TD(PRG_GDE) = c_cube * w->t1_subl[k] * w->diffu[k] * w->ssati[k] * rvs * n0_g *
                        (t1_qg_sd * pow(w->ilamg[k], CGE(10, 1)) +
                         t2_qg_sd * w->vsc2[k] * w->rhof2[k] * pow(w->ilamg[k], CGE(11, ig)));
          if (TD(PRG_GDE) < 0.0) {
            TD(PRG_GDE) = fmax3(-w->rg[k] * odt, TD(PRG_GDE), rate_max);
            TD(PNG_GDE) = TD(PRG_GDE) * w->ng[k] / w->rg[k];
          } else {
            TD(PRG_GDE) = fmin2(TD(PRG_GDE), rate_max);
          }
        }
      }
    }
  }
}

/* melting (main:3021-3119) */
static void melting(ws_t *w, double dt, double odt) {
  int nz = w->nz;
  double *tw = w->tw;
  get_t1_subl(w);
  for (int k = 0; k < nz; k++) {
    double tempc = w->temp[k] - t0;
    double rvs = w->rho[k] * w->qvsi[k];
    if (w->temp[k] > t0) {
      if (w->l_qs[k]) {
        TD(PRR_SML) = (tempc * w->tcond[k] - lvap0 * w->diffu[k] * w->delqvs[k]) *
                      (t1_qs_me * w->smo1[k] + t2_qs_me * w->rhof2[k] * w->vsc2[k] * w->smof[k]);
        if (TD(PRR_SML) > 0.0) {
          TD(PRR_SML) = TD(PRR_SML) + 4218.0 * olfus * tempc * (TD(PRR_RCS) + TD(PRS_SCW));
          TD(PRR_SML) = fmin2(w->rs[k] * odt, fmax2(0.0, TD(PRR_SML)));
          TD(PNR_SML) = w->smo0[k] / w->rs[k] * TD(PRR_SML) * pow(10.0, -0.25 * tempc);
          TD(PNR_SML) = fmin2(w->smo0[k] * odt, TD(PNR_SML));
        } else {
          TD(PRR_SML) = 0.0;
          TD(PNR_SML) = 0.0;
          if (w->ssati[k] < 0.0) {
            TD(PRS_SDE) = c_cube * w->t1_subl[k] * w->diffu[k] * w->ssati[k] * rvs *
                          (t1_qs_sd * w->smo1[k] + t2_qs_sd * w->rhof2[k] * w->vsc2[k] * w->smof[k]);
            TD(PRS_SDE) = fmax2(-w->rs[k] * odt, TD(PRS_SDE));
          }
        }
      }
      if (w->l_qg[k]) {
        int ig = w->idx_bg[k];
        double n0_g = w->ng[k] * ogg2 * pow(1.0 / w->ilamg[k], CGE(2, 1));
        double n0_melt = w->ng[k] * ogg2 * pow(1.0 / w->ilamg[k], CGE(2, 1));
        if ((w->rg[k] * w->ng[k]) < 1.e-4) {
          double lamg = 1. / w->ilamg[k];
          n0_melt = (1.e-4 / w->rg[k]) * ogg2 * pow(lamg, CGE(2, 1));
        }
        double t2_qg_me = pi * 4.0 * c_cube * olfus * 0.28 * sc3 * sqrt(AV_G(ig)) * CGG(11, ig);
        TD(PRR_GML) = (tempc * w->tcond[k] - lvap0 * w->diffu[k] * w->delqvs[k]) * n0_melt *
                      (t1_qg_me * pow(w->ilamg[k], CGE(10, 1)) +
                       t2_qg_me * w->rhof2[k] * w->vsc2[k] * pow(w->ilamg[k], CGE(11, ig)));
        TD(PRR_GML) = fmin2(w->rg[k] * odt, fmax2(0.0, TD(PRR_GML)));
        if (TD(PRR_GML) > 0.0) {
          double melt_f = fmax2(0.05, fmin2(TD(PRR_GML) * dt / w->rg[k], 1.0));
          TD(PBG_GML) = meters3_to_liters * TD(PRR_GML) /
                        fmax2(fmin2(melt_f * RHO_G(ig), rho_w), 50.0);
          TD(PNR_GML) = TD(PRR_GML) * w->ng[k] / w->rg[k] * pow(10.0, -0.33 * (w->temp[k] - t0));
        } else {
          TD(PRR_GML) = 0.0;
          TD(PNR_GML) = 0.0;
          TD(PBG_GML) = 0.0;
          if (w->ssati[k] < 0.0) {
            double t2_qg_sd = 0.28 * sc3 * sqrt(AV_G(ig)) * CGG(11, ig);
            TD(PRG_GDE) = c_cube * w->t1_subl[k] * w->diffu[k] * w->ssati[k] * rvs * n0_g *
                          (t1_qg_sd * pow(w->ilamg[k], CGE(10, 1)) +
                           t2_qg_sd * w->vsc2[k] * w->rhof2[k] * pow(w->ilamg[k], CGE(11, ig)));
            TD(PRG_GDE) = fmax2(-w->rg[k] * odt, TD(PRG_GDE));
            TD(PNG_GDE) = TD(PRG_GDE) * w->ng[k] / w->rg[k];
          }
        }
      }
      if (dt > timestep_conversion_rime_to_rain) {
        TD(PRR_RCW) = TD(PRR_RCW) + TD(PRS_SCW) + TD(PRG_GCW);
        TD(PRS_SCW) = 0.0;
        TD(PRG_GCW) = 0.0;
      }
    }
  }
}

/* aerosol_scavenging (main:3122-3193) */
static void aerosol_scavenging(ws_t *w, double odt) {
  int nz = w->nz;
  double *tw = w->tw;
  const double wf_aerosol_size = 0.04e-6, if_aerosol_size = 0.8e-6;
  for (int k = 0; k < nz; k++) {
    if (w->l_qr[k] && w->mvd_r[k] > d0r) {
      double ef_ra = aerosol_collection_efficiency(w->mvd_r[k], wf_aerosol_size, w->visco[k],
                                                   w->rho[k], w->temp[k], 'r');
      double lamr = 1.0 / w->ilamr[k];
      double n0_r = w->nr[k] * org2 * pow(lamr, CRE(2));
      TD(PNA_RCA) = w->rhof[k] * t1_qr_qc * ef_ra * w->nwfa[k] * n0_r * pow(lamr + fv_r, -CRE(9));
      TD(PNA_RCA) = fmin2(w->nwfa[k] * odt, TD(PNA_RCA));
      ef_ra = aerosol_collection_efficiency(w->mvd_r[k], if_aerosol_size, w->visco[k], w->rho[k],
                                            w->temp[k], 'r');
      TD(PND_RCD) = w->rhof[k] * t1_qr_qc * ef_ra * w->nifa[k] * n0_r * pow(lamr + fv_r, -CRE(9));
      TD(PND_RCD) = fmin2(w->nifa[k] * odt, TD(PND_RCD));
    }
    if (w->l_qs[k] && w->rs[k] > r_s[0]) {
      double xds = w->smoc[k] / w->smob[k];
      double ef_sa = aerosol_collection_efficiency(xds, wf_aerosol_size, w->visco[k], w->rho[k],
                                                   w->temp[k], 's');
      TD(PNA_SCA) = w->rhof[k] * t1_qs_qc * ef_sa * w->nwfa[k] * w->smoe[k];
      TD(PNA_SCA) = fmin2(w->nwfa[k] * odt, TD(PNA_SCA));
      ef_sa = aerosol_collection_efficiency(xds, if_aerosol_size, w->visco[k], w->rho[k], w->temp[k],
                                            's');
      TD(PND_SCD) = w->rhof[k] * t1_qs_qc * ef_sa * w->nifa[k] * w->smoe[k];
      TD(PND_SCD) = fmin2(w->nifa[k] * odt, TD(PND_SCD));
    }
    if (w->l_qg[k] && w->rg[k] > r_g[0]) {
      int ig = w->idx_bg[k];
      double xdg = (bm_g + mu_g + 1.0) * w->ilamg[k];
      double ef_ga = aerosol_collection_efficiency(xdg, wf_aerosol_size, w->visco[k], w->rho[k],
                                                   w->temp[k], 'g');
      double t1_qg_qc = pi * .25 * AV_G(ig) * CGG(9, ig);
      double n0_g = w->ng[k] * ogg2 * pow(1.0 / w->ilamg[k], CGE(2, 1));
      TD(PNA_GCA) = w->rhof[k] * t1_qg_qc * ef_ga * w->nwfa[k] * n0_g * pow(w->ilamg[k], CGE(9, ig));
      TD(PNA_GCA) = fmin2(w->nwfa[k] * odt, TD(PNA_GCA));
      ef_ga = aerosol_collection_efficiency(xdg, if_aerosol_size, w->visco[k], w->rho[k], w->temp[k],
                                            'g');
      TD(PND_GCD) = w->rhof[k] * t1_qg_qc * ef_ga * w->nifa[k] * n0_g * pow(w->ilamg[k], CGE(9, ig));
      TD(PND_GCD) = fmin2(w->nifa[k] * odt, TD(PND_GCD));
    }
  }
}

/* cloud_condensation (main:1980-2056) */
static void cloud_condensation(ws_t *w, const double *w1d, const double *nwfa1d, int have_ncsave,
                               double dt, double odt) {
  int nz = w->nz;
  double *tw = w->tw;
  for (int k = 0; k < nz; k++) {
    if (fabs(w->ssatw[k]) < eps) continue;
    double orho = 1.0 / w->rho[k];
    double clap = (w->qv[k] - w->qvs[k]) / (1.0 + w->lvt2[k] * w->qvs[k]);
    for (int n = 1; n <= 3; n++) {
      double fcd = w->qvs[k] * exp(w->lvt2[k] * clap) - w->qv[k] + clap;
      double dfcd = w->qvs[k] * w->lvt2[k] * exp(w->lvt2[k] * clap) + 1.0;
      clap = clap - fcd / dfcd;
    }
    double xrc = w->rc[k] + clap * w->rho[k];
    double xnc = 0.0;
    if (xrc > r1) {
      TD(PRW_VCD) = clap * odt;
      if (clap > eps) {
        if (nwfa1d)
          xnc = fmax2(nt_c_min, activate_cloud_number(w->temp[k], w1d[k], w->nwfa[k]));
        else if (have_ncsave)
          xnc = w->ncsave[k];
        else
          xnc = nt_c_l;
        TD(PNC_WCD) = 0.5 * (xnc - w->nc[k] + fabs(xnc - w->nc[k])) * odt * orho;
      } else if (w->l_qc[k] && w->ssatw[k] < -1.e-6 && clap < -eps) {
        double otemp = 1.0 / w->temp[k];
        double rvs = w->rho[k] * w->qvs[k];
        double rvs_p = rvs * otemp * (w->lvap[k] * otemp * orv - 1.0);
        double rvs_pp = rvs * (otemp * (w->lvap[k] * otemp * orv - 1.0) * otemp *
                                   (w->lvap[k] * otemp * orv - 1.0) +
                               (-2.0 * w->lvap[k] * otemp * otemp * otemp * orv) + otemp * otemp);
        double gamsc = w->lvap[k] * w->diffu[k] / w->tcond[k] * rvs_p;
        double alphsc = 0.5 * (gamsc / (1.0 + gamsc)) * (gamsc / (1.0 + gamsc)) * rvs_pp / rvs_p *
                        rvs / rvs_p;
        alphsc = fmax2(1.e-9, alphsc);
        double xsat = w->ssatw[k];
        if (fabs(xsat) < 1.e-9) xsat = 0.0;
        double t1_evap = 2.0 * pi *
                         (1.0 - alphsc * xsat + 2.0 * alphsc * alphsc * xsat * xsat -
                          5.0 * alphsc * alphsc * alphsc * xsat * xsat * xsat) /
                         (1.0 + gamsc);
        double dc_star = sqrt(-2.0 * dt * t1_evap / (2.0 * pi) * 4.0 * w->diffu[k] * w->ssatw[k] *
                              rvs / rho_w);
        int idx_d = imax(1, imin((int)(1.e6 * dc_star), nbc));
        int idx_c, idx_n;
        get_cloud_table_index(w->rc[k], w->nc[k], &idx_c, &idx_n);
        TRACE(k, TR_EVAP, idx_d | (idx_c << 8) | (idx_n << 16) | (1 << 24));
        TD(PRW_VCD) = fmax2(-w->rc[k] * 0.99 * orho * odt, TD(PRW_VCD));
        TD(PNC_WCD) = fmax2(-w->nc[k] * 0.99 * orho * odt,
                            -TNC_WEV(idx_d, idx_c, idx_n) * orho * odt);
      }
    } else {
      TD(PRW_VCD) = -w->rc[k] * orho * odt;
      TD(PNC_WCD) = -w->nc[k] * orho * odt;
    }
  }
}

/* rain_evaporation (main:2059-2121) */
static void rain_evaporation(ws_t *w, double odt) {
  int nz = w->nz;
  double *tw = w->tw;
  for (int k = 0; k < nz; k++) {
    if (w->l_qr[k]) {
      if ((w->ssatw[k] < -eps) && TD(PRW_VCD) <= 0.0) {
        double orho = 1.0 / w->rho[k];
        double tempc = w->temp[k] - t0;
        double otemp = 1.0 / w->temp[k];
        double rvs = w->rho[k] * w->qvs[k];
        double rvs_p = rvs * otemp * (w->lvap[k] * otemp * orv - 1.0);
        double rvs_pp = rvs * (otemp * (w->lvap[k] * otemp * orv - 1.0) * otemp *
                                   (w->lvap[k] * otemp * orv - 1.0) +
                               (-2.0 * w->lvap[k] * otemp * otemp * otemp * orv) + otemp * otemp);
        double gamsc = w->lvap[k] * w->diffu[k] / w->tcond[k] * rvs_p;
        double alphsc = 0.5 * (gamsc / (1.0 + gamsc)) * (gamsc / (1.0 + gamsc)) * rvs_pp / rvs_p *
                        rvs / rvs_p;
        alphsc = fmax2(1.e-9, alphsc);
        double xsat = fmin2(-1.e-9, w->ssatw[k]);
        double t1_evap = 2.0 * pi *
                         (1.0 - alphsc * xsat + 2.0 * alphsc * alphsc * xsat * xsat -
                          5.0 * alphsc * alphsc * alphsc * xsat * xsat * xsat) /
                         (1.0 + gamsc);
        if (w->qv[k] / w->qvs[k] < 0.95 && w->rr[k] * orho <= 1.e-8) {
          TD(PRV_REV) = w->rr[k] * orho * odt;
        } else {
          double lamr = 1.0 / w->ilamr[k];
          double n0_r = w->nr[k] * org2 * pow(lamr, CRE(2));
          TD(PRV_REV) = t1_evap * w->diffu[k] * (-w->ssatw[k]) * n0_r * rvs *
                        (t1_qr_ev * pow(w->ilamr[k], CRE(10)) +
                         t2_qr_ev * w->vsc2[k] * w->rhof2[k] * pow(lamr + 0.5 * fv_r, -CRE(11)));
          double rate_max = fmin2((w->rr[k] * orho * odt), (w->qvs[k] - w->qv[k]) * odt);
          TD(PRV_REV) = fmin2(rate_max, TD(PRV_REV) * orho);
          if (TD(PRR_GML) > 0.0) {
            double eva_factor = fmin2(1.0, 0.01 + (0.99 - 0.01) * (tempc / 20.0));
            TD(PRV_REV) = TD(PRV_REV) * eva_factor;
          }
        }
        TD(PNR_REV) = fmin2(w->nr[k] * 0.99 * orho * odt, TD(PRV_REV) * w->nr[k] / w->rr[k]);
      }
    }
  }
}

/* freeze_cloud_melt_ice (main:2124-2165) */
static void freeze_cloud_melt_ice(ws_t *w, const double *qi1d, const double *ni1d,
                                  const double *qc1d, const double *nc1d, int have_ncsave,
                                  double dt, double odt) {
  int nz = w->nz;
  for (int k = 0; k < nz; k++) {
    double xri = fmax2(0.0, qi1d[k] + w->qiten[k] * dt);
    if ((w->temp[k] > t0) && (xri > 0.0)) {
      w->qcten[k] = w->qcten[k] + xri * odt;
      w->ncten[k] = w->ncten[k] + ni1d[k] * odt;
      w->qiten[k] = w->qiten[k] - xri * odt;
      w->niten[k] = -ni1d[k] * odt;
      w->tten[k] = w->tten[k] - lfus * w->ocp[k] * xri * odt;
    }
    double xrc = fmax2(0.0, qc1d[k] + w->qcten[k] * dt);
    if ((w->temp[k] < hgfrz) && (xrc > 0.0)) {
      double lfus2 = lsub - w->lvap[k], xnc;
      if (nc1d)
        xnc = nc1d[k] + w->ncten[k] * dt;
      else if (have_ncsave)
        xnc = w->ncsave[k] / w->rho[k] + w->ncten[k] * dt;
      else
        xnc = nt_c_l / w->rho[k] + w->ncten[k] * dt;
      w->qiten[k] = w->qiten[k] + xrc * odt;
      w->niten[k] = w->niten[k] + xnc * odt;
      w->qcten[k] = w->qcten[k] - xrc * odt;
      w->ncten[k] = w->ncten[k] - xnc * odt;
      w->tten[k] = w->tten[k] + lfus2 * w->ocp[k] * xrc * odt;
    }
  }
}

/* ------------------------------------------------------------------------------ */
/* diagnostics (diags.F90)                                                          */
/* ------------------------------------------------------------------------------ */
static void snow_moments_all(ws_t *w, int k, int full) {
  double tc0 = fmin2(-0.1, w->temp[k] - t0);
  if (full == 1)
    o_snow_moments(w->rs[k], tc0, &w->smob[k], &w->smoc[k], &w->ns[k], &w->smo0[k], &w->smo1[k],
                   &w->smo2[k], &w->smoe[k], &w->smof[k], &w->smog[k], NULL);
  else if (full == 0)
    o_snow_moments(w->rs[k], tc0, &w->smob[k], &w->smoc[k], NULL, NULL, NULL, &w->smo2[k], NULL,
                   NULL, NULL, NULL);
  else
    o_snow_moments(w->rs[k], tc0, &w->smob[k], &w->smoc[k], NULL, NULL, NULL, &w->smo2[k], NULL,
                   NULL, NULL, &w->smoz[k]);
}

/* effective_radius (diags:13-56) */
static void effective_radius(ws_t *w, double *re_qc, double *re_qi, double *re_qs) {
  int nz = w->nz;
  for (int k = 0; k < nz; k++) {
    re_qc[k] = 0.0;
    re_qi[k] = 0.0;
    re_qs[k] = 0.0;
    if (w->l_qc[k]) {
      int nu_c = o_get_nuc(w->nc[k]);
      re_qc[k] = fmax2(2.51e-6, fmin2(0.5 * (3.0 + (double)nu_c) * w->ilamc[k], 50.e-6));
    }
    if (w->l_qi[k]) re_qi[k] = fmax2(2.51e-6, fmin2(0.5 * (3.0 + mu_i) * w->ilami[k], 125.e-6));
    if (w->l_qs[k]) {
      double tc0 = fmin2(-0.1, w->temp[k] - t0), smob, smoc;
      o_snow_moments(w->rs[k], tc0, &smob, &smoc, NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL);
      re_qs[k] = fmax2(5.01e-6, fmin2(0.5 * (smoc / smob), 999.e-6));
    }
  }
}

/* complex_water_ray (diags:144-173): refractive index of water after Ray (1972), Appl.
 * Opt. 11, 1836, for temperature t (Celsius) and wavelength lambda (m) */
static double complex complex_water_ray(double lambda, double t) {
  double epsinf = 5.27137 + 0.02164740 * t - 0.00131198 * t * t;
  double epss = 78.54 * (1.0 - 4.579e-3 * (t - 25.0) + 1.190e-5 * (t - 25.0) * (t - 25.0) -
                         2.800e-8 * (t - 25.0) * (t - 25.0) * (t - 25.0));
  double alpha = -16.8129 / (t + 273.16) + 0.0609265;
  double lambdas = 0.00033836 * exp(2513.98 / (t + 273.16)) * 1e-2;
  double nenner = 1.0 + 2.0 * pow(lambdas / lambda, 1.0 - alpha) * sin(alpha * pi * 0.5) +
                  pow(lambdas / lambda, 2.0 - 2.0 * alpha);
  double epsr = epsinf + ((epss - epsinf) * (pow(lambdas / lambda, 1.0 - alpha) *
                                                 sin(alpha * pi * 0.5) + 1.0)) / nenner;
  double epsi = ((epss - epsinf) * (pow(lambdas / lambda, 1.0 - alpha) * cos(alpha * pi * 0.5) +
                                    0.0)) / nenner + lambda * 1.25664 / 1.88496;
  return csqrt(CMPLX(epsr, -epsi));
}

/* complex_ice_maetzler (diags:176-203): refractive index of ice after Maetzler (1998) */
static double complex complex_ice_maetzler(double lambda, double t) {
  double c = 2.99e8, tk = t + 273.16, f = c / lambda * 1e-9;
  double b1 = 0.0207, b2 = 1.16e-11, b = 335.0;
  double deltabeta = exp(-10.02 + 0.0364 * (tk - 273.16));
  double e = exp(b / tk) - 1.0;
  double betam = (b1 / tk) * (exp(b / tk) / (e * e)) + b2 * f * f;
  double beta = betam + deltabeta;
  double theta = 300.0 / tk - 1.0;
  double alfa = (0.00504 + 0.0062 * theta) * exp(-22.1 * theta);
  double complex ri = 3.1884 + 9.1e-4 * (tk - 273.16);
  ri = ri + CMPLX(0.0, (alfa / f + beta * f));
  return csqrt(conj(ri));
}

/* rayleigh_soak_wetgraupel (diags:311-394): backscatter cross section of a wet snow or
 * graupel particle of mass x_g, Maxwell-Garnett mixing and the Rayleigh approximation */
static double rayleigh_soak_wetgraupel(double x_g, double a_geo, double b_geo, double fmelt,
                                       double lambda_radar, double meltratio_outside,
                                       double complex m_w, double complex m_i) {
  double complex m_air = CMPLX(1.0, 0.0);
  double fm = fmax2(fmin2(fmelt, 1.0), 0.0);
  double mra = fmax2(fmin2(meltratio_outside, 1.0), 0.0);
  mra = mra + (1.0 - mra) * fm;
  double x_w = x_g * fm;
  double d_g = a_geo * pow(x_g, b_geo);
  if (!(d_g >= r1)) return 0.0;
  double vg = pi / 6.0 * d_g * d_g * d_g;
  double rhog = fmax2(fmin2(x_g / vg, 900.0), 10.0);
  vg = x_g / rhog;
  double meltratio_outside_grenz = 1.0 - rhog / 1000.0;
  double volg;
  if (mra <= meltratio_outside_grenz) {
    volg = vg * (1.0 - mra * fm);
  } else {
    double fmgrenz = (900.0 - rhog) / (mra * 900.0 - rhog + 900.0 * rhog / 1000.0);
    if (fm <= fmgrenz)
      volg = (1.0 - mra * fm) * vg;
    else
      volg = (x_g - x_w) / 900.0 + x_w / 1000.0;
  }
  double d_large = pow(6.0 / pi * volg, 1.0 / 3.0);
  double volice = (x_g - x_w) / (volg * 900.0);
  double volwater = x_w / (1000.0 * volg);
  double volair = 1.0 - volice - volwater;
  double volmix1 = volice / fmax2(volice + volwater, 1e-10);
  double volmix2 = 1.0 - volmix1;
  (void)volmix2;
  /* ice in water */
  double complex m1t = m_w * m_w, m2t = m_air * m_air, m3t = m_i * m_i;
  double vol2 = 0.0, vol3 = volmix1;
  double complex beta2 = 2.0 * m1t / (m2t - m1t) * (m2t / (m2t - m1t) * clog(m2t / m1t) - 1.0);
  double complex beta3 = 2.0 * m1t / (m3t - m1t) * (m3t / (m3t - m1t) * clog(m3t / m1t) - 1.0);
  double complex m_tmp = csqrt(((1.0 - vol2 - vol3) * m1t + vol2 * beta2 * m2t + vol3 * beta3 * m3t) /
                               (1.0 - vol2 - vol3 + vol2 * beta2 + vol3 * beta3));
  /* air in the mixture */
  m1t = m_tmp * m_tmp;
  m2t = m_air * m_air;
  m3t = (2.0 * m_air) * (2.0 * m_air);
  vol2 = volair;
  vol3 = 0.0;
  beta2 = 2.0 * m1t / (m2t - m1t) * (m2t / (m2t - m1t) * clog(m2t / m1t) - 1.0);
  beta3 = 2.0 * m1t / (m3t - m1t) * (m3t / (m3t - m1t) * clog(m3t / m1t) - 1.0);
  double complex m_core = csqrt(((1.0 - vol2 - vol3) * m1t + vol2 * beta2 * m2t + vol3 * beta3 * m3t) /
                                (1.0 - vol2 - vol3 + vol2 * beta2 + vol3 * beta3));
  double kk = cabs((m_core * m_core - 1.0) / (m_core * m_core + 2.0));
  double d6 = ipow(d_large, 6);
  return kk * kk * pi * pi * pi * pi * pi * d6 /
         (lambda_radar * lambda_radar * lambda_radar * lambda_radar);
}

/* Simpson weights over the radar bins (diags:224-231) */
static void simpson_weights(double *simpson) {
  const double basis[3] = {1.0 / 3.0, 4.0 / 3.0, 1.0 / 3.0};
  for (int n = 0; n < radar_bins + 1; n++) simpson[n] = 0.0;
  for (int n = 1; n <= radar_bins - 1; n += 2) {
    simpson[n - 1] += basis[0];
    simpson[n] += basis[1];
    simpson[n + 1] += basis[2];
  }
}

/* reflectivity_from_melting_graupel (diags:206-248) */
static double reflectivity_from_melting_graupel(double rg, double ng, double ilamg, int idx,
                                                double rr) {
  const double melt_outside = 0.9, lambda_radar = 0.10;
  double simpson[radar_bins + 1];
  simpson_weights(simpson);
  double complex m_w_0 = complex_water_ray(lambda_radar, 0.0);
  double complex m_i_0 = complex_ice_maetzler(lambda_radar, 0.0);
  double kw1 = cabs((m_w_0 * m_w_0 - 1.0) / (m_w_0 * m_w_0 + 2.0));
  double k_w = kw1 * kw1;
  double sr = fmax2(0.01, fmin2(1.0 - rg / fmax2(rg + rr, r1), 0.99));
  double fmelt = sr * sr;
  double eta = 0.0;
  double lamg = 1.0 / ilamg;
  double n0_g = ng * ogg2 * pow(lamg, CGE(2, 1));
  for (int n = 0; n < radar_bins; n++) {
    double mass = AM_G(idx) * pow(gbins_radar[n], bm_g);
    double backscatter = rayleigh_soak_wetgraupel(mass, OCMG(idx), obmg, fmelt, lambda_radar,
                                                  melt_outside, m_w_0, m_i_0);
    double f_d = n0_g * pow(gbins_radar[n], mu_g) * exp(-lamg * gbins_radar[n]);
    eta = eta + f_d * backscatter * simpson[n] * dgbins_radar[n];
  }
  return lambda_radar * lambda_radar * lambda_radar * lambda_radar / (pi * pi * pi * pi * pi * k_w) * eta;
}

/* reflectivity_from_melting_snow (diags:251-308) */
static double reflectivity_from_melting_snow(double rs, double smob, double smoc, double rr) {
  const double melt_outside = 0.9, lambda_radar = 0.10;
  double simpson[radar_bins + 1];
  simpson_weights(simpson);
  double complex m_w_0 = complex_water_ray(lambda_radar, 0.0);
  double complex m_i_0 = complex_ice_maetzler(lambda_radar, 0.0);
  double kw1 = cabs((m_w_0 * m_w_0 - 1.0) / (m_w_0 * m_w_0 + 2.0));
  double k_w = kw1 * kw1;
  double sr = fmax2(0.01, fmin2(1.0 - rs / (rs + rr), 0.99));
  double fmelt = sr * sr;
  double eta = 0.0;
  double om3 = 1.0 / smoc;
  double m0 = smob * om3;
  double mrat = smob * m0 * m0 * m0;
  double slam1 = m0 * lam0, slam2 = m0 * lam1;
  for (int n = 0; n < radar_bins; n++) {
    double mass = am_s * pow(sbins_radar[n], bm_s);
    double backscatter = rayleigh_soak_wetgraupel(mass, ocms, obms, fmelt, lambda_radar,
                                                  melt_outside, m_w_0, m_i_0);
    double f_d = mrat * (kap0 * exp(-slam1 * sbins_radar[n]) +
                         kap1 * pow(m0 * sbins_radar[n], mu_s) * exp(-slam2 * sbins_radar[n]));
    eta = eta + f_d * backscatter * simpson[n] * dsbins_radar[n];
  }
  return lambda_radar * lambda_radar * lambda_radar * lambda_radar / (pi * pi * pi * pi * pi * k_w) * eta;
}

/* find_melting_level (diags:124-141); 1-based level, 1 = none found */
static int find_melting_level(const ws_t *w) {
  int nz = w->nz, k_melt = 1;
  for (int k = nz - 1; k >= 1; k--) /* reference k = nz-1 .. 1 */
    if (w->temp[k - 1] > t0 && w->l_qr[k - 1] && (w->l_qs[k] || w->l_qg[k])) {
      k_melt = imax(k + 1, k_melt);
      break;
    }
  return k_melt;
}

/* reflectivity_10cm (diags:59-121), with the melting contributions of snow and graupel
 * below the melting level when `melting` */
static void reflectivity_10cm(ws_t *w, double *dbz, int melting) {
  int nz = w->nz;
  int k_melt = melting ? find_melting_level(w) : 1;
  for (int k = 0; k < nz; k++) {
    w->ze_r[k] = 1.e-22;
    w->ze_s[k] = 1.e-22;
    w->ze_g[k] = 1.e-22;
  }
  for (int k = nz - 1; k >= 0; k--) {
    const int kf = k + 1; /* the reference's level index */
    const int melt_here = melting && k_melt > 2 && kf < k_melt - 1;
    dbz[k] = -35.0;
    if (w->l_qr[k]) {
      double lamr = 1.0 / w->ilamr[k];
      double n0_r = w->nr[k] * org2 * pow(lamr, CRE(2));
      w->ze_r[k] = n0_r * CRG(4) * pow(w->ilamr[k], CRE(4));
    }
    if (w->l_qs[k]) {
      w->ze_s[k] = (0.176 / 0.93) * (6.0 / pi) * (6.0 / pi) * (am_s / 900.0) * (am_s / 900.0) * w->smoz[k];
      if (melt_here)
        w->ze_s[k] = reflectivity_from_melting_snow(w->rs[k], w->smob[k], w->smoc[k], w->rr[k]);
    }
    if (w->l_qg[k]) {
      int ig = w->idx_bg[k];
      double n0_g = w->ng[k] * ogg2 * pow(1.0 / w->ilamg[k], CGE(2, 1));
      w->ze_g[k] = (0.176 / 0.93) * (6.0 / pi) * (6.0 / pi) * (AM_G(ig) / 900.0) * (AM_G(ig) / 900.0) *
                   n0_g * CGG(4, 1) * pow(w->ilamg[k], CGE(4, 1));
      if (melt_here)
        w->ze_g[k] = reflectivity_from_melting_graupel(w->rg[k], w->ng[k], w->ilamg[k], ig, w->rr[k]);
    }
    dbz[k] = fmax2(-35.0, 10.0 * log10((w->ze_r[k] + w->ze_s[k] + w->ze_g[k]) * 1.e18));
  }
}

/* max_hail_diam (diags:398-438) */
static void max_hail_diam(ws_t *w, double *mhd) {
  int nz = w->nz;
  const double threshold_conc = 0.0005;
  for (int k = 0; k < nz; k++) {
    mhd[k] = 0.0;
    if (w->rg[k] / w->rho[k] >= 1.e-6) {
      if (RHO_G(w->idx_bg[k]) < 350.0) continue;
      double lamg = 1.0 / w->ilamg[k];
      double n0_g = w->ng[k] * ogg2 * pow(lamg, CGE(2, 1));
      double sum_nh = 0.0, sum_t = 0.0, hail_max;
      int n;
      for (n = nhbins; n >= 1; n--) {
        double f_d = n0_g * pow(hbins[n - 1], mu_g) * exp(-lamg * hbins[n - 1]) * dhbins[n - 1];
        sum_nh = sum_nh + f_d;
        if (sum_nh > threshold_conc) break;
        sum_t = sum_nh;
      }
      if (n >= nhbins)
        hail_max = hbins[nhbins - 1];
      else if (hbins[n] > 1.e-3)
        hail_max = hbins[n - 1] - (sum_nh - threshold_conc) / (sum_nh - sum_t) * (hbins[n - 1] - hbins[n]);
      else
        hail_max = 1.e-4;
      mhd[k] = 1000.0 * hail_max;
    }
  }
}

/* ------------------------------------------------------------------------------ */
/* tempo_main (main:73-864)                                                         */
/* ------------------------------------------------------------------------------ */
typedef struct {
  double *refl, *re_c, *re_i, *re_s, *mvd_r, *mvd_g, *mhd, *ncmr; /* nz each, NULL if off */
  const double *qc_bl, *qcfrac_bl; /* the boundary-layer cloud of the column, or NULL */
} colout_t;

/* cloud-number network of the ML path (ml:104-176): input scaler, two dense layers
 * with ReLU, clamp to [-6, log10(2e9)], bias correction, 10**x.  The weights come from
 * the host (oracle_set_ml), as the reference's come from its ML module. */
static double ml_mean[7], ml_var[7], ml_w00[168], ml_b00[24], ml_w01[24], ml_b01[1];
static int ml_loaded = 0;

int oracle_set_ml(const double *mean, const double *var, const double *w00, const double *b00,
                  const double *w01, const double *b01) {
  memcpy(ml_mean, mean, sizeof ml_mean);
  memcpy(ml_var, var, sizeof ml_var);
  memcpy(ml_w00, w00, sizeof ml_w00);
  memcpy(ml_b00, b00, sizeof ml_b00);
  memcpy(ml_w01, w01, sizeof ml_w01);
  memcpy(ml_b01, b01, sizeof ml_b01);
  ml_loaded = 1;
  return 0;
}

static double ml_predict_nc(double qc, double qr, double qi, double qs, double pres, double temp,
                            double w) {
  const double logmin = -6.0, logmax = 9.3010299957;
  const double in[7] = {qc, qr, qi, qs, pres, temp, w};
  double x[7], h[24];
  for (int j = 0; j < 7; j++) x[j] = (in[j] - ml_mean[j]) / sqrt(ml_var[j]);
  for (int i = 0; i < 24; i++) { /* weights00 = reshape(w00, [24, 7]) */
    double acc = 0.0;
    for (int j = 0; j < 7; j++) acc = acc + ml_w00[j * 24 + i] * x[j];
    h[i] = fmax2(acc + ml_b00[i], 0.0);
  }
  double acc = 0.0;
  for (int i = 0; i < 24; i++) acc = acc + ml_w01[i] * h[i];
  double out = fmax2(acc + ml_b01[0], 0.0);
  double pe = fmin2(logmax, fmax2(logmin, out));
  double corr = 1.0;
  if (pe >= 0.0 && pe < 3.0)
    corr = -0.2704 * ipow(pe, 5) + 1.838 * ipow(pe, 4) - 5.127 * ipow(pe, 3) + 8.547 * ipow(pe, 2) -
           8.439 * pe + 4.297;
  return corr * pow(10.0, pe);
}

static double resolve_nc_value(const ocfg_t *cfg) {
  const char *s = cfg->single_moment_nc_opt;
  while (*s == ' ') s++;
  char buf[33];
  strncpy(buf, s, 32);
  buf[32] = 0;
  for (int i = (int)strlen(buf) - 1; i >= 0 && buf[i] == ' '; i--) buf[i] = 0;
  if (!strcmp(buf, "land")) return nt_c_l;
  if (!strcmp(buf, "ocean")) return nt_c_o;
  char *end = NULL;
  double v = strtod(buf, &end);
  if (end == buf) return nt_c_l;
  return v;
}

static void tempo_main_col(const ocfg_t *cfg, int is_first_step, double *qv1d, double *qc1d,
                           double *qi1d, double *qr1d, double *qs1d, double *qg1d, double *qb1d,
                           double *ni1d, double *nr1d, double *nc1d, double *ng1d, double *nwfa1d,
                           double *nifa1d, double *t1d, const double *p1d, const double *w1d,
                           const double *dz1d, const int *land1d, double dt, ws_t *w, mdiag_t *md,
                           colout_t *co) {
  int nz = w->nz;
  double *tw = w->tw;
  int k, supersaturated = 0, have_ncsave = 0;
  double odt = 1.0 / dt;
  int hail_ng_qb = (ng1d != NULL) && (qb1d != NULL);

  memset(tw, 0, sizeof(double) * (size_t)NTEND * nz); /* :269 */
  for (k = 0; k < nz; k++) {                         /* :272-298 */
    w->tten[k] = w->qvten[k] = w->qcten[k] = w->qiten[k] = w->qrten[k] = w->qsten[k] = 0.0;
    w->qgten[k] = w->ngten[k] = w->qbten[k] = w->niten[k] = w->nrten[k] = w->ncten[k] = 0.0;
    w->nwfaten[k] = w->nifaten[k] = 0.0;
    w->smo0[k] = w->smo1[k] = w->smo2[k] = w->smob[k] = w->smoc[k] = 0.0;
    w->smoe[k] = w->smof[k] = w->smog[k] = w->smoz[k] = w->ns[k] = 0.0;
    w->vtboost[k] = 1.0;
  }
  for (k = 0; k <= nz; k++) /* :301-311 */
    w->vtrr[k] = w->vtnr[k] = w->vtrs[k] = w->vtri[k] = w->vtni[k] = w->vtrc[k] = w->vtnc[k] =
        w->vtrg[k] = w->vtng[k] = 0.0;
  memset(md, 0, sizeof *md);

  for (k = 0; k < nz; k++) { /* :321-326 */
    w->temp[k] = t1d[k];
    w->qv[k] = fmax2(min_qv, qv1d[k]);
    w->pres[k] = p1d[k];
    w->rho[k] = roverrv * w->pres[k] / (rdry * w->temp[k] * (w->qv[k] + roverrv));
  }
  /* :328-342 */
  if (nwfa1d) {
    if (is_first_step) {
      double s = 0;
      for (k = 0; k < nz; k++) s += nwfa1d[k];
      if (s < eps) init_aerosols(nz, dz1d, w->nwfa, w->hgt, naccn0, naccn1);
    }
  } else {
    init_aerosols(nz, dz1d, w->nwfa, w->hgt, naccn0, naccn1);
  }
  if (nifa1d) {
    if (is_first_step) {
      double s = 0;
      for (k = 0; k < nz; k++) s += nifa1d[k];
      if (s < eps) init_aerosols(nz, dz1d, w->nifa, w->hgt, nain0, nain1);
    }
  } else {
    init_aerosols(nz, dz1d, w->nifa, w->hgt, nain0, nain1);
  }
  aerosol_check_and_update(nz, w->rho, nwfa1d, nifa1d, w->nwfa, w->nifa, w->nwfaten, w->nifaten, dt);
  t_tpass = 0;
  rain_check_and_update(nz, w->rho, w->l_qr, qr1d, nr1d, w->rr, w->nr, w->qrten, w->nrten,
                        w->ilamr, w->mvd_r, dt, odt);
  ice_check_and_update(nz, w->rho, w->l_qi, qi1d, ni1d, w->ri, w->ni, w->qiten, w->niten, w->ilami,
                       dt, odt);
  snow_check_and_update(nz, w->rho, w->l_qs, qs1d, w->rs, w->qsten, dt, odt);
  for (k = 0; k < nz; k++) /* :353-361 */
    if (w->l_qs[k]) snow_moments_all(w, k, 1);
  if (!nc1d) { /* :364-380 */
    if (cfg->ml_for_nc_flag) {
      for (k = 0; k < nz; k++) {
        const double xq = qc1d[k] <= 1.e-12 ? 0.0 : qc1d[k];
        w->nc[k] = ml_predict_nc(xq, qr1d[k], qi1d[k], qs1d[k], w->pres[k], w->temp[k], w1d[k]) * w->rho[k];
      }
    } else {
      double v;
      if (land1d)
        v = (*land1d != 1) ? nt_c_o : nt_c_l;
      else
        v = resolve_nc_value(cfg);
      for (k = 0; k < nz; k++) w->nc[k] = v;
    }
    for (k = 0; k < nz; k++) w->ncsave[k] = w->nc[k];
    have_ncsave = 1;
  }
  cloud_check_and_update(nz, w->rho, w->l_qc, qc1d, nc1d, have_ncsave ? w->ncsave : NULL, w->rc,
                         w->nc, w->qcten, w->ncten, w->ilamc, w->mvd_c, dt, odt);
  if (is_first_step) { /* :387-393 */
    if (hail_ng_qb) {
      double sqg = 0, sng = 0, sqb = 0;
      for (k = 0; k < nz; k++) {
        sqg += qg1d[k];
        sng += ng1d[k];
        sqb += qb1d[k];
      }
      if (sqg > r1 && sng < eps && sqb < eps) graupel_init(nz, w->rho, qg1d, ng1d, qb1d);
    }
  }
  graupel_check_and_update(nz, w->rho, w->l_qg, qg1d, ng1d, qb1d, w->rg, w->ng, w->rb, w->idx_bg,
                           w->qgten, w->ngten, w->qbten, w->ilamg, w->mvd_g, dt, odt);
  for (k = 0; k < nz; k++) { /* :399-410 */
    w->qcten[k] = w->qiten[k] = w->qrten[k] = w->qsten[k] = w->qgten[k] = 0.0;
    w->ngten[k] = w->qbten[k] = w->niten[k] = w->nrten[k] = w->ncten[k] = 0.0;
  }
  thermo_vars(w, &supersaturated);
  /* :417-418 early exit */
  int do_micro = 0;
  for (k = 0; k < nz; k++)
    if (w->l_qc[k] || w->l_qr[k] || w->l_qi[k] || w->l_qs[k] || w->l_qg[k]) do_micro = 1;
  if (!do_micro && !supersaturated) {
    md->early_exit = 1;
    return;
  }

  if (!cfg->turn_off_micro_flag) { /* :421-450 */
    warm_rain(w, odt);
    rain_snow_rain_graupel(w, odt);
    ice_nucleation(w, w1d, nwfa1d, nifa1d, dt, odt);
    ice_processes(w, w1d, odt);
    riming(w, odt);
    melting(w, dt, odt);
    if (nwfa1d || nifa1d) aerosol_scavenging(w, odt);
  }
  check_over_depletion(w, odt);
  sum_tendencies(w);

  for (k = 0; k < nz; k++) { /* :460-468 */
    w->temp[k] = t1d[k] + w->tten[k] * dt;
    w->qv[k] = fmax2(min_qv, qv1d[k] + w->qvten[k] * dt);
    w->rho[k] = roverrv * w->pres[k] / (rdry * w->temp[k] * (w->qv[k] + roverrv));
    w->nwfaten[k] = w->nwfaten[k] - (TD(PNA_RCA) + TD(PNA_SCA) + TD(PNA_GCA) + TD(PNI_IHA)) / w->rho[k];
    w->nifaten[k] = w->nifaten[k] - (TD(PND_RCD) + TD(PND_SCD) + TD(PND_GCD)) / w->rho[k];
  }
  aerosol_check_and_update(nz, w->rho, nwfa1d, nifa1d, w->nwfa, w->nifa, w->nwfaten, w->nifaten, dt);

  /* :475-526 checks on temporaries */
  memcpy(w->xrx, qc1d, sizeof(double) * nz);
  double *xncx = NULL;
  if (nc1d) {
    memcpy(w->xncx, nc1d, sizeof(double) * nz);
    xncx = w->xncx;
  }
  t_tpass = 1;
  cloud_check_and_update(nz, w->rho, w->l_qc, w->xrx, xncx, have_ncsave ? w->ncsave : NULL, w->rc,
                         w->nc, w->qcten, w->ncten, w->ilamc, w->mvd_c, dt, odt);
  memcpy(w->xrx, qr1d, sizeof(double) * nz);
  memcpy(w->xnx, nr1d, sizeof(double) * nz);
  rain_check_and_update(nz, w->rho, w->l_qr, w->xrx, w->xnx, w->rr, w->nr, w->qrten, w->nrten,
                        w->ilamr, w->mvd_r, dt, odt);
  memcpy(w->xrx, qi1d, sizeof(double) * nz);
  memcpy(w->xnx, ni1d, sizeof(double) * nz);
  ice_check_and_update(nz, w->rho, w->l_qi, w->xrx, w->xnx, w->ri, w->ni, w->qiten, w->niten,
                       w->ilami, dt, odt);
  memcpy(w->xrx, qs1d, sizeof(double) * nz);
  snow_check_and_update(nz, w->rho, w->l_qs, w->xrx, w->rs, w->qsten, dt, odt);
  for (k = 0; k < nz; k++) {
    w->smo0[k] = w->smo1[k] = w->smo2[k] = w->smob[k] = w->smoc[k] = 0.0;
    w->smoe[k] = w->smof[k] = w->smog[k] = w->ns[k] = 0.0;
    if (w->l_qs[k]) snow_moments_all(w, k, 0);
  }
  memcpy(w->xrx, qg1d, sizeof(double) * nz);
  double *xngx = NULL, *xqbx = NULL;
  if (hail_ng_qb) {
    memcpy(w->xngx, ng1d, sizeof(double) * nz);
    memcpy(w->xqbx, qb1d, sizeof(double) * nz);
    xngx = w->xngx;
    xqbx = w->xqbx;
  }
  graupel_check_and_update(nz, w->rho, w->l_qg, w->xrx, xngx, xqbx, w->rg, w->ng, w->rb, w->idx_bg,
                           w->qgten, w->ngten, w->qbten, w->ilamg, w->mvd_g, dt, odt);
  thermo_vars(w, &supersaturated);

  if (!cfg->turn_off_micro_flag && cfg->cloud_condensation_flag) { /* :530-560 */
    cloud_condensation(w, w1d, nwfa1d, have_ncsave, dt, odt);
    for (k = 0; k < nz; k++) {
      w->qvten[k] = w->qvten[k] - TD(PRW_VCD);
      w->qcten[k] = w->qcten[k] + TD(PRW_VCD);
      w->ncten[k] = w->ncten[k] + TD(PNC_WCD);
      w->nwfaten[k] = w->nwfaten[k] - TD(PNC_WCD);
      w->tten[k] = w->tten[k] + w->lvap[k] * w->ocp[k] * TD(PRW_VCD);
    }
    memcpy(w->xrx, qc1d, sizeof(double) * nz);
    if (nc1d) memcpy(w->xncx, nc1d, sizeof(double) * nz);
    t_tpass = 2;
    cloud_check_and_update(nz, w->rho, w->l_qc, w->xrx, xncx, have_ncsave ? w->ncsave : NULL,
                           w->rc, w->nc, w->qcten, w->ncten, w->ilamc, w->mvd_c, dt, odt);
    for (k = 0; k < nz; k++) {
      w->qv[k] = fmax2(min_qv, qv1d[k] + w->qvten[k] * dt);
      w->temp[k] = t1d[k] + w->tten[k] * dt;
      w->rho[k] = roverrv * w->pres[k] / (rdry * w->temp[k] * (w->qv[k] + roverrv));
    }
    thermo_vars(w, &supersaturated);
  }
  if (!cfg->turn_off_micro_flag) { /* :563-588 */
    rain_evaporation(w, odt);
    for (k = 0; k < nz; k++) {
      w->qrten[k] = w->qrten[k] - TD(PRV_REV);
      w->qvten[k] = w->qvten[k] + TD(PRV_REV);
      w->nrten[k] = w->nrten[k] - TD(PNR_REV);
      w->nwfaten[k] = w->nwfaten[k] + TD(PNR_REV);
      w->tten[k] = w->tten[k] - w->lvap[k] * w->ocp[k] * TD(PRV_REV);
    }
    memcpy(w->xrx, qr1d, sizeof(double) * nz);
    memcpy(w->xnx, nr1d, sizeof(double) * nz);
    t_tpass = 3;
    rain_check_and_update(nz, w->rho, w->l_qr, w->xrx, w->xnx, w->rr, w->nr, w->qrten, w->nrten,
                          w->ilamr, w->mvd_r, dt, odt);
    for (k = 0; k < nz; k++) {
      w->qv[k] = fmax2(min_qv, qv1d[k] + w->qvten[k] * dt);
      w->temp[k] = t1d[k] + w->tten[k] * dt;
      w->rho[k] = roverrv * w->pres[k] / (rdry * w->temp[k] * (w->qv[k] + roverrv));
    }
    thermo_vars(w, &supersaturated);
  }

  /* :593-727 sedimentation */
  int ktop, steps, any;
  any = 0;
  for (k = 0; k < nz; k++) any |= w->l_qr[k];
  if (any) {
    rain_fallspeed(nz, w->rhof, w->rr, w->ilamr, dz1d, w->vtrr, w->vtnr, &steps, &ktop, dt);
    TRACE_COL(0, steps);
    TRACE_COL(4, ktop);
    if (cfg->semi_sedi_flag) { /* :599-613 */
      steps = imax((int)(steps / semi_sedi_factor) + 1, 1);
      md->substeps[0] = steps;
      for (int n = 1; n <= steps; n++) {
        semilagrangian_sedimentation(nz, dz1d, w->rho, w->rr, w->qrten, w->vtrr, steps, r1,
                                     &md->rain_precip, dt, odt);
        semilagrangian_sedimentation(nz, dz1d, w->rho, w->nr, w->nrten, w->vtnr, steps, r2, NULL,
                                     dt, odt);
        memset(w->vtrr, 0, sizeof(double) * (nz + 1));
        memset(w->vtnr, 0, sizeof(double) * (nz + 1));
        memcpy(w->xrx, qr1d, sizeof(double) * nz);
        memcpy(w->xnx, nr1d, sizeof(double) * nz);
        rain_check_and_update(nz, w->rho, w->l_qr, w->xrx, w->xnx, w->rr, w->nr, w->qrten,
                              w->nrten, w->ilamr, w->mvd_r, dt, odt);
        rain_fallspeed(nz, w->rhof, w->rr, w->ilamr, dz1d, w->vtrr, w->vtnr, NULL, NULL, dt);
      }
    } else {
      md->substeps[0] = steps;
      for (int n = 1; n <= steps; n++) {
        sedimentation(nz, w->rr, w->vtrr, dz1d, w->rho, w->qrten, r1, steps, ktop, &md->rain_precip,
                      dt, w->sed_r);
        sedimentation(nz, w->nr, w->vtnr, dz1d, w->rho, w->nrten, r2, steps, ktop, NULL, dt, w->sed_r);
      }
    }
  }
  any = 0;
  for (k = 0; k < nz; k++) any |= w->l_qg[k];
  if (any) {
    graupel_fallspeed(nz, w->rhof, w->rho, w->visco, w->rg, w->rb, qb1d != NULL, w->idx_bg,
                      w->ilamg, dz1d, w->vtrg, w->vtng, &steps, &ktop, dt);
    TRACE_COL(1, steps);
    TRACE_COL(5, ktop);
    if (cfg->semi_sedi_flag) { /* :640-671 */
      steps = imax((int)(steps / semi_sedi_factor) + 1, 1);
      md->substeps[1] = steps;
      for (int n = 1; n <= steps; n++) {
        semilagrangian_sedimentation(nz, dz1d, w->rho, w->rg, w->qgten, w->vtrg, steps, r1,
                                     &md->graupel_liquid_equiv_precip, dt, odt);
        semilagrangian_sedimentation(nz, dz1d, w->rho, w->ng, w->ngten, w->vtng, steps, r2, NULL,
                                     dt, odt);
        semilagrangian_sedimentation(nz, dz1d, w->rho, w->rb, w->qbten, w->vtrg, steps,
                                     meters3_to_liters * r1 / RHO_G(nrhg), NULL, dt, odt);
        memset(w->vtrg, 0, sizeof(double) * (nz + 1));
        memset(w->vtng, 0, sizeof(double) * (nz + 1));
        memcpy(w->xrx, qg1d, sizeof(double) * nz);
        double *xngx = NULL, *xqbx = NULL;
        if (hail_ng_qb) {
          memcpy(w->xngx, ng1d, sizeof(double) * nz);
          memcpy(w->xqbx, qb1d, sizeof(double) * nz);
          xngx = w->xngx;
          xqbx = w->xqbx;
        }
        graupel_check_and_update(nz, w->rho, w->l_qg, w->xrx, xngx, xqbx, w->rg, w->ng, w->rb,
                                 w->idx_bg, w->qgten, w->ngten, w->qbten, w->ilamg, w->mvd_g, dt, odt);
        graupel_fallspeed(nz, w->rhof, w->rho, w->visco, w->rg, w->rb, qb1d != NULL, w->idx_bg,
                          w->ilamg, dz1d, w->vtrg, w->vtng, NULL, NULL, dt);
      }
    } else {
      md->substeps[1] = steps;
      for (int n = 1; n <= steps; n++) {
        sedimentation(nz, w->rg, w->vtrg, dz1d, w->rho, w->qgten, r1, steps, ktop,
                      &md->graupel_liquid_equiv_precip, dt, w->sed_r);
        sedimentation(nz, w->ng, w->vtng, dz1d, w->rho, w->ngten, r2, steps, ktop, NULL, dt, w->sed_r);
        sedimentation(nz, w->rb, w->vtrg, dz1d, w->rho, w->qbten, meters3_to_liters * r1 / RHO_G(nrhg),
                      steps, ktop, NULL, dt, w->sed_r);
      }
    }
  }
  any = 0;
  for (k = 0; k < nz; k++) any |= w->l_qs[k];
  if (any) {
    snow_fallspeed(nz, w->rhof, w->rs, tw + (long)PRR_SML * nz, w->smob, w->smoc, w->rr, w->vtrr,
                   dz1d, w->vtrs, w->vtboost, &steps, &ktop, dt);
    TRACE_COL(2, steps);
    TRACE_COL(6, ktop);
    md->substeps[2] = steps;
    for (int n = 1; n <= steps; n++)
      sedimentation(nz, w->rs, w->vtrs, dz1d, w->rho, w->qsten, r1, steps, ktop,
                    &md->snow_liquid_equiv_precip, dt, w->sed_r);
  }
  any = 0;
  for (k = 0; k < nz; k++) any |= w->l_qi[k];
  if (any) {
    ice_fallspeed(nz, w->rhof, w->ri, w->ilami, dz1d, w->vtri, w->vtni, &steps, &ktop, dt);
    TRACE_COL(3, steps);
    TRACE_COL(7, ktop);
    md->substeps[3] = steps;
    sedimentation(nz, w->ri, w->vtri, dz1d, w->rho, w->qiten, r1, steps, ktop,
                  &md->ice_liquid_equiv_precip, dt, w->sed_r);
    sedimentation(nz, w->ni, w->vtni, dz1d, w->rho, w->niten, r2, steps, ktop, NULL, dt, w->sed_r);
  }
  any = 0;
  for (k = 0; k < nz; k++) any |= w->l_qc[k];
  if (any) {
    cloud_fallspeed(nz, w->rhof, w1d, w->rc, w->nc, w->ilamc, dz1d, w->vtrc, w->vtnc, &ktop);
    TRACE_COL(8, ktop);
    md->substeps[4] = 1;
    sedimentation(nz, w->rc, w->vtrc, dz1d, w->rho, w->qcten, r1, 1, ktop, &md->cloud_precip, dt,
                  w->sed_r);
    sedimentation(nz, w->nc, w->vtnc, dz1d, w->rho, w->ncten, r2, 1, ktop, NULL, dt, w->sed_r);
  }

  if (!cfg->turn_off_micro_flag) /* :731-735 */
    freeze_cloud_melt_ice(w, qi1d, ni1d, qc1d, nc1d, have_ncsave, dt, odt);

  for (k = 0; k < nz; k++) { /* :738-748 */
    t1d[k] = t1d[k] + w->tten[k] * dt;
    qv1d[k] = fmax2(min_qv, (qv1d[k] + w->qvten[k] * dt));
    w->rho[k] = roverrv * w->pres[k] / (rdry * w->temp[k] * (w->qv[k] + roverrv));
    if (nwfa1d) nwfa1d[k] = fmax2(nwfa_default, fmin2(aero_max, (nwfa1d[k] + w->nwfaten[k] * dt)));
    if (nifa1d) nifa1d[k] = fmax2(nifa_default, fmin2(aero_max, (nifa1d[k] + w->nifaten[k] * dt)));
  }
  t_tpass = 4;
  cloud_check_and_update(nz, w->rho, w->l_qc, qc1d, nc1d, have_ncsave ? w->ncsave : NULL, w->rc,
                         w->nc, w->qcten, w->ncten, w->ilamc, w->mvd_c, dt, odt);
  rain_check_and_update(nz, w->rho, w->l_qr, qr1d, nr1d, w->rr, w->nr, w->qrten, w->nrten, w->ilamr,
                        w->mvd_r, dt, odt);
  ice_check_and_update(nz, w->rho, w->l_qi, qi1d, ni1d, w->ri, w->ni, w->qiten, w->niten, w->ilami,
                       dt, odt);
  snow_check_and_update(nz, w->rho, w->l_qs, qs1d, w->rs, w->qsten, dt, odt);
  for (k = 0; k < nz; k++) {
    w->smo0[k] = w->smo1[k] = w->smo2[k] = w->smob[k] = w->smoc[k] = 0.0;
    w->smoe[k] = w->smof[k] = w->smog[k] = w->smoz[k] = w->ns[k] = 0.0;
    if (w->l_qs[k]) snow_moments_all(w, k, 2);
  }
  t_tie_bit = 2; /* a tie in the final check moves only this level's graupel diagnostics */
  graupel_check_and_update(nz, w->rho, w->l_qg, qg1d, ng1d, qb1d, w->rg, w->ng, w->rb, w->idx_bg,
                           w->qgten, w->ngten, w->qbten, w->ilamg, w->mvd_g, dt, odt);

  /* :785-863 diagnostics */
  md->frozen_fraction =
      (md->ice_liquid_equiv_precip + md->snow_liquid_equiv_precip + md->graupel_liquid_equiv_precip) /
      (md->ice_liquid_equiv_precip + md->snow_liquid_equiv_precip + md->graupel_liquid_equiv_precip +
       md->rain_precip + r1);
  md->frz_rain_precip = 0.0;
  if ((w->temp[0] - t0) < -0.5) md->frz_rain_precip = md->rain_precip + md->cloud_precip;
  if (co->ncmr)
    for (k = 0; k < nz; k++) co->ncmr[k] = w->nc[k] * w->rho[k];
  if (co->mvd_r)
    for (k = 0; k < nz; k++) co->mvd_r[k] = w->mvd_r[k];
  if (co->mvd_g)
    for (k = 0; k < nz; k++) co->mvd_g[k] = w->mvd_g[k];
  if (co->mhd) max_hail_diam(w, co->mhd);
  if (co->refl) reflectivity_10cm(w, co->refl, cfg->refl10cm_from_melting_flag);
  if (co->re_c) {
    if (co->qc_bl && co->qcfrac_bl) {
      /* :832-857: the in-cloud boundary-layer water joins the resolved cloud, the network
       * predicts its number, and the cloud check recomputes rc, nc and ilamc for the
       * effective radius (the state of the step is not touched) */
      for (k = 0; k < nz; k++) {
        double xq = qc1d[k];
        if (xq <= r1 && co->qc_bl[k] > 1.e-9 && co->qcfrac_bl[k] > 0.0) xq = xq + co->qc_bl[k] / co->qcfrac_bl[k];
        if (xq <= 1.e-12) xq = 0.0;
        w->xrx[k] = xq;
        w->xncx[k] = ml_predict_nc(xq, qr1d[k], qi1d[k], qs1d[k], w->pres[k], w->temp[k], w1d[k]);
        w->qcten[k] = 0.0;
        w->ncten[k] = 0.0;
      }
      cloud_check_and_update(nz, w->rho, w->l_qc, w->xrx, w->xncx, NULL, w->rc, w->nc, w->qcten,
                             w->ncten, w->ilamc, w->mvd_c, dt, odt);
    }
    effective_radius(w, co->re_c, co->re_i, co->re_s);
  }
}

/* ------------------------------------------------------------------------------ */
/* tempo_run (driver:187-513)                                                       */
/* ------------------------------------------------------------------------------ */
static long g_stats[8];

void oracle_last_stats(long out[8]) { memcpy(out, g_stats, sizeof g_stats); }

int oracle_run(const ocfg_t *cfg, double dt, int itimestep, double *t, double *th,
               const double *pii, const double *p, const double *w3, const double *dz, double *qv,
               double *qc, double *qr, double *qi, double *qs, double *qg, double *ni, double *nr,
               double *nc, double *nwfa, double *nifa, double *ng, double *qb, const double *qc_bl,
               const double *qcfrac_bl, const int *land_input, const int b[18], odiag_t *dg,
               int nthreads) {
  int ims = b[6], ime = b[7], jms = b[8], jme = b[9], kms = b[10], kme = b[11];
  int its = b[12], ite = b[13], jts = b[14], jte = b[15], kts = b[16], kte = b[17];
  (void)jme;
  if (cfg->ml_for_nc_flag && !nc && !ml_loaded) return -3;
  if (qc_bl && qcfrac_bl && !ml_loaded) return -3;
  if (!t && !(th && pii)) return -2;
  int nz = kte - kts + 1;
  long ni_ = ime - ims + 1, nk_ = kme - kms + 1;
  long ti = ite - its + 1, tk = kte - kts + 1;
#define I3(i, k, j) (((long)(i)-ims) + ((long)(k)-kms) * ni_ + ((long)(j)-jms) * ni_ * nk_)
#define T2(i, j) (((long)(i)-its) + ((long)(j)-jts) * ti)
#define T3(i, k, j) (((long)(i)-its) + ((long)(k)-kts) * ti + ((long)(j)-jts) * ti * tk)
  int use_temperature = t != NULL;
  int is_first_step = (itimestep == 1);
  long ncols = (long)(ite - its + 1) * (jte - jts + 1);
  long early = 0, maxsub[5] = {0, 0, 0, 0, 0};
  /* driver:302-386: reset the diagnostics that tempo_run allocates; a diagnostic whose
   * flag is off is neither allocated nor touched */
  for (long c = 0; c < ncols; c++) {
    double *d2[] = {dg->rain_precip, dg->ice_liquid_equiv_precip, dg->snow_liquid_equiv_precip,
                    dg->graupel_liquid_equiv_precip, dg->frozen_fraction, dg->frz_rain_precip,
                    dg->max_hail_diameter_sfc, dg->max_hail_diameter_column};
    for (int a = 0; a < 8; a++)
      if (d2[a] && (a < 6 || cfg->max_hail_diameter_flag)) d2[a][c] = 0.0;
  }
  long n3 = ncols * tk;
  for (long c = 0; c < n3; c++) {
    if (dg->refl10cm && cfg->refl10cm_flag) dg->refl10cm[c] = -35.0;
    double *d3[] = {dg->re_cloud, dg->re_ice, dg->re_snow, dg->rain_med_vol_diam,
                    dg->graupel_med_vol_diam, dg->cloud_number_mixing_ratio};
    const int on3[] = {cfg->re_cloud_flag, cfg->re_ice_flag, cfg->re_snow_flag,
                       cfg->rain_med_vol_diam_flag, cfg->graupel_med_vol_diam_flag,
                       cfg->cloud_number_mixing_ratio_flag};
    for (int a = 0; a < 6; a++)
      if (d3[a] && on3[a]) d3[a][c] = 0.0;
  }
  if (nthreads > 0) {
#ifdef _OPENMP
    omp_set_num_threads(nthreads);
#endif
  }
#pragma omp parallel reduction(+ : early)
  {
    ws_t *w = ws_new(nz);
    double *buf = (double *)calloc((size_t)nz * 32, sizeof(double));
    double *qcbl1d = buf + 30 * nz, *qcfbl1d = buf + 31 * nz;
    double *t1d = buf, *p1d = buf + nz, *w1d = buf + 2 * nz, *dz1d = buf + 3 * nz,
           *qv1d = buf + 4 * nz, *qc1d = buf + 5 * nz, *qi1d = buf + 6 * nz, *qr1d = buf + 7 * nz,
           *qs1d = buf + 8 * nz, *qg1d = buf + 9 * nz, *ni1d = buf + 10 * nz, *nr1d = buf + 11 * nz,
           *nc1d = buf + 12 * nz, *nwfa1d = buf + 13 * nz, *nifa1d = buf + 14 * nz,
           *ng1d = buf + 15 * nz, *qb1d = buf + 16 * nz;
    double *o_refl = buf + 17 * nz, *o_rec = buf + 18 * nz, *o_rei = buf + 19 * nz,
           *o_res = buf + 20 * nz, *o_mvr = buf + 21 * nz, *o_mvg = buf + 22 * nz,
           *o_mhd = buf + 23 * nz, *o_ncm = buf + 24 * nz;
    long lmax[5] = {0, 0, 0, 0, 0};
#pragma omp for schedule(dynamic, 16)
    for (long c = 0; c < ncols; c++) {
      int i = its + (int)(c % (ite - its + 1));
      int j = jts + (int)(c / (ite - its + 1));
      for (int k = kts; k <= kte; k++) {
        int k0 = k - kts;
        long a = I3(i, k, j);
        t1d[k0] = use_temperature ? t[a] : th[a] * pii[a];
        p1d[k0] = p[a];
        w1d[k0] = w3[a];
        dz1d[k0] = dz[a];
        qv1d[k0] = qv[a];
        qc1d[k0] = qc[a];
        qi1d[k0] = qi[a];
        qr1d[k0] = qr[a];
        qs1d[k0] = qs[a];
        qg1d[k0] = qg[a];
        ni1d[k0] = ni[a];
        nr1d[k0] = nr[a];
        if (nwfa) nwfa1d[k0] = nwfa[a];
        if (nifa) nifa1d[k0] = nifa[a];
        if (nc) nc1d[k0] = nc[a];
        if (ng && qb) {
          ng1d[k0] = ng[a];
          qb1d[k0] = qb[a];
        }
        if (qc_bl && qcfrac_bl) {
          qcbl1d[k0] = qc_bl[a];
          qcfbl1d[k0] = qcfrac_bl[a];
        }
      }
      int land1d = 0;
      if (land_input) land1d = land_input[((long)i - ims) + ((long)j - jms) * ni_];
      colout_t co = {0};
      co.refl = (cfg->refl10cm_flag && dg->refl10cm) ? o_refl : NULL;
      int all_re = cfg->re_cloud_flag && cfg->re_ice_flag && cfg->re_snow_flag;
      co.re_c = all_re ? o_rec : NULL;
      co.re_i = all_re ? o_rei : NULL;
      co.re_s = all_re ? o_res : NULL;
      co.mvd_r = cfg->rain_med_vol_diam_flag ? o_mvr : NULL;
      co.mvd_g = cfg->graupel_med_vol_diam_flag ? o_mvg : NULL;
      co.mhd = cfg->max_hail_diameter_flag ? o_mhd : NULL;
      co.ncmr = cfg->cloud_number_mixing_ratio_flag ? o_ncm : NULL;
      co.qc_bl = (qc_bl && qcfrac_bl) ? qcbl1d : NULL;
      co.qcfrac_bl = (qc_bl && qcfrac_bl) ? qcfbl1d : NULL;
      mdiag_t md;
      t_tie = 0;
      t_tie_bit = 1;
      {
        const long ct = (long)(i - its) + (long)(j - jts) * (ite - its + 1);
        t_trace = g_trace ? g_trace + ct * nz * TRP : NULL;
        t_trace_col = g_trace ? g_trace + ncols * nz * TRP + ct * TRC : NULL;
      }
      tempo_main_col(cfg, is_first_step, qv1d, qc1d, qi1d, qr1d, qs1d, qg1d, qb ? qb1d : NULL,
                     ni1d, nr1d, nc ? nc1d : NULL, ng ? ng1d : NULL, nwfa ? nwfa1d : NULL,
                     nifa ? nifa1d : NULL, t1d, p1d, w1d, dz1d, land_input ? &land1d : NULL, dt, w,
                     &md, &co);
      if (md.early_exit) early++;
      for (int s = 0; s < 5; s++)
        if (md.substeps[s] > lmax[s]) lmax[s] = md.substeps[s];
      long c2 = T2(i, j);
      if (g_tie_sink) g_tie_sink[c2] = t_tie;
      if (dg->rain_precip) dg->rain_precip[c2] = md.rain_precip;
      if (dg->ice_liquid_equiv_precip) dg->ice_liquid_equiv_precip[c2] = md.ice_liquid_equiv_precip;
      if (dg->snow_liquid_equiv_precip) dg->snow_liquid_equiv_precip[c2] = md.snow_liquid_equiv_precip;
      if (dg->graupel_liquid_equiv_precip)
        dg->graupel_liquid_equiv_precip[c2] = md.graupel_liquid_equiv_precip;
      /* early-exit columns keep 0 (the reference leaves intent(out) frozen_fraction stale) */
      if (dg->frozen_fraction) dg->frozen_fraction[c2] = md.early_exit ? 0.0 : md.frozen_fraction;
      if (dg->frz_rain_precip) dg->frz_rain_precip[c2] = md.frz_rain_precip;
      if (!md.early_exit) {
        for (int k = kts; k <= kte; k++) {
          int k0 = k - kts;
          long c3 = T3(i, k, j);
          if (dg->cloud_number_mixing_ratio && co.ncmr) dg->cloud_number_mixing_ratio[c3] = o_ncm[k0];
          if (dg->rain_med_vol_diam && co.mvd_r) dg->rain_med_vol_diam[c3] = o_mvr[k0];
          if (dg->graupel_med_vol_diam && co.mvd_g) dg->graupel_med_vol_diam[c3] = o_mvg[k0];
          if (dg->re_cloud && co.re_c) dg->re_cloud[c3] = o_rec[k0];
          if (dg->re_ice && co.re_i) dg->re_ice[c3] = o_rei[k0];
          if (dg->re_snow && co.re_s) dg->re_snow[c3] = o_res[k0];
          if (dg->refl10cm && co.refl) dg->refl10cm[c3] = o_refl[k0];
        }
        if (dg->max_hail_diameter_sfc && dg->max_hail_diameter_column && co.mhd) {
          double mx = o_mhd[0];
          for (int k0 = 1; k0 < nz; k0++)
            if (o_mhd[k0] > mx) mx = o_mhd[k0];
          dg->max_hail_diameter_sfc[c2] = o_mhd[0];
          dg->max_hail_diameter_column[c2] = mx;
        }
      }
      for (int k = kts; k <= kte; k++) {
        int k0 = k - kts;
        long a = I3(i, k, j);
        if (nc) nc[a] = nc1d[k0];
        if (nwfa) nwfa[a] = nwfa1d[k0];
        if (nifa) nifa[a] = nifa1d[k0];
        if (ng && qb) {
          ng[a] = ng1d[k0];
          qb[a] = qb1d[k0];
        }
        qv[a] = qv1d[k0];
        qc[a] = qc1d[k0];
        qi[a] = qi1d[k0];
        qr[a] = qr1d[k0];
        qs[a] = qs1d[k0];
        qg[a] = qg1d[k0];
        ni[a] = ni1d[k0];
        nr[a] = nr1d[k0];
        if (use_temperature)
          t[a] = t1d[k0];
        else
          th[a] = t1d[k0] / pii[a];
      }
    }
#pragma omp critical
    for (int s = 0; s < 5; s++)
      if (lmax[s] > maxsub[s]) maxsub[s] = lmax[s];
    free(buf);
    ws_free(w);
  }
  g_stats[0] = ncols;
  g_stats[1] = early;
  for (int s = 0; s < 5; s++) g_stats[2 + s] = maxsub[s];
#undef I3
#undef T2
#undef T3
  return 0;
}

/* unit-test exports of the table-index routines (main:23-27 under -Dunit_testing) */
void oracle_get_cloud_table_index(double rc, double nc, int *a, int *b) { get_cloud_table_index(rc, nc, a, b); }
void oracle_get_snow_table_index(double rs, int *a) { get_snow_table_index(rs, a); }
void oracle_get_temperature_table_index(double tk, int *a) { get_temperature_table_index(tk, a); }
void oracle_get_rain_table_index(double rr, double il, int *a, int *b) { get_rain_table_index(rr, il, a, b); }
void oracle_get_graupel_table_index(double rg, double il, int idx, int *a, int *b) {
  get_graupel_table_index(rg, il, idx, a, b);
}
void oracle_get_ice_table_index(double ri, double ni, int *a, int *b) { get_ice_table_index(ri, ni, a, b); }
