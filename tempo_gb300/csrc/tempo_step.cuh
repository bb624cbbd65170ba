// tempo_step.cuh -- the TEMPO column step (tempo_run -> tempo_main) as one sm_103a kernel.
//
// One thread owns one column of the host's (ims:ime, kms:kme, jms:jme) arrays; with
// i fastest, the 32 threads of a warp read and write 32 consecutive columns of a
// level, so every global access is coalesced.  The step runs in three phases:
//
//   A  pointwise physics, level by level (main:321-588): initial checks, process
//      rates, limiter, tendency sums, provisional update, saturation adjustment,
//      rain evaporation, and each species' fall-speed candidate;
//   B  the vertically coupled part (main:593-727): fall-speed fill from above,
//      CFL substep counts, and the explicit upwind sedimentation sweeps;
//   C  pointwise again (main:731-863): instant freeze/melt, final update and
//      checks, diagnostics.
//
// The per-level state that crosses phases lives in a scratch buffer laid out
// [field][level][column] (column fastest, coalesced); the prognostic arrays
// themselves carry the checked values between A and C, as tempo_main's inout
// 1-D arrays do.  Columns whose early-exit test holds (main:417-418) only run the
// initial checks.
#pragma once

#include "tempo_rates.cuh"

namespace tg {

template <class S> __device__ __forceinline__ D ldd(const S* p) { return D(*p); }

template <class R, class S>
__global__ void __launch_bounds__(128) tempo_column_kernel(const __grid_constant__ StepArgs<S> a,
                                                            const __grid_constant__ Tables<R> T,
                                                            const __grid_constant__ TempoConsts<R> cst,
                                                            const __grid_constant__ TempoConsts<D> cstd) {
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.ncol) return;
  const int ii = (int)(c % a.ti), jj = (int)(c / a.ti);
  const long NI = a.NI;
  const long base = (long)(a.i0 + ii) + (long)a.k0 * NI + (long)(a.j0 + jj) * NI * a.NK;
  const int nz = a.nz;
  const uint32_t f = a.flags;
  const bool has_nc = f & F_NC, has_nwfa = f & F_NWFA, has_nifa = f & F_NIFA, hail = f & F_HAIL;
  const bool use_t = f & F_USE_T;
  const R dt = R(a.dt), odt = R(1.0 / a.dt);
  const D dtd = a.dt;
  const long tile2 = (long)ii + (long)jj * a.ti;
  auto at = [&](int k) { return base + (long)k * NI; };
  auto tile3 = [&](int k) { return (long)ii + (long)k * a.ti + (long)jj * a.ti * nz; };

  // ncsave: single-moment cloud number when nc is absent (main:364-380)
  R ncsave = R(nt_c_l);
  if (!has_nc) {
    if (f & F_LAND)
      ncsave = (a.land[(long)(a.i0 + ii) + (long)(a.j0 + jj) * NI] != 1) ? R(nt_c_o) : R(nt_c_l);
    else
      ncsave = R(a.nc_single);
  }
  const R ncsave_cond = has_nc ? R(nt_c_l) : ncsave;

  // ---- pre-pass: early-exit test and first-step column sums ----
  bool do_micro = false, supersat = false;
  D sqg = 0, sng = 0, sqb = 0;
  for (int k = 0; k < nz; k++) {
    const long e = at(k);
    D t1 = use_t ? ldd(a.t + e) : ldd(a.th + e) * ldd(a.pii + e);
    D qv = Max(min_qv, ldd(a.qv + e));
    D p = ldd(a.p + e);
    do_micro |= (ldd(a.qc + e) > r1) | (ldd(a.qr + e) > r1) | (ldd(a.qi + e) > r1) |
                (ldd(a.qs + e) > r1) | (ldd(a.qg + e) > r1);
    D qvsi = (t1 - t0 <= 0.0) ? calc_rsif(p, t1) : calc_rslf(p, t1);
    D ssati = qv / qvsi - 1.0;
    if (Fabs(ssati) < eps) ssati = 0.0;
    supersat |= ssati > 0.0;
    if (hail && (f & F_FIRST)) {
      sqg = sqg + ldd(a.qg + e);
      sng = sng + ldd(a.ng + e);
      sqb = sqb + ldd(a.qb + e);
    }
  }
  const bool do_ginit = hail && (f & F_FIRST) && sqg > r1 && sng < eps && sqb < eps;
  const bool early = !do_micro && !supersat;

  auto load_level = [&](Lev<R>& L, int k) {
    const long e = at(k);
    L.t1d = use_t ? ldd(a.t + e) : ldd(a.th + e) * ldd(a.pii + e);
    L.qv1d = ldd(a.qv + e);
    L.pres = R(a.p[e]);
    L.qc1d = R(a.qc[e]);
    L.qr1d = R(a.qr[e]);
    L.qi1d = R(a.qi[e]);
    L.qs1d = R(a.qs[e]);
    L.qg1d = R(a.qg[e]);
    L.ni1d = R(a.ni[e]);
    L.nr1d = R(a.nr[e]);
    L.nc1d = has_nc ? R(a.nc[e]) : R(0);
    L.ng1d = hail ? R(a.ng[e]) : R(0);
    L.qb1d = hail ? R(a.qb[e]) : R(0);
    L.temp = L.t1d;
    L.qv = Max(min_qv, L.qv1d);
    L.rho = rho_of(cstd, D(L.pres), L.temp, L.qv);
    L.tten = L.qvten = 0.0;
    L.qcten = L.ncten = L.qiten = L.niten = L.qrten = L.nrten = L.qsten = L.qgten = L.ngten =
        L.qbten = L.nwfaten = L.nifaten = R(0);
    L.smob = L.smoc = L.smo0 = L.smo1 = L.smo2 = L.smoe = L.smof = L.smog = L.smoz = R(0);
    L.vtboost = R(1);
  };
  auto initial_checks = [&](Lev<R>& L) {
    rain_check(L, L.qr1d, L.nr1d, dt, odt);
    ice_check(L, L.qi1d, L.ni1d, dt, odt);
    snow_check(L, L.qs1d, dt, odt);
    if (L.l_qs) snow_moments(L, R(Min(-0.1, L.temp - t0)), 1);
    if (!has_nc) L.nc = ncsave;
    cloud_check(L, L.qc1d, L.nc1d, has_nc, ncsave, dt, odt);
    if (do_ginit) graupel_init(L);
    graupel_check(L, L.qg1d, L.ng1d, L.qb1d, hail, dt, odt);
  };
  auto store_checked = [&](const Lev<R>& L, int k) {
    const long e = at(k);
    a.qc[e] = S(L.qc1d);
    a.qr[e] = S(L.qr1d);
    a.nr[e] = S(L.nr1d);
    a.qi[e] = S(L.qi1d);
    a.ni[e] = S(L.ni1d);
    a.qs[e] = S(L.qs1d);
    a.qg[e] = S(L.qg1d);
    if (has_nc) a.nc[e] = S(L.nc1d);
    if (hail) {
      a.ng[e] = S(L.ng1d);
      a.qb[e] = S(L.qb1d);
    }
  };
  auto diag_defaults = [&]() {
    if (a.rain_precip) a.rain_precip[tile2] = S(0);
    if (a.ice_precip) a.ice_precip[tile2] = S(0);
    if (a.snow_precip) a.snow_precip[tile2] = S(0);
    if (a.graupel_precip) a.graupel_precip[tile2] = S(0);
    if (a.frozen_fraction) a.frozen_fraction[tile2] = S(0);
    if (a.frz_rain) a.frz_rain[tile2] = S(0);
    if (a.mhd_sfc) a.mhd_sfc[tile2] = S(0);
    if (a.mhd_col) a.mhd_col[tile2] = S(0);
    for (int k = 0; k < nz; k++) {
      const long e3 = tile3(k);
      if (a.refl10cm) a.refl10cm[e3] = S(-35.0);
      if (a.re_cloud) a.re_cloud[e3] = S(0);
      if (a.re_ice) a.re_ice[e3] = S(0);
      if (a.re_snow) a.re_snow[e3] = S(0);
      if (a.mvd_r) a.mvd_r[e3] = S(0);
      if (a.mvd_g) a.mvd_g[e3] = S(0);
      if (a.ncmr) a.ncmr[e3] = S(0);
    }
  };

  if (early) {
    for (int k = 0; k < nz; k++) {
      Lev<R> L;
    L.cs = &cst;
    L.cd = &cstd;
      load_level(L, k);
      initial_checks(L);
      store_checked(L, k);
    }
    diag_defaults();
    atomicAdd(a.stats, 1ull);
    return;
  }

  // ---------------- phase A ----------------
  double* sd = a.sd + c;
  R* sr = reinterpret_cast<R*>(a.sr) + c;
  const long cs = a.ncol_pad;                 // stride between levels
  const long fsd = (long)nz * cs;             // stride between fields
  bool any_qr = false, any_qg = false, any_qs = false, any_qi = false, any_qc = false;
  // aerosol initial profiles (init_*_friendly_aerosols, aerosols:14-73): hgt(1) = 0,
  // so h_01 = 0.8 and the k = 1 value uses hgt(2)
  D hgt = 0.0, hgt2 = 0.0;
  const D h_01 = 0.8;
  const D niccn3 = -1.0 * log(naccn1 / naccn0) / h_01;
  const D niin3 = -1.0 * log(nain1 / nain0) / h_01;
  if (nz > 1) hgt2 = ldd(a.dz + at(1));

  for (int k = 0; k < nz; k++) {
    const long e = at(k);
    Lev<R> L;
    L.cs = &cst;
    L.cd = &cstd;
    load_level(L, k);
    const R w = R(a.w[e]);
    if (k > 0) hgt = hgt + ldd(a.dz + e);
    const D hk = (k == 0) ? hgt2 : hgt;
    const R nwfa_in = has_nwfa ? R(a.nwfa[e]) : R(naccn1 + naccn0 * exp(-(hk / 1000.0) * niccn3));
    const R nifa_in = has_nifa ? R(a.nifa[e]) : R(nain1 + nain0 * exp(-(hk / 1000.0) * niin3));
    L.nwfa = nwfa_in;
    L.nifa = nifa_in;
    aerosol_check(L, f, dt);
    initial_checks(L);
    L.qcten = L.qiten = L.qrten = L.qsten = L.qgten = L.ngten = L.qbten = L.niten = L.nrten =
        L.ncten = R(0);
    thermo(L);

    Tend<R> td = {};
    if (!(f & F_NOMICRO)) {
      warm_rain(L, td, T, odt);
      rain_snow_rain_graupel(L, td, T, odt);
      ice_nucleation(L, td, T, w, f, dt, odt);
      const R t1s = t1_subl_of(L);
      ice_processes(L, td, T, w, t1s, odt);
      riming(L, td, T, odt);
      melting(L, td, t1s, f, dt, odt);
      if (has_nwfa || has_nifa) aerosol_scavenging(L, td, odt);
    }
    check_over_depletion(L, td, odt);
    sum_tendencies(L, td);

    // provisional update (main:460-468)
    L.temp = L.t1d + L.tten * dtd;
    L.qv = Max(min_qv, L.qv1d + L.qvten * dtd);
    L.rho = rho_of(cstd, D(L.pres), L.temp, L.qv);
    {
      R rho = R(L.rho);
      L.nwfaten = L.nwfaten - (td.pna_rca + td.pna_sca + td.pna_gca + td.pni_iha) / rho;
      L.nifaten = L.nifaten - (td.pnd_rcd + td.pnd_scd + td.pnd_gcd) / rho;
    }
    if (has_nwfa) L.nwfa = nwfa_in;
    if (has_nifa) L.nifa = nifa_in;
    aerosol_check(L, f, dt);

    // checks on temporaries (main:475-522)
    R xq = L.qc1d, xn = L.nc1d, xb;
    cloud_check(L, xq, xn, has_nc, ncsave, dt, odt);
    xq = L.qr1d;
    xn = L.nr1d;
    rain_check(L, xq, xn, dt, odt);
    xq = L.qi1d;
    xn = L.ni1d;
    ice_check(L, xq, xn, dt, odt);
    xq = L.qs1d;
    snow_check(L, xq, dt, odt);
    L.smo0 = L.smo1 = L.smo2 = L.smob = L.smoc = L.smoe = L.smof = L.smog = R(0);
    if (L.l_qs) snow_moments(L, R(Min(-0.1, L.temp - t0)), 0);
    xq = L.qg1d;
    xn = L.ng1d;
    xb = L.qb1d;
    graupel_check(L, xq, xn, xb, hail, dt, odt);
    thermo(L);

    if (!(f & F_NOMICRO) && (f & F_COND)) {  // main:530-560
      cloud_condensation(L, td, T, w, f, ncsave_cond, dt, odt);
      L.qvten = L.qvten - D(td.prw_vcd);
      L.qcten = L.qcten + td.prw_vcd;
      L.ncten = L.ncten + td.pnc_wcd;
      L.nwfaten = L.nwfaten - td.pnc_wcd;
      L.tten = L.tten + D(L.lvap) * D(L.ocp) * D(td.prw_vcd);
      xq = L.qc1d;
      xn = L.nc1d;
      cloud_check(L, xq, xn, has_nc, ncsave, dt, odt);
      L.qv = Max(min_qv, L.qv1d + L.qvten * dtd);
      L.temp = L.t1d + L.tten * dtd;
      L.rho = rho_of(cstd, D(L.pres), L.temp, L.qv);
      thermo(L);
    }
    if (!(f & F_NOMICRO)) {  // main:563-588
      rain_evaporation(L, td, odt);
      L.qrten = L.qrten - td.prv_rev;
      L.qvten = L.qvten + D(td.prv_rev);
      L.nrten = L.nrten - td.pnr_rev;
      L.nwfaten = L.nwfaten + td.pnr_rev;
      L.tten = L.tten - D(L.lvap) * D(L.ocp) * D(td.prv_rev);
      xq = L.qr1d;
      xn = L.nr1d;
      rain_check(L, xq, xn, dt, odt);
      L.qv = Max(min_qv, L.qv1d + L.qvten * dtd);
      L.temp = L.t1d + L.tten * dtd;
      L.rho = rho_of(cstd, D(L.pres), L.temp, L.qv);
      thermo(L);
    }

    // fall-speed candidates (main:1770-1977), unfilled; < 0 marks "absent"
    const TempoConsts<R>& cc = cst;
    R vtr = R(-1), vtnr = R(-1), vtg = R(-1), vtng = R(-1), vsa = R(-1), vsb = R(0);
    R vti = R(-1), vtni = R(-1), vtc = R(0), vtnc = R(0);
    if (L.rr > R(r1)) {
      R lamr = R(1.0) / L.ilamr;
      vtr = L.rhof * R(av_r) * cc.crg[5] * cc.org3 * Pow(lamr, cc.cre[2]) * Pow(lamr + R(fv_r), -cc.cre[5]);
      vtnr = L.rhof * R(av_r) * cc.crg[6] / cc.crg[11] * Pow(lamr, cc.cre[11]) * Pow(lamr + R(fv_r), -cc.cre[6]);
    }
    if (L.rg > R(r1)) {
      R afall, bfall;
      if (f & F_QB) {
        R dens_g = Max(rho_g<R>(1), Min(R(meters3_to_liters) * L.rg / L.rb, rho_g<R>(nrhg)));
        afall = R(a_coeff) * Pow((R(4.0) * dens_g * R(earth_gravity)) / (R(3.0) * R(L.rho)), R(b_coeff));
        afall = afall * Pow(L.visco, R(1.0) - R(2.0) * R(b_coeff));
        bfall = R(3.0) * R(b_coeff) - R(1.0);
      } else {
        afall = R(av_g_old);
        bfall = R(bv_g_old);
      }
      const int ig = L.idx_bg;
      R pb = Pow(L.ilamg, bfall);
      vtg = L.rhof * afall * cc.cgg[ig - 1][5] * cc.ogg3 * pb;
      vtng = L.rhof * afall * cc.cgg[ig - 1][6] / cc.cgg[ig - 1][11] * pb;
    }
    if (L.rs > R(r1)) {
      R xds = L.smoc / L.smob;
      R mrat = R(1.0) / xds;
      R ils1 = R(1.0) / (mrat * R(lam0) + R(fv_s));
      R ils2 = R(1.0) / (mrat * R(lam1) + R(fv_s));
      R mrmu = Pow(mrat, R(mu_s));
      R t1_vts = R(kap0) * cc.csg[3] * Pow(ils1, cc.cse[3]);
      R t2_vts = R(kap1) * mrmu * cc.csg[9] * Pow(ils2, cc.cse[9]);
      ils1 = R(1.0) / (mrat * R(lam0));
      ils2 = R(1.0) / (mrat * R(lam1));
      R t3_vts = R(kap0) * cc.csg[0] * Pow(ils1, cc.cse[0]);
      R t4_vts = R(kap1) * mrmu * cc.csg[6] * Pow(ils2, cc.cse[6]);
      R vts = L.rhof * R(av_s) * (t1_vts + t2_vts) / (t3_vts + t4_vts);
      if (td.prr_sml > R(0.0)) {
        // mixed with the rain speed at fill time, with rr after rain sedimentation
        // (snow_fallspeed is called after the rain sweeps updated rr in place, main:699)
        vsa = vts;
        vsb = R(1.0);
      } else {
        vsa = vts * L.vtboost;
        vsb = R(0);
      }
    }
    if (L.ri > R(r1)) {
      R pb = Pow(L.ilami, R(bv_i));
      vti = L.rhof * R(av_i) * cc.cig[2] * cc.oig2 * pb;
      vtni = L.rhof * R(av_i) * cc.cig[5] / cc.cig[6] * pb;
    }
    if (L.rc > R(r1) && w < R(0.1)) {
      int nu_c = get_nuc(L.nc);
      R pb = Pow(L.ilamc, R(bv_c));
      vtc = L.rhof * R(av_c) * cc.ccg[nu_c - 1][4] * cc.ocg2[nu_c - 1] * pb;
      vtnc = L.rhof * R(av_c) * cc.ccg[nu_c - 1][3] * cc.ocg1[nu_c - 1] * pb;
    }
    any_qr |= L.l_qr;
    any_qg |= L.l_qg;
    any_qs |= L.l_qs;
    any_qi |= L.l_qi;
    any_qc |= L.l_qc;

    const long o = (long)k * cs;
    sd[SD_TTEN * fsd + o] = L.tten;
    sd[SD_QV * fsd + o] = L.qv;
    sd[SD_RHO * fsd + o] = L.rho;
    sd[SD_XRR * fsd + o] = D(L.rr);
    sd[SD_XNR * fsd + o] = D(L.nr);
    sd[SD_XRG * fsd + o] = D(L.rg);
    sd[SD_XNG * fsd + o] = D(L.ng);
    sd[SD_XRB * fsd + o] = D(L.rb);
    sd[SD_XRS * fsd + o] = D(L.rs);
    sd[SD_XRI * fsd + o] = D(L.ri);
    sd[SD_XNI * fsd + o] = D(L.ni);
    sd[SD_XRC * fsd + o] = D(L.rc);
    sd[SD_XNC * fsd + o] = D(L.nc);
    sd[SD_TQR * fsd + o] = D(L.qrten);
    sd[SD_TNR * fsd + o] = D(L.nrten);
    sd[SD_TQG * fsd + o] = D(L.qgten);
    sd[SD_TNG * fsd + o] = D(L.ngten);
    sd[SD_TQB * fsd + o] = D(L.qbten);
    sd[SD_TQS * fsd + o] = D(L.qsten);
    sd[SD_TQI * fsd + o] = D(L.qiten);
    sd[SD_TNI * fsd + o] = D(L.niten);
    sd[SD_TQC * fsd + o] = D(L.qcten);
    sd[SD_TNC * fsd + o] = D(L.ncten);
    sr[SR_VTR * fsd + o] = vtr;
    sr[SR_VTNR * fsd + o] = vtnr;
    sr[SR_VTG * fsd + o] = vtg;
    sr[SR_VTNG * fsd + o] = vtng;
    sr[SR_VTSA * fsd + o] = vsa;
    sr[SR_VTSB * fsd + o] = vsb;
    sr[SR_VTI * fsd + o] = vti;
    sr[SR_VTNI * fsd + o] = vtni;
    sr[SR_VTC * fsd + o] = vtc;
    sr[SR_VTNC * fsd + o] = vtnc;

    // outputs final after phase A: checked prognostics, qv, aerosols (main:738-748)
    store_checked(L, k);
    a.qv[e] = S(Max(min_qv, (L.qv1d + L.qvten * dtd)));
    if (has_nwfa) a.nwfa[e] = S(Max(R(nwfa_default), Min(R(aero_max), (nwfa_in + L.nwfaten * dt))));
    if (has_nifa) a.nifa[e] = S(Max(R(nifa_default), Min(R(aero_max), (nifa_in + L.nifaten * dt))));
  }

  // ---------------- phase B: sedimentation (main:593-727) ----------------
  D prec_r = 0, prec_g = 0, prec_s = 0, prec_i = 0, prec_c = 0;
  const double* rho = sd + SD_RHO * fsd;
  const S* dzp = a.dz + base;
  // fills vt (and vtn) from above in place, computes ktop and substeps
  auto fill = [&](int fv, int fvn, bool use_max, bool snow, int& steps, int& ktop) {
    steps = 1;
    ktop = 1;
    R vup = R(0), vnup = R(0);
    for (int k = nz - 1; k >= 0; k--) {
      const long o = (long)k * cs;
      R v, vn = R(0);
      if (snow) {
        R A = sr[SR_VTSA * fsd + o];
        if (A >= R(0)) {
          if (sr[SR_VTSB * fsd + o] != R(0)) {
            R vrain = any_qr ? sr[SR_VTR * fsd + o] : R(0);
            R rsk = R(sd[SD_XRS * fsd + o]);
            R srr = rsk / (rsk + R(sd[SD_XRR * fsd + o]));
            v = A * srr + (R(1.0) - srr) * vrain;
          } else {
            v = A;
          }
        } else {
          v = vup;
        }
      } else {
        v = sr[fv * fsd + o];
        vn = sr[fvn * fsd + o];
        if (v < R(0)) {
          v = vup;
          vn = vnup;
        }
        sr[fvn * fsd + o] = vn;
      }
      sr[fv * fsd + o] = v;
      vup = v;
      vnup = vn;
      R vm = use_max ? Max(v, vn) : v;
      if (vm > R(1.e-3)) {
        ktop = max(ktop, k + 1);
        R dz_by_vt = R(dzp[k * NI]) / vm;
        steps = max(steps, Int(dt / dz_by_vt + R(1.0)));
      }
    }
    if (ktop == nz) ktop = nz - 1;
  };
  // one substep on a field whose fall speed sits in the R scratch
  auto sweep = [&](int fx, int ften, int fv, D limit, int steps, int ktop, D* precip) {
    double* x = sd + fx * fsd;
    double* ten = sd + ften * fsd;
    const R* vt = sr + fv * fsd;
    const D osteps = 1.0 / (D)steps;
    int k = nz - 1;
    D s_top = D(vt[k * cs]) * x[k * cs];
    D odz = 1.0 / ldd(dzp + k * NI), orho = 1.0 / rho[k * cs];
    ten[k * cs] = ten[k * cs] - s_top * odz * osteps * orho;
    x[k * cs] = Max(limit, x[k * cs] - s_top * odz * dtd * osteps);
    D s_up = (ktop == nz - 1) ? s_top : D(vt[ktop * cs]) * x[ktop * cs];
    D s0 = (nz == 1) ? s_top : D(vt[0]) * x[0];
    for (k = ktop - 1; k >= 0; k--) {
      D s_k = D(vt[k * cs]) * x[k * cs];
      odz = 1.0 / ldd(dzp + k * NI);
      orho = 1.0 / rho[k * cs];
      ten[k * cs] = ten[k * cs] + (s_up - s_k) * odz * osteps * orho;
      x[k * cs] = Max(limit, x[k * cs] + (s_up - s_k) * odz * dtd * osteps);
      if (k == 0) s0 = s_k;
      s_up = s_k;
    }
    if (precip && x[0] > low_limit_mass_for_precip) *precip = *precip + s0 * dtd * osteps;
  };
  int steps, ktop;
  unsigned sub[5] = {0, 0, 0, 0, 0};
  if (any_qr) {
    fill(SR_VTR, SR_VTNR, true, false, steps, ktop);
    sub[0] = steps;
    for (int n = 0; n < steps; n++) {
      sweep(SD_XRR, SD_TQR, SR_VTR, r1, steps, ktop, &prec_r);
      sweep(SD_XNR, SD_TNR, SR_VTNR, r2, steps, ktop, nullptr);
    }
  }
  if (any_qg) {
    fill(SR_VTG, SR_VTNG, false, false, steps, ktop);
    sub[1] = steps;
    for (int n = 0; n < steps; n++) {
      sweep(SD_XRG, SD_TQG, SR_VTG, r1, steps, ktop, &prec_g);
      sweep(SD_XNG, SD_TNG, SR_VTNG, r2, steps, ktop, nullptr);
      sweep(SD_XRB, SD_TQB, SR_VTG, meters3_to_liters * r1 / rho_gd(nrhg), steps, ktop, nullptr);
    }
  }
  if (any_qs) {
    fill(SR_VTSA, SR_VTSA, false, true, steps, ktop);
    sub[2] = steps;
    for (int n = 0; n < steps; n++) sweep(SD_XRS, SD_TQS, SR_VTSA, r1, steps, ktop, &prec_s);
  }
  if (any_qi) {
    fill(SR_VTI, SR_VTNI, false, false, steps, ktop);
    sub[3] = steps;
    sweep(SD_XRI, SD_TQI, SR_VTI, r1, steps, ktop, &prec_i);
    sweep(SD_XNI, SD_TNI, SR_VTNI, r2, steps, ktop, nullptr);
  }
  if (any_qc) {  // cloud_fallspeed (main:1945-1977): settles only below 500 m
    int kt = 1;
    D hgtc = 0.0;
    for (int k = 1; k <= nz - 1; k++) {
      if (sd[SD_XRC * fsd + (long)(k - 1) * cs] > r2) kt = k;
      hgtc = hgtc + ldd(dzp + (long)(k - 1) * NI);
      if (hgtc > 500.0) break;
    }
    for (int k = kt; k < nz; k++) {  // vt stays zero above ktop
      sr[SR_VTC * fsd + (long)k * cs] = R(0);
      sr[SR_VTNC * fsd + (long)k * cs] = R(0);
    }
    sub[4] = 1;
    sweep(SD_XRC, SD_TQC, SR_VTC, r1, 1, kt, &prec_c);
    sweep(SD_XNC, SD_TNC, SR_VTNC, r2, 1, kt, nullptr);
  }
  for (int s = 0; s < 5; s++)
    if (sub[s]) atomicMax(a.stats + 1 + s, (unsigned long long)sub[s]);

  // ---------------- phase C (main:731-863) ----------------
  D mhd_max = 0.0, mhd_sfc = 0.0, temp_sfc = 0.0;
  for (int k = 0; k < nz; k++) {
    const long e = at(k), o = (long)k * cs;
    Lev<R> L;
    L.cs = &cst;
    L.cd = &cstd;
    L.t1d = use_t ? ldd(a.t + e) : ldd(a.th + e) * ldd(a.pii + e);
    L.pres = R(a.p[e]);
    L.tten = sd[SD_TTEN * fsd + o];
    L.qv = sd[SD_QV * fsd + o];
    L.rho = sd[SD_RHO * fsd + o];
    L.temp = L.t1d + L.tten * dtd;
    if (k == 0) temp_sfc = L.temp;
    D ocp = 1.0 / (cp * (1.0 + 0.887 * L.qv));
    D lvap = lvap0 + (2106.0 - 4218.0) * (L.temp - t0);
    L.qc1d = R(a.qc[e]);
    L.nc1d = has_nc ? R(a.nc[e]) : R(0);
    L.qr1d = R(a.qr[e]);
    L.nr1d = R(a.nr[e]);
    L.qi1d = R(a.qi[e]);
    L.ni1d = R(a.ni[e]);
    L.qs1d = R(a.qs[e]);
    L.qg1d = R(a.qg[e]);
    L.ng1d = hail ? R(a.ng[e]) : R(0);
    L.qb1d = hail ? R(a.qb[e]) : R(0);
    L.qrten = R(sd[SD_TQR * fsd + o]);
    L.nrten = R(sd[SD_TNR * fsd + o]);
    L.qgten = R(sd[SD_TQG * fsd + o]);
    L.ngten = R(sd[SD_TNG * fsd + o]);
    L.qbten = R(sd[SD_TQB * fsd + o]);
    L.qsten = R(sd[SD_TQS * fsd + o]);
    L.qiten = R(sd[SD_TQI * fsd + o]);
    L.niten = R(sd[SD_TNI * fsd + o]);
    L.qcten = R(sd[SD_TQC * fsd + o]);
    L.ncten = R(sd[SD_TNC * fsd + o]);
    L.smob = L.smoc = L.smo2 = L.smoz = R(0);
    if (!(f & F_NOMICRO)) {  // freeze_cloud_melt_ice (main:2124-2165)
      R xri = Max(R(0.0), L.qi1d + L.qiten * dt);
      if ((L.temp > t0) && (xri > R(0.0))) {
        L.qcten = L.qcten + xri * odt;
        L.ncten = L.ncten + L.ni1d * odt;
        L.qiten = L.qiten - xri * odt;
        L.niten = -(L.ni1d * odt);
        L.tten = L.tten - cstd.lfus * ocp * D(xri) * D(odt);
      }
      R xrc = Max(R(0.0), L.qc1d + L.qcten * dt);
      if ((L.temp < hgfrz) && (xrc > R(0.0))) {
        D lfus2 = lsub - lvap;
        R xnc;
        if (has_nc)
          xnc = L.nc1d + L.ncten * dt;
        else
          xnc = ncsave / R(L.rho) + L.ncten * dt;
        L.qiten = L.qiten + xrc * odt;
        L.niten = L.niten + xnc * odt;
        L.qcten = L.qcten - xrc * odt;
        L.ncten = L.ncten - xnc * odt;
        L.tten = L.tten + lfus2 * ocp * D(xrc) * D(odt);
      }
    }
    const D tnew = L.t1d + L.tten * dtd;
    if (use_t)
      a.t[e] = S(tnew);
    else
      a.th[e] = S(tnew / ldd(a.pii + e));
    // final checks (main:750-781)
    cloud_check(L, L.qc1d, L.nc1d, has_nc, ncsave, dt, odt);
    rain_check(L, L.qr1d, L.nr1d, dt, odt);
    ice_check(L, L.qi1d, L.ni1d, dt, odt);
    snow_check(L, L.qs1d, dt, odt);
    if (L.l_qs) snow_moments(L, R(Min(-0.1, L.temp - t0)), 2);
    graupel_check(L, L.qg1d, L.ng1d, L.qb1d, hail, dt, odt);
    store_checked(L, k);
    // diagnostics (main:796-863)
    const long e3 = tile3(k);
    if (a.ncmr) a.ncmr[e3] = S(L.nc * R(L.rho));
    if (a.mvd_r) a.mvd_r[e3] = S(L.mvd_r);
    if (a.mvd_g) a.mvd_g[e3] = S(L.mvd_g);
    if (f & F_MHD) {
      D m = D(max_hail_diam(L));
      if (k == 0) {
        mhd_sfc = m;
        mhd_max = m;
      } else if (m > mhd_max) {
        mhd_max = m;
      }
    }
    if (a.refl10cm) a.refl10cm[e3] = S(reflectivity_10cm(L));
    if (f & F_RE) {  // effective_radius (diags:13-56)
      R rec = R(0), rei = R(0), res = R(0);
      if (L.l_qc) {
        int nu_c = get_nuc(L.nc);
        rec = Max(R(2.51e-6), Min(R(0.5) * (R(3.0) + R(nu_c)) * L.ilamc, R(50.e-6)));
      }
      if (L.l_qi) rei = Max(R(2.51e-6), Min(R(0.5) * (R(3.0) + R(mu_i)) * L.ilami, R(125.e-6)));
      if (L.l_qs) res = Max(R(5.01e-6), Min(R(0.5) * (L.smoc / L.smob), R(999.e-6)));
      if (a.re_cloud) a.re_cloud[e3] = S(rec);
      if (a.re_ice) a.re_ice[e3] = S(rei);
      if (a.re_snow) a.re_snow[e3] = S(res);
    } else {
      if (a.re_cloud) a.re_cloud[e3] = S(0);
      if (a.re_ice) a.re_ice[e3] = S(0);
      if (a.re_snow) a.re_snow[e3] = S(0);
    }
  }
  // column diagnostics (main:785-794; driver:452-484)
  const D ffrac = (prec_i + prec_s + prec_g) / (prec_i + prec_s + prec_g + prec_r + r1);
  const D frz = ((temp_sfc - t0) < -0.5) ? prec_r + prec_c : 0.0;
  if (a.rain_precip) a.rain_precip[tile2] = S(prec_r);
  if (a.ice_precip) a.ice_precip[tile2] = S(prec_i);
  if (a.snow_precip) a.snow_precip[tile2] = S(prec_s);
  if (a.graupel_precip) a.graupel_precip[tile2] = S(prec_g);
  if (a.frozen_fraction) a.frozen_fraction[tile2] = S(ffrac);
  if (a.frz_rain) a.frz_rain[tile2] = S(frz);
  if (a.mhd_sfc) a.mhd_sfc[tile2] = S((f & F_MHD) ? mhd_sfc : 0.0);
  if (a.mhd_col) a.mhd_col[tile2] = S((f & F_MHD) ? mhd_max : 0.0);
}

}  // namespace tg
