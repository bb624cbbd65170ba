// tempo_rates.cuh -- process rates, limiter and tendency sums of the TEMPO step for one
// level (src/module_mp_tempo_main.F90:1313-1513, 1980-3193), plus the table-index
// routines (main:2493-2635, 2839-2858) and the pointwise diagnostics
// (src/module_mp_tempo_diags.F90:13-121, 398-438).
#pragma once

#include "tempo_level.cuh"

namespace tg {

// ---------------------------------------------------------------------------------
// table indices
// ---------------------------------------------------------------------------------
// decade search shared by get_*_table_index: find n with 1 <= x/10**n < 10 among
// nint(log10(x)) + {-1, 0, +1}, then the linear bin index (main:2501-2507); 10**n from
// the constant set's table (the same values as the powering)
template <class C, class R>
__device__ __forceinline__ R pow10_of(const TempoConsts<C>& c, int m) {
  return (m >= kP10Min && m <= kP10Max) ? R(c.p10[m - kP10Min]) : Ipow(R(10.0), m);
}
template <class C, class R>
__device__ __forceinline__ int decade_index(const TempoConsts<C>& c, R x, int n2, int nmax) {
  int nx = Nint(Log10(x)), n = 0;
  R q = R(0.0);
  for (int nn = nx - 1; nn <= nx + 1; nn++) {
    n = nn;
    q = x / pow10_of<C, R>(c, nn);
    if (q >= R(1.0) && q < R(10.0)) break;
  }
  int idx = Int(q) + 10 * (n - n2) - (n - n2);
  return max(1, min(idx, nmax));
}
template <class R> __device__ __forceinline__ int temperature_index(Isl<R> tempk) {  // main:2511-2523
  Isl<R> tempc = tempk - t0;
  int it = Int((R(tempc) - R(2.5)) / R(5.0)) - 1;
  it = max(1, -it);
  return min(it, ntb_t);
}
template <class C, class R>
__device__ __forceinline__ void rain_index(const TempoConsts<C>& c, R rr, R ilamr, int& idx_r, int& idx_r1) {  // :2526-2555
  idx_r = decade_index(c, rr, c.nir2, ntb_r);
  R lamr = R(1.) / ilamr;
  R lam_exp = lamr * c.rain_n0_k;
  R n0_exp = c.org1 * rr / c.am_r * PowCre<0>(lam_exp, c.cre[0]);
  idx_r1 = decade_index(c, n0_exp, c.nir3, ntb_r1);
}
// graupel intercept ng ogg2 lamg**cge(2,1) and ilamg**cge(9,idx_bg) (main:2458-2462,
// 3002, 3074, 3180-3188), and rain intercept nr org2 lamr**cre(2) and
// (lamr + fv_r)**(-cre(9)) with lamr = 1/ilamr (main:2970-2975, 3148-3156), once per
// level and rate stage
template <class R>
__device__ __forceinline__ R graupel_n0(const Lev<R>& L) {
  if (!(L.psd_have & 1)) {
    L.psd_n0g = L.ng * L.cs->ogg2 * PowCge<1>(R(1.0) / L.ilamg, L.cs->cge[0][1]);
    L.psd_have |= 1;
  }
  return L.psd_n0g;
}
template <class R>
__device__ __forceinline__ R graupel_pg9(const Lev<R>& L) {
  if (!(L.psd_have & 2)) {
    L.psd_pg9 = Pow(L.ilamg, L.cs->cge[L.idx_bg - 1][8]);
    L.psd_have |= 2;
  }
  return L.psd_pg9;
}
template <class R>
__device__ __forceinline__ void rain_n0_pf9(const Lev<R>& L, R& n0_r, R& pf9) {
  if (!(L.psd_have & 4)) {
    const R lamr = R(1.0) / L.ilamr;
    L.psd_n0r = L.nr * L.cs->org2 * PowCre<1>(lamr, L.cs->cre[1]);
    L.psd_pf9 = PowCre<8, -1>(lamr + R(fv_r), -L.cs->cre[8]);
    L.psd_have |= 4;
  }
  n0_r = L.psd_n0r;
  pf9 = L.psd_pf9;
}

// rain_index of the level's rain state (L.rr, L.ilamr), formed once per level
template <class R>
__device__ __forceinline__ void level_rain_index(const Lev<R>& L, int& idx_r, int& idx_r1) {
  if (L.rain_idx == 0) rain_index(*L.cs, L.rr, L.ilamr, L.rain_idx, L.rain_idx1);
  idx_r = L.rain_idx;
  idx_r1 = L.rain_idx1;
}
template <class C, class R>
__device__ __forceinline__ void graupel_index(const TempoConsts<C>& c, R rg, R ilamg, int idx, int& idx_g, int& idx_g1) {  // main:2558-2588
  idx_g = decade_index(c, rg, c.nig2, ntb_g);
  R lamg = R(1.) / ilamg;
  R lam_exp = lamg * c.graupel_n0_k;
  R n0_exp = c.ogg1 * rg / c.am_g[idx - 1] * PowCge<0>(lam_exp, c.cge[0][0]);
  idx_g1 = decade_index(c, n0_exp, c.nig3, ntb_g1);
}
// The bin of a value whose reference index is a non-decreasing function of it built on
// libm's log (main:2341, 2391, 2607).  `guess` is that function in this device's
// arithmetic; the edges (least value of each bin, tempo_consts.h make_index_edges,
// computed with the host's libm) settle the bin exactly, so the index is the host
// arithmetic's for the same value even where the device's log differs in its last bit.
__device__ __forceinline__ double edge_arg(double x) { return x; }
__device__ __forceinline__ double edge_arg(float x) { return (double)x; }
template <class T, int N> __device__ __forceinline__ double edge_arg(const Dual<T, N>& x) { return (double)x.v; }
__device__ __forceinline__ int edge_index(const double* e, int n, double x, int guess) {
  int g = max(1, min(guess, n));
  while (g < n && x >= __ldg(e + g)) g++;
  while (g > 1 && x < __ldg(e + g - 1)) g--;
  return g;
}

template <class C, class R>
__device__ __forceinline__ void cloud_index(const TempoConsts<C>& c, const double* edges, R rc, R nc,
                                            int& idx_c, int& idx_n) {  // :2591-2609
  idx_c = decade_index(c, rc, c.nic2, ntb_c);
  int in = Nint(R(1.0) + R(nbc) * Log(nc / c.t_nc1) / c.nic1);
  idx_n = edge_index(edges + kEdgesN, nbc, edge_arg(nc), in);
}

// ---------------------------------------------------------------------------------
// rates
// ---------------------------------------------------------------------------------
// warm_rain (main:2279-2355)
template <class R>
__device__ void warm_rain(const Lev<R>& L, Tend<R>& t, const Tables<Cst<R>>& T, R odt) {
  const TempoConsts<Cst<R>>& c = *L.cs;
  if (L.l_qr) {
    if (L.mvd_r > R(d0r)) {
      TG_TRACE(L, TR_RW, 1 << 16);
      R ef_rr = Max(R(-0.1), R(1.0) - Exp(R(2300.0) * (L.mvd_r - R(1950.0e-6))));
      t.pnr_rcr = ef_rr * R(2.0) * L.nr * L.rr;
    }
  }
  if (L.l_qc) {
    if (L.rc > R(0.01e-3)) {
      TG_TRACE(L, TR_RW, 1 << 17);
      int nu_c = get_nuc(L.nc);
      R lamc = R(1.0) / L.ilamc;
      R xdc = Max(R(d0c) * R(1.e6), (PowObm(L.rc / (c.am_r * L.nc), c.obmr)) * R(1.e6));
      R dc_g = (c.dc_g_k[nu_c - 1] / lamc) * R(1.e6);
      R dc_b = Pow(xdc * xdc * xdc * dc_g * dc_g * dc_g - xdc * xdc * xdc * xdc * xdc * xdc,
                   R(1.0) / R(6.0));
      R zeta1 = R(0.5) * ((R(6.25e-6) * xdc * dc_b * dc_b * dc_b - R(0.4)) +
                          Fabs(R(6.25e-6) * xdc * dc_b * dc_b * dc_b - R(0.4)));
      R zeta = R(0.027) * L.rc * zeta1;
      R taud = R(0.5) * ((R(0.5) * dc_b - R(7.5)) + Fabs(R(0.5) * dc_b - R(7.5))) + R(r1);
      R tau = R(3.72) / (L.rc * taud);
      t.prr_wau = zeta / tau;
      t.prr_wau = Min(L.rc * odt, t.prr_wau);
      t.pnr_wau = t.prr_wau / (c.am_r * R(nu_c) * R(autocon_nr_factor) * R(d0r) * R(d0r) * R(d0r));
      t.pnc_wau = Min(L.nc * odt, t.prr_wau / (c.am_r * L.mvd_c * L.mvd_c * L.mvd_c));
    }
  }
  if (L.l_qr && L.l_qc) {
    if (L.mvd_r > R(d0r) && L.mvd_c > R(d0c)) {
      R lamr = (R(3.0) + R(mu_r) + R(0.672)) / L.mvd_r;
      int idx = 1 + Int(R(nbr) * Log(L.mvd_r / c.dr1) / Log(c.drn / c.dr1));
      idx = edge_index(T.edges + kEdgesR, nbr, edge_arg(L.mvd_r), idx);
      int mc = Int(L.mvd_c * R(1.e6));
      TG_TRACE(L, TR_RW, idx | (mc << 8) | (1 << 18));
      TG_RANGE(L, RG_EFRW, idx, 1, nbr);
      TG_RANGE(L, RG_EFRW, mc, 1, nbc);
      R ef_rw = ld(T.t_efrw + (idx - 1) + (long)(mc - 1) * nbr);
      R n0_r = L.nr * c.org2 * PowCre<1>(lamr, c.cre[1]);
      t.prr_rcw =
          L.rhof * c.t1_qr_qc * ef_rw * L.rc * n0_r * PowCre<8, -1>(lamr + R(fv_r), -c.cre[8]);
      t.prr_rcw = Min(L.rc * odt, t.prr_rcw);
      t.pnc_rcw =
          L.rhof * c.t1_qr_qc * ef_rw * L.nc * n0_r * PowCre<8, -1>(lamr + R(fv_r), -c.cre[8]);
      t.pnc_rcw = Min(L.nc * odt, t.pnc_rcw);
    }
  }
}

// rain_snow_rain_graupel (main:2638-2727)
template <class R>
__device__ void rain_snow_rain_graupel(const Lev<R>& L, Tend<R>& t, const Tables<Cst<R>>& T, R odt) {
  const TempoConsts<Cst<R>>& c = *L.cs;
  if (L.l_qr && L.l_qs) {
    if (L.rr >= c.r_r1 && L.rs >= c.r_s1) {
      int idx_t = temperature_index<R>(L.temp), idx_r, idx_r1;
      level_rain_index(L, idx_r, idx_r1);
      int idx_s = decade_index(c, L.rs, c.nis2, ntb_s);
      TG_TRACE(L, TR_RS, idx_s | (idx_t << 6) | (idx_r1 << 12) | (idx_r << 18) | (1 << 24));
      TG_RANGE(L, RG_QS, idx_s, 1, ntb_s);
      TG_RANGE(L, RG_QS, idx_t, 1, ntb_t);
      TG_RANGE(L, RG_QS, idx_r1, 1, ntb_r1);
      TG_RANGE(L, RG_QS, idx_r, 1, ntb_r);
      const Cst<R>* e = T.qs + 12L * ((idx_s - 1) + (long)(idx_t - 1) * ntb_s +
                                 (long)(idx_r1 - 1) * ntb_s * ntb_t +
                                 (long)(idx_r - 1) * ntb_s * ntb_t * ntb_r1);
      R tcs_racs1 = ld(e + 0), tmr_racs1 = ld(e + 1), tmr_racs2 = ld(e + 3);
      R tcr_sacr1 = ld(e + 4), tms_sacr1 = ld(e + 5), tcr_sacr2 = ld(e + 6);
      if (L.temp < t0) {
        R tnr_racs1 = ld(e + 8), tnr_racs2 = ld(e + 9), tnr_sacr1 = ld(e + 10), tnr_sacr2 = ld(e + 11);
        t.prr_rcs = -(tmr_racs2 + tcr_sacr2 + tmr_racs1 + tcr_sacr1);
        t.prs_rcs = tmr_racs2 + tcr_sacr2 - tcs_racs1 - tms_sacr1;
        t.prg_rcs = tmr_racs1 + tcr_sacr1 + tcs_racs1 + tms_sacr1;
        t.prr_rcs = Max(-L.rr * odt, t.prr_rcs);
        t.prs_rcs = Max(-L.rs * odt, t.prs_rcs);
        t.prg_rcs = Min((L.rr + L.rs) * odt, t.prg_rcs);
        t.pnr_rcs = tnr_racs1 + tnr_racs2 + tnr_sacr1 + tnr_sacr2;
        t.pnr_rcs = Min(L.nr * odt, t.pnr_rcs);
        t.png_rcs = t.pnr_rcs;
        t.pbg_rcs = R(meters3_to_liters) * t.prg_rcs / R(rho_i);
      } else {
        t.prs_rcs = -tcs_racs1 - tms_sacr1 + tmr_racs2 + tcr_sacr2;
        t.prs_rcs = Max(-L.rs * odt, t.prs_rcs);
        t.prr_rcs = -t.prs_rcs;
      }
    }
  }
  if (L.l_qr && L.l_qg) {
    if (L.rr >= c.r_r1 && L.rg >= c.r_g1) {
      int ig = L.idx_bg;
      int idx_r, idx_r1, idx_g, idx_g1;
      level_rain_index(L, idx_r, idx_r1);
      graupel_index(c, L.rg, L.ilamg, ig, idx_g, idx_g1);
      TG_TRACE(L, TR_RG, idx_g1 | (idx_g << 6) | (idx_r1 << 12) | (idx_r << 18) | (1 << 24));
      TG_RANGE(L, RG_QG, idx_g1, 1, ntb_g1);
      TG_RANGE(L, RG_QG, idx_g, 1, ntb_g);
      TG_RANGE(L, RG_QG, ig, 1, nrhg);
      TG_RANGE(L, RG_QG, idx_r1, 1, ntb_r1);
      TG_RANGE(L, RG_QG, idx_r, 1, ntb_r);
      const Cst<R>* e = T.qg + 5L * ((idx_g1 - 1) + (long)(idx_g - 1) * ntb_g1 +
                                (long)(ig - 1) * ntb_g1 * ntb_g +
                                (long)(idx_r1 - 1) * ntb_g1 * ntb_g * nrhg +
                                (long)(idx_r - 1) * ntb_g1 * ntb_g * nrhg * ntb_r1);
      if (L.temp < t0) {
        t.prg_rcg = ld(e + 1) + ld(e + 2);
        t.prg_rcg = Min(L.rr * odt, t.prg_rcg);
        t.prr_rcg = -t.prg_rcg;
        t.pnr_rcg = ld(e + 3) + ld(e + 4);
        t.pnr_rcg = Min(L.nr * odt, t.pnr_rcg);
        t.pbg_rcg = R(meters3_to_liters) * t.prg_rcg / R(rho_i);
      } else {
        t.prr_rcg = ld(e + 0);
        t.prr_rcg = Min(L.rg * odt, t.prr_rcg);
        t.prg_rcg = -t.prr_rcg;
        t.png_rcg = ld(e + 3);
        t.png_rcg = Min(L.ng * odt, t.png_rcg);
        t.pbg_rcg = R(meters3_to_liters) * t.prg_rcg / rho_g<R>(ig);
        t.pnr_rcg = R(-1.5) * ld(e + 4);
      }
    }
  }
}

// demott_nucleation (main:2823-2836)
template <class C, class R>
__device__ __forceinline__ R demott_nucleation(const TempoConsts<C>& c, R tempc, R rho, R nifa) {
  R nifa_cc = Max(R(0.5), nifa * c.rho_not0 * R(1.e-6) / rho);
  R xni = (R(5.94e-5) * Pow(-tempc, R(3.33))) * (Pow(nifa_cc, (-(R(0.0264) * (tempc))) + R(0.0033)));
  xni = xni * rho / c.rho_not0 * R(1000.0);
  return Max(R(0.0), xni);
}

// koop_nucleation (main:2168-2195)
template <class C, class R>
__device__ __forceinline__ R koop_nucleation(const TempoConsts<C>& c, R temp, R satw, R naero, R dt) {
  R xni = R(0.0);
  R mu_diff = R(210368.0) + (R(131.438) * temp) - (R(3.32373e6) / temp) - (R(41729.1) * Log(temp));
  R a_w_i = Exp(mu_diff / (R(r_uni) * temp));
  R delta_aw = satw - a_w_i;
  R log_j_rate = R(-906.7) + (R(8502.0) * delta_aw) - (R(26924.0) * delta_aw * delta_aw) +
                 (R(29180.0) * delta_aw * delta_aw * delta_aw);
  log_j_rate = Min(R(20.0), log_j_rate);
  R j_rate = Pow10(log_j_rate);
  R prob_h = Min(R(1.0) - Exp(-j_rate * c.ar_volume * dt), R(1.0));
  if (prob_h > R(0.0)) xni = Min(prob_h * naero, R(1000.e3));
  return Max(R(0.0), xni);
}

// ice_nucleation (main:2730-2820)
template <class R>
__device__ void ice_nucleation(const Lev<R>& L, Tend<R>& t, const Tables<Cst<R>>& T, R w, uint32_t f,
                               R dt, R odt) {
  const TempoConsts<Cst<R>>& c = *L.cs;
  if (!(L.temp < t0)) return;
  R tempc = R(L.temp - t0);
  int idx_tc = max(1, min(Nint(-tempc), 45));
  R rate_max = R((L.qv - L.qvsi) * L.rho) * odt * R(0.999);
  R rho = R(L.rho);
  R xni, xnc;
  // DeMott's number (main:2754 and :2798, the same arguments): evaluated once, and only
  // where a reader follows -- the freezing tables' nucleus index (rain or cloud
  // freezing) or the deposition-nucleation branch
  const bool fz_r = L.rr > c.r_r1, fz_c = L.rc > c.r_c1;
  const bool nuc = (L.ssati >= demott_nuc_ssati) || (L.ssatw > eps && tempc < R(demott_nuc_tempc));
  const R xni_demott =
      ((f & F_NIFA) && (fz_r || fz_c || nuc)) ? demott_nucleation(c, tempc, rho, L.nifa) : R(0.0);
  if (f & F_NIFA)
    xni = xni_demott;
  else
    xni = R(1.0) * R(1000.0);
  int idx_in = ((fz_r || fz_c) && xni > c.nt_in1) ? decade_index(c, xni, c.niin2, ntb_in) : 1;
  if (fz_r) {
    int idx_r, idx_r1;
    level_rain_index(L, idx_r, idx_r1);
    TG_TRACE(L, TR_FZR, idx_r | (idx_r1 << 6) | (idx_tc << 12) | (idx_in << 18) | (1 << 24));
    TG_RANGE(L, RG_QRFZ, idx_r, 1, ntb_r);
    TG_RANGE(L, RG_QRFZ, idx_r1, 1, ntb_r1);
    TG_RANGE(L, RG_QRFZ, idx_tc, 1, ntb_t1);
    TG_RANGE(L, RG_QRFZ, idx_in, 1, ntb_in);
    const Cst<R>* e = T.qrfz + 4L * ((idx_r - 1) + (long)(idx_r1 - 1) * ntb_r +
                                (long)(idx_tc - 1) * ntb_r * ntb_r1 +
                                (long)(idx_in - 1) * ntb_r * ntb_r1 * ntb_t1);
    t.prg_rfz = ld(e + 2) * odt;
    t.pri_rfz = ld(e + 0) * odt;
    t.pni_rfz = ld(e + 1) * odt;
    t.pnr_rfz = ld(e + 3) * odt;
    t.prg_rfz = Min(L.rr * odt, t.prg_rfz);
    t.pnr_rfz = Min(L.nr * odt, t.pnr_rfz);
    t.png_rfz = t.pnr_rfz * Max(Min((Pow10(-(R(0.1) * w)) + R(0.1)), R(1.0)), R(0.1));
  } else if (L.rr > R(r1) && L.temp < hgfrz) {
    TG_TRACE(L, TR_FZR, 1 << 25);
    t.pri_rfz = L.rr * odt;
    t.pni_rfz = L.nr * odt;
  }
  t.pbg_rfz = R(meters3_to_liters) * t.prg_rfz / R(rho_i);
  if (fz_c) {
    int idx_c, idx_n;
    cloud_index(c, T.edges, L.rc, L.nc, idx_c, idx_n);
    TG_TRACE(L, TR_FZC, idx_c | (idx_n << 8) | (1 << 16));
    TG_RANGE(L, RG_QCFZ, idx_c, 1, ntb_c);
    TG_RANGE(L, RG_QCFZ, idx_n, 1, nbc);
    TG_RANGE(L, RG_QCFZ, idx_tc, 1, ntb_t1);
    TG_RANGE(L, RG_QCFZ, idx_in, 1, ntb_in);
    const Cst<R>* e = T.qcfz + 2L * ((idx_c - 1) + (long)(idx_n - 1) * ntb_c +
                                (long)(idx_tc - 1) * ntb_c * nbc +
                                (long)(idx_in - 1) * ntb_c * nbc * ntb_t1);
    t.pri_wfz = ld(e + 0) * odt;
    t.pri_wfz = Min(L.rc * odt, t.pri_wfz);
    t.pni_wfz = ld(e + 1) * odt;
    t.pni_wfz = Min3(L.nc * odt, t.pri_wfz / (R(2.0) * R(xm0i)), t.pni_wfz);
  } else if (L.rc > R(r1) && L.temp < hgfrz) {
    TG_TRACE(L, TR_FZC, 1 << 17);
    t.pri_wfz = L.rc * odt;
    t.pni_wfz = L.nc * odt;
  }
  if (nuc) {
    if (f & F_NIFA)
      xnc = xni_demott;
    else
      xnc = Min(R(icenuc_max), R(tno) * Exp(R(ato) * R(t0 - L.temp)));
    xni = L.ni + (t.pni_rfz + t.pni_wfz) * dt;
    t.pni_inu = R(0.5) * (xnc - xni + Fabs(xnc - xni)) * odt;
    t.pri_inu = Min(rate_max, R(xm0i) * t.pni_inu);
    t.pni_inu = t.pri_inu / R(xm0i);
  }
  xni = L.smo0 + L.ni + (t.pni_rfz + t.pni_wfz + t.pni_inu) * dt;
  if (f & F_NWFA) {
    if ((xni <= R(max_ni)) && (L.temp < 238.0) && (L.ssati >= 0.4)) {
      xnc = koop_nucleation(c, R(L.temp), R(L.ssatw), L.nwfa, dt);
      t.pni_iha = xnc * odt;
      t.pri_iha = Min(rate_max, R(xm0i) * R(0.1) * t.pni_iha);
      t.pni_iha = t.pri_iha / (R(xm0i) * R(0.1));
    }
  }
}

// get_t1_subl (main:2861-2888) for one level
template <class R>
__device__ __forceinline__ R t1_subl_of(const Lev<R>& L) {
  const TempoConsts<Cst<R>>& c = *L.cs;
  R otemp = R(1.0 / L.temp);
  R rvs = R(L.rho * L.qvsi);
  R rvs_p = rvs * otemp * (R(lsub) * otemp * c.orv - R(1.0));
  R rvs_pp = rvs * (otemp * (R(lsub) * otemp * c.orv - R(1.0)) * otemp * (R(lsub) * otemp * c.orv - R(1.0)) +
                    (-(R(2.) * R(lsub) * otemp * otemp * otemp * c.orv)) + otemp * otemp);
  R gamsc = R(lsub) * L.diffu / L.tcond * rvs_p;
  R alphsc = R(0.5) * (gamsc / (R(1.0) + gamsc)) * (gamsc / (R(1.0) + gamsc)) * rvs_pp / rvs_p * rvs / rvs_p;
  alphsc = Max(R(1.e-9), alphsc);
  R xsat = R(L.ssati);
  if (Fabs(xsat) < R(1.e-9)) xsat = R(0.0);
  return R(4.0) * R(pi) *
         (R(1.0) - alphsc * xsat + R(2.0) * alphsc * alphsc * xsat * xsat -
          R(5.0) * alphsc * alphsc * alphsc * xsat * xsat * xsat) /
         (R(1.0) + gamsc);
}

// ice_processes (main:2891-3018)
template <class R>
__device__ void ice_processes(const Lev<R>& L, Tend<R>& t, const Tables<Cst<R>>& T, R w, R t1_subl,
                              R odt) {
  const TempoConsts<Cst<R>>& c = *L.cs;
  if (!(L.temp < t0)) return;
  R rvs = R(L.rho * L.qvsi);
  R rate_max = R((L.qv - L.qvsi) * L.rho) * odt * R(0.999);
  R ssati = R(L.ssati);
  if (L.l_qi) {
    int idx_i = decade_index(c, L.ri, c.nii2, ntb_i), idx_i1 = decade_index(c, L.ni, c.nii3, ntb_i1);
    TG_TRACE(L, TR_ICE, idx_i | (idx_i1 << 8) | (1 << 16));
    TG_RANGE(L, RG_ICE, idx_i, 1, ntb_i);
    TG_RANGE(L, RG_ICE, idx_i1, 1, ntb_i1);
    R xdi = Max(R(c.d0i), (R(bm_i) + R(mu_i) + R(1.)) * L.ilami);
    R xmi = c.am_i * PowBm(xdi);
    R oxmi = R(1.0) / xmi;
    t.pri_ide = R(c_cube) * t1_subl * L.diffu * ssati * rvs * c.oig1 * c.cig[4] * L.ni * L.ilami;
    const long ii = (idx_i - 1) + (long)(idx_i1 - 1) * ntb_i;
    if (t.pri_ide < R(0.0)) {
      t.pri_ide = Max3(-L.ri * odt, t.pri_ide, rate_max);
      t.pni_ide = t.pri_ide * oxmi;
      t.pni_ide = Max(-L.ni * odt, t.pni_ide);
    } else {
      R tpi = ld(T.tpi_ide + ii);
      t.pri_ide = Min(t.pri_ide, rate_max);
      t.prs_ide = (R(1.0) - tpi) * t.pri_ide;
      t.pri_ide = tpi * t.pri_ide;
    }
    if ((idx_i == ntb_i) || (xdi > R(5.0) * R(d0s))) {
      t.prs_iau = L.ri * R(.99) * odt;
      t.pni_iau = L.ni * R(.95) * odt;
    } else if (xdi < R(0.1) * R(d0s)) {
      t.prs_iau = R(0.0);
      t.pni_iau = R(0.0);
    } else {
      t.prs_iau = ld(T.tps_iaus + ii) * odt;
      t.prs_iau = Min(L.ri * R(.99) * odt, t.prs_iau);
      t.pni_iau = ld(T.tni_iaus + ii) * odt;
      t.pni_iau = Min(L.ni * R(.95) * odt, t.pni_iau);
    }
    // main:2959-2962 recompute the same xdi/xmi from ilami
    xdi = Max(R(c.d0i), (R(bm_i) + R(mu_i) + R(1.)) * L.ilami);
    xmi = c.am_i * PowBm(xdi);
    oxmi = R(1.) / xmi;
    if (L.rs >= c.r_s1) {
      t.prs_sci = c.t1_qs_qi * L.rhof * R(ef_si) * L.ri * L.smoe;
      t.pni_sci = t.prs_sci * oxmi;
    }
    if (L.rr >= c.r_r1 && L.mvd_r > R(4.0) * xdi) {
      R lamr = R(1.0) / L.ilamr;
      R n0_r, pf9;
      rain_n0_pf9(L, n0_r, pf9);
      t.pri_rci = L.rhof * c.t1_qr_qi * R(ef_ri) * L.ri * n0_r * pf9;
      t.pnr_rci = L.rhof * c.t1_qr_qi * R(ef_ri) * L.ni * n0_r * pf9;
      t.pnr_rci = Min(L.nr * odt, t.pnr_rci);
      t.png_rci = t.pnr_rci * Max(Min((Pow10(-(R(0.1) * w)) + R(0.1)), R(1.0)), R(0.1));
      t.pni_rci = t.pri_rci * oxmi;
      t.prr_rci = L.rhof * c.t2_qr_qi * R(ef_ri) * L.ni * n0_r *
                  PowCre<7, -1>(lamr + R(fv_r), -c.cre[7]);
      t.prr_rci = Min(L.rr * odt, t.prr_rci);
      t.prg_rci = t.pri_rci + t.prr_rci;
      t.pbg_rci = t.prg_rci / R(rho_i);
    }
  }
  if (L.l_qs) {
    R c_snow = R(c_sqrd) + (R(L.temp - t0) + R(1.5)) * (R(c_cube) - R(c_sqrd)) / (R(-30.0) + R(1.5));
    c_snow = Max(R(c_sqrd), Min(c_snow, R(c_cube)));
    t.prs_sde = c_snow * t1_subl * L.diffu * ssati * rvs *
                (c.t1_qs_sd * L.smo1 + c.t2_qs_sd * L.rhof2 * L.vsc2 * L.smof);
    if (t.prs_sde < R(0.0))
      t.prs_sde = Max3(-L.rs * odt, t.prs_sde, rate_max);
    else
      t.prs_sde = Min(t.prs_sde, rate_max);
  }
  if (L.l_qg) {
    if (L.ssati < -eps) {
      const int ig = L.idx_bg;
      R n0_g = graupel_n0(L);
      R t2_qg_sd = R(0.28) * c.sc3 * Sqrt(c.av_g[ig - 1]) * c.cgg[ig - 1][10];
      t.prg_gde = R(c_cube) * t1_subl * L.diffu * ssati * rvs * n0_g *
                  (c.t1_qg_sd * PowCge<9>(L.ilamg, c.cge[0][9]) +
                   t2_qg_sd * L.vsc2 * L.rhof2 * Pow(L.ilamg, c.cge[ig - 1][10]));
      if (t.prg_gde < R(0.0)) {
        t.prg_gde = Max3(-L.rg * odt, t.prg_gde, rate_max);
        t.png_gde = t.prg_gde * L.ng / L.rg;
      } else {
        t.prg_gde = Min(t.prg_gde, rate_max);
      }
    }
  }
}

// riming (main:2358-2490); sets vtboost
template <class R>
__device__ void riming(Lev<R>& L, Tend<R>& t, const Tables<Cst<R>>& T, R odt) {
  const TempoConsts<Cst<R>>& c = *L.cs;
  R tempc = R(L.temp - t0);
  L.vtboost = R(1.0);
  if (L.l_qc && L.l_qs) {
    R xds = L.smoc / L.smob;
    if ((L.mvd_c > R(d0c)) && (xds > R(d0s))) {
      int idxs = 1 + Int(R(nbs) * Log(xds / c.ds1) / Log(c.dsn / c.ds1));
      idxs = edge_index(T.edges + kEdgesS, nbs, edge_arg(xds), idxs);
      int mc = Int(L.mvd_c * R(1.e6));
      TG_TRACE(L, TR_RIME, idxs | (mc << 8) | (1 << 16));
      TG_RANGE(L, RG_EFSW, idxs, 1, nbs);
      TG_RANGE(L, RG_EFSW, mc, 1, nbc);
      R ef_sw = ld(T.t_efsw + (idxs - 1) + (long)(mc - 1) * nbs);
      t.prs_scw = L.rhof * c.t1_qs_qc * ef_sw * L.rc * L.smoe;
      t.prs_scw = Min(L.rc * odt, t.prs_scw);
      t.pnc_scw = L.rhof * c.t1_qs_qc * ef_sw * L.nc * L.smoe;
      t.pnc_scw = Min(L.nc * odt, t.pnc_scw);
      if (L.temp < t0) {
        if (t.prs_scw > R(rime_threshold) * t.prs_sde && t.prs_sde > R(eps)) {
          R r_frac = Min(R(30.0), t.prs_scw / t.prs_sde);
          R g_frac = Min(R(rime_conversion), R(0.15) + (r_frac - R(2.0)) * R(.028));
          L.vtboost = Min(R(1.5), R(1.1) + (r_frac - R(2.)) * R(.014));
          t.prg_scw = g_frac * t.prs_scw;
          t.png_scw = t.prg_scw * L.smo0 / L.rs;
          R vts = R(av_s) * Pow(xds, R(bv_s)) * Exp(-(R(fv_s) * xds));
          R const_ri = -(R(1.0) * (L.mvd_c * R(0.5e6)) * vts / Min(R(-0.1), tempc));
          const_ri = Max(R(0.1), Min(const_ri, R(10.0)));
          R rime_dens = (R(0.051) + R(0.114) * const_ri - R(0.0055) * const_ri * const_ri) * R(1000.0);
          if (rime_dens < R(150.0)) {
            g_frac = R(0.0);
            t.prg_scw = R(0.0);
            t.png_scw = R(0.0);
          }
          R snow_dens_frac = Min(R(1.0), Max(R(0.0), L.rs * odt / (L.rs * odt + t.prg_scw)));
          t.pbg_scw = R(meters3_to_liters) * t.prg_scw /
                      (R(rho_s) * snow_dens_frac + rime_dens * (R(1.0) - snow_dens_frac));
          t.prs_scw = (R(1.0) - g_frac) * t.prs_scw;
        }
      }
    }
  }
  if (L.l_qc && L.l_qg) {
    if (L.rg >= c.r_g1 && L.mvd_c > R(d0c)) {
      const int ig = L.idx_bg;
      R xdg = (R(bm_g) + R(mu_g) + R(1.0)) * L.ilamg;
      R vtg = L.rhof * c.av_g[ig - 1] * c.cgg[ig - 1][5] * c.ogg3 * Pow(L.ilamg, c.bv_g[ig - 1]);
      R stoke_g = L.mvd_c * L.mvd_c * vtg * R(rho_w) / (R(9.0) * L.visco * xdg);
      R const_ri = -(R(1.0) * (L.mvd_c * R(0.5e6)) * vtg / Min(R(-0.1), tempc));
      const_ri = Max(R(0.1), Min(const_ri, R(10.0)));
      R rime_dens = (R(0.051) + R(0.114) * const_ri - R(0.0055) * const_ri * const_ri) * R(1000.0);
      if (xdg > R(d0g)) {
        R ef_gw = R(0.0);
        if (stoke_g >= R(0.4) && stoke_g <= R(10.0))
          ef_gw = R(0.55) * Log10(R(2.51) * stoke_g);
        else if (stoke_g < R(0.4))
          ef_gw = R(0.0);
        else if (stoke_g > R(10.0))
          ef_gw = R(0.77);
        if (L.temp > t0) ef_gw = ef_gw * R(0.1);
        R t1_qg_qc = R(pi) * R(.25) * c.av_g[ig - 1] * c.cgg[ig - 1][8];
        R n0_g = graupel_n0(L);
        R pg9 = graupel_pg9(L);
        t.prg_gcw = L.rhof * t1_qg_qc * ef_gw * L.rc * n0_g * pg9;
        t.pnc_gcw = L.rhof * t1_qg_qc * ef_gw * L.nc * n0_g * pg9;
        t.pnc_gcw = Min(L.nc * odt, t.pnc_gcw);
        if (L.temp < t0) t.pbg_gcw = R(meters3_to_liters) * t.prg_gcw / rime_dens;
        if (L.temp < t0) {
          if (t.prg_gcw > R(eps) && tempc > R(-8.0)) {
            R tf = R(0.0);
            if (tempc >= R(-5.0) && tempc < R(-3.0))
              tf = R(0.5) * (R(-3.0) - tempc);
            else if (tempc > R(-8.0) && tempc < R(-5.0))
              tf = R(0.33333333) * (R(8.0) + tempc);
            t.pni_ihm = R(3.5e8) * tf * t.prg_gcw;
            t.pri_ihm = R(xm0i) * t.pni_ihm;
            t.prs_ihm = t.prs_scw / (t.prs_scw + t.prg_gcw) * t.pri_ihm;
            t.prg_ihm = t.prg_gcw / (t.prs_scw + t.prg_gcw) * t.pri_ihm;
          }
        }
      }
    }
  }
}

// melting (main:3021-3119)
template <class R>
__device__ void melting(const Lev<R>& L, Tend<R>& t, R t1_subl, uint32_t f, R dt, R odt) {
  const TempoConsts<Cst<R>>& c = *L.cs;
  if (!(L.temp > t0)) return;
  R tempc = R(L.temp - t0);
  R rvs = R(L.rho * L.qvsi);
  R ssati = R(L.ssati);
  R delqvs = R(L.delqvs);
  if (L.l_qs) {
    t.prr_sml = (tempc * L.tcond - R(lvap0) * L.diffu * delqvs) *
                (c.t1_qs_me * L.smo1 + c.t2_qs_me * L.rhof2 * L.vsc2 * L.smof);
    if (t.prr_sml > R(0.0)) {
      t.prr_sml = t.prr_sml + R(4218.0) * c.olfus * tempc * (t.prr_rcs + t.prs_scw);
      t.prr_sml = Min(L.rs * odt, Max(R(0.0), t.prr_sml));
      t.pnr_sml = L.smo0 / L.rs * t.prr_sml * Pow10(-(R(0.25) * tempc));
      t.pnr_sml = Min(L.smo0 * odt, t.pnr_sml);
    } else {
      t.prr_sml = R(0.0);
      t.pnr_sml = R(0.0);
      if (ssati < R(0.0)) {
        t.prs_sde = R(c_cube) * t1_subl * L.diffu * ssati * rvs *
                    (c.t1_qs_sd * L.smo1 + c.t2_qs_sd * L.rhof2 * L.vsc2 * L.smof);
        t.prs_sde = Max(-L.rs * odt, t.prs_sde);
      }
    }
  }
  if (L.l_qg) {
    const int ig = L.idx_bg;
    R n0_g = graupel_n0(L);
    R n0_melt = n0_g;
    if ((L.rg * L.ng) < R(1.e-4)) {
      R lamg = R(1.) / L.ilamg;
      n0_melt = (R(1.e-4) / L.rg) * c.ogg2 * PowCge<1>(lamg, c.cge[0][1]);
    }
    R sqav = Sqrt(c.av_g[ig - 1]);
    R t2_qg_me = R(pi) * R(4.0) * R(c_cube) * c.olfus * R(0.28) * c.sc3 * sqav * c.cgg[ig - 1][10];
    R p10 = PowCge<9>(L.ilamg, c.cge[0][9]);
    R p11 = Pow(L.ilamg, c.cge[ig - 1][10]);
    t.prr_gml = (tempc * L.tcond - R(lvap0) * L.diffu * delqvs) * n0_melt *
                (c.t1_qg_me * p10 + t2_qg_me * L.rhof2 * L.vsc2 * p11);
    t.prr_gml = Min(L.rg * odt, Max(R(0.0), t.prr_gml));
    if (t.prr_gml > R(0.0)) {
      R melt_f = Max(R(0.05), Min(t.prr_gml * dt / L.rg, R(1.0)));
      t.pbg_gml = R(meters3_to_liters) * t.prr_gml / Max(Min(melt_f * rho_g<R>(ig), R(rho_w)), R(50.0));
      t.pnr_gml = t.prr_gml * L.ng / L.rg * Pow10(-(R(0.33) * tempc));
    } else {
      t.prr_gml = R(0.0);
      t.pnr_gml = R(0.0);
      t.pbg_gml = R(0.0);
      if (ssati < R(0.0)) {
        R t2_qg_sd = R(0.28) * c.sc3 * sqav * c.cgg[ig - 1][10];
        t.prg_gde = R(c_cube) * t1_subl * L.diffu * ssati * rvs * n0_g *
                    (c.t1_qg_sd * p10 + t2_qg_sd * L.vsc2 * L.rhof2 * p11);
        t.prg_gde = Max(-L.rg * odt, t.prg_gde);
        t.png_gde = t.prg_gde * L.ng / L.rg;
      }
    }
  }
  if (f & F_DT_RIME) {
    t.prr_rcw = t.prr_rcw + t.prs_scw + t.prg_gcw;
    t.prs_scw = R(0.0);
    t.prg_gcw = R(0.0);
  }
}

// aerosol_collection_efficiency (src/module_mp_tempo_aerosols.F90:76-118) of one
// collector for the two aerosol diameters the step uses (0.04 and 0.8 um): the terms
// that depend only on the collector (fall speed, Reynolds number) are formed once.
template <class C, class R>
__device__ void aerosol_eff(const TempoConsts<C>& c, R d, R visc, R rhoa, R temp, int species,
                            R& eff_wf, R& eff_if) {
  const R boltzman = R(1.3806503e-23);
  R vt = R(1.0), rho_p = R(rho_w);
  if (species == 0) {  // rain
    vt = R(-0.1021) + R(4.932e3) * d - R(0.9551e6) * d * d + R(0.07934e9) * d * d * d -
         R(0.002362e12) * d * d * d * d;
    rho_p = R(rho_w);
  } else if (species == 1) {  // snow
    vt = R(av_s) * Pow(d, R(bv_s));
    rho_p = R(rho_s);
  } else {  // graupel
    vt = c.av_g[idx_bg1 - 1] * Pow(d, c.bv_g[idx_bg1 - 1]);
    rho_p = rho_g<R>(idx_bg1);
  }
  R re = R(0.5) * rhoa * d * vt / visc;
  R aval = Log(R(1.0) + re);
  R st2 = (R(1.2) + R(1.0 / 12.0) * aval) / (R(1.0) + aval);
  R sre = Sqrt(re);
#pragma unroll
  for (int i = 0; i < 2; i++) {
    const R da = i == 0 ? R(0.04e-6) : R(0.8e-6);
    R cc = c.aer_cc[i];
    R diff = boltzman * temp * cc / (R(3.0) * R(pi) * visc * da);
    R scn = visc / (rhoa * diff);
    R st = (rho_p - rhoa) * da * da * vt * cc / (R(9.0) * visc * d);
    R eff = R(4.0) / (re * scn) * (R(1.0) + R(0.4) * sre * Pow(scn, R(0.3333)) + R(0.16) * sre * Sqrt(scn)) +
            R(4.0) * da / d * (R(0.02) + da / d * (R(1.0) + R(2.0) * sre));
    if (st > st2) eff = eff + Pow((st - st2) / (st - st2 + R(0.666667)), R(1.5));
    (i == 0 ? eff_wf : eff_if) = Max(R(1.e-5), Min(eff, R(1.0)));
  }
}

// aerosol_scavenging (main:3122-3193)
template <class R>
__device__ void aerosol_scavenging(const Lev<R>& L, Tend<R>& t, R odt) {
  const TempoConsts<Cst<R>>& c = *L.cs;
  R temp = R(L.temp), rho = R(L.rho);
  R ef_wf, ef_if;
  if (L.l_qr && L.mvd_r > R(d0r)) {
    aerosol_eff(c, L.mvd_r, L.visco, rho, temp, 0, ef_wf, ef_if);
    R n0_r, pf9;
    rain_n0_pf9(L, n0_r, pf9);
    t.pna_rca = L.rhof * c.t1_qr_qc * ef_wf * L.nwfa * n0_r * pf9;
    t.pna_rca = Min(L.nwfa * odt, t.pna_rca);
    t.pnd_rcd = L.rhof * c.t1_qr_qc * ef_if * L.nifa * n0_r * pf9;
    t.pnd_rcd = Min(L.nifa * odt, t.pnd_rcd);
  }
  if (L.l_qs && L.rs > c.r_s1) {
    R xds = L.smoc / L.smob;
    aerosol_eff(c, xds, L.visco, rho, temp, 1, ef_wf, ef_if);
    t.pna_sca = L.rhof * c.t1_qs_qc * ef_wf * L.nwfa * L.smoe;
    t.pna_sca = Min(L.nwfa * odt, t.pna_sca);
    t.pnd_scd = L.rhof * c.t1_qs_qc * ef_if * L.nifa * L.smoe;
    t.pnd_scd = Min(L.nifa * odt, t.pnd_scd);
  }
  if (L.l_qg && L.rg > c.r_g1) {
    const int ig = L.idx_bg;
    R xdg = (R(bm_g) + R(mu_g) + R(1.0)) * L.ilamg;
    aerosol_eff(c, xdg, L.visco, rho, temp, 2, ef_wf, ef_if);
    R t1_qg_qc = R(pi) * R(.25) * c.av_g[ig - 1] * c.cgg[ig - 1][8];
    R n0_g = graupel_n0(L);
    R pg9 = graupel_pg9(L);
    t.pna_gca = L.rhof * t1_qg_qc * ef_wf * L.nwfa * n0_g * pg9;
    t.pna_gca = Min(L.nwfa * odt, t.pna_gca);
    t.pnd_gcd = L.rhof * t1_qg_qc * ef_if * L.nifa * n0_g * pg9;
    t.pnd_gcd = Min(L.nifa * odt, t.pnd_gcd);
  }
}

// check_over_depletion (main:1313-1438)
template <class R>
__device__ void check_over_depletion(const Lev<R>& L, Tend<R>& t, R odt) {
  R sump, rate_max, ratio;
  sump = t.pri_inu + t.pri_ide + t.prs_ide + t.prs_sde + t.prg_gde + t.pri_iha;
  rate_max = R((L.qv - L.qvsi) * L.rho) * odt * R(0.999);
  if ((sump > R(eps) && sump > rate_max) || (sump < R(-eps) && sump < rate_max)) {
    TG_TRACE(L, TR_LIMIT, 1 << 0);
    ratio = rate_max / sump;
    t.pri_inu = t.pri_inu * ratio;
    t.pri_ide = t.pri_ide * ratio;
    t.pni_ide = t.pni_ide * ratio;
    t.prs_ide = t.prs_ide * ratio;
    t.prs_sde = t.prs_sde * ratio;
    t.prg_gde = t.prg_gde * ratio;
    t.pri_iha = t.pri_iha * ratio;
  }
  sump = -t.prr_wau - t.pri_wfz - t.prr_rcw - t.prs_scw - t.prg_scw - t.prg_gcw;
  rate_max = -L.rc * odt;
  if (L.l_qc && sump < rate_max) {
    TG_TRACE(L, TR_LIMIT, 1 << 1);
    ratio = rate_max / sump;
    t.prr_wau = t.prr_wau * ratio;
    t.pri_wfz = t.pri_wfz * ratio;
    t.prr_rcw = t.prr_rcw * ratio;
    t.prs_scw = t.prs_scw * ratio;
    t.prg_scw = t.prg_scw * ratio;
    t.prg_gcw = t.prg_gcw * ratio;
  }
  sump = t.pri_ide - t.prs_iau - t.prs_sci - t.pri_rci;
  rate_max = -L.ri * odt;
  if (L.l_qi && sump < rate_max) {
    TG_TRACE(L, TR_LIMIT, 1 << 2);
    ratio = rate_max / sump;
    t.pri_ide = t.pri_ide * ratio;
    t.prs_iau = t.prs_iau * ratio;
    t.prs_sci = t.prs_sci * ratio;
    t.pri_rci = t.pri_rci * ratio;
  }
  sump = -t.prg_rfz - t.pri_rfz - t.prr_rci + t.prr_rcs + t.prr_rcg;
  rate_max = -L.rr * odt;
  if (L.l_qr && sump < rate_max) {
    TG_TRACE(L, TR_LIMIT, 1 << 3);
    ratio = rate_max / sump;
    t.prg_rfz = t.prg_rfz * ratio;
    t.pbg_rfz = t.pbg_rfz * ratio;
    t.pri_rfz = t.pri_rfz * ratio;
    t.prr_rci = t.prr_rci * ratio;
    t.prr_rcs = t.prr_rcs * ratio;
    t.prr_rcg = t.prr_rcg * ratio;
  }
  sump = t.prs_sde - t.prs_ihm - t.prr_sml + t.prs_rcs;
  rate_max = -L.rs * odt;
  if (L.l_qs && sump < rate_max) {
    TG_TRACE(L, TR_LIMIT, 1 << 4);
    ratio = rate_max / sump;
    t.prs_sde = t.prs_sde * ratio;
    t.prs_ihm = t.prs_ihm * ratio;
    t.prr_sml = t.prr_sml * ratio;
    t.prs_rcs = t.prs_rcs * ratio;
  }
  sump = t.prg_gde - t.prg_ihm - t.prr_gml + t.prg_rcg;
  rate_max = -L.rg * odt;
  if (L.l_qg && sump < rate_max) {
    TG_TRACE(L, TR_LIMIT, 1 << 5);
    ratio = rate_max / sump;
    t.prg_gde = t.prg_gde * ratio;
    t.prg_ihm = t.prg_ihm * ratio;
    t.prr_gml = t.prr_gml * ratio;
    t.prg_rcg = t.prg_rcg * ratio;
    t.pbg_rcg = t.pbg_rcg * ratio;
  }
  t.pri_ihm = t.prs_ihm + t.prg_ihm;
  ratio = Min(Fabs(t.prr_rcg), Fabs(t.prg_rcg));
  t.prr_rcg = ratio * Copysign(R(1.0), t.prr_rcg);
  t.prg_rcg = -t.prr_rcg;
  t.pbg_rcg = R(meters3_to_liters) * t.prg_rcg / R(rho_i);
  if (L.temp > t0) {
    ratio = Min(Fabs(t.prr_rcs), Fabs(t.prs_rcs));
    t.prr_rcs = ratio * Copysign(R(1.0), t.prr_rcs);
    t.prs_rcs = -t.prr_rcs;
  }
}

// sum_tendencies (main:1441-1513)
template <class R>
__device__ void sum_tendencies(Lev<R>& L, const Tend<R>& t) {
  using I = Isl<R>;
  R orho = R(1. / L.rho);
  I orho_d = 1. / L.rho;
  I lfus2 = lsub - I(L.lvap);
  L.qvten = L.qvten + I(-t.pri_inu - t.pri_iha - t.pri_ide - t.prs_ide - t.prs_sde - t.prg_gde) * orho_d;
  L.qcten = L.qcten + (-t.prr_wau - t.pri_wfz - t.prr_rcw - t.prs_scw - t.prg_scw - t.prg_gcw) * orho;
  L.ncten = L.ncten + (-t.pnc_wau - t.pnc_rcw - t.pni_wfz - t.pnc_scw - t.pnc_gcw) * orho;
  L.qiten = L.qiten + (t.pri_inu + t.pri_iha + t.pri_ihm + t.pri_wfz + t.pri_rfz + t.pri_ide -
                       t.prs_iau - t.prs_sci - t.pri_rci) * orho;
  L.niten = L.niten + (t.pni_inu + t.pni_iha + t.pni_ihm + t.pni_wfz + t.pni_rfz + t.pni_ide -
                       t.pni_iau - t.pni_sci - t.pni_rci) * orho;
  L.qrten = L.qrten + (t.prr_wau + t.prr_rcw + t.prr_sml + t.prr_gml + t.prr_rcs + t.prr_rcg -
                       t.prg_rfz - t.pri_rfz - t.prr_rci) * orho;
  L.nrten = L.nrten + (t.pnr_wau + t.pnr_sml + t.pnr_gml -
                       (t.pnr_rfz + t.pnr_rcr + t.pnr_rcg + t.pnr_rcs + t.pnr_rci + t.pni_rfz)) * orho;
  L.qsten = L.qsten + (t.prs_iau + t.prs_sde + t.prs_sci + t.prs_scw + t.prs_rcs + t.prs_ide -
                       t.prs_ihm - t.prr_sml) * orho;
  L.qgten = L.qgten + (t.prg_scw + t.prg_rfz + t.prg_gde + t.prg_rcg + t.prg_gcw + t.prg_rci +
                       t.prg_rcs - t.prg_ihm - t.prr_gml) * orho;
  L.ngten = L.ngten + (t.png_scw + t.png_rfz - t.png_rcg + t.png_rci + t.png_rcs + t.png_gde -
                       t.pnr_gml) * orho;
  L.qbten = L.qbten + (t.pbg_scw + t.pbg_rfz + t.pbg_gcw + t.pbg_rci + t.pbg_rcs + t.pbg_rcg +
                       t.pbg_sml - t.pbg_gml +
                       R(meters3_to_liters) * (t.prg_gde - t.prg_ihm) / rho_g<R>(L.idx_bg)) * orho;
  if constexpr (std::is_same<Cst<R>, float>::value) {
    // magnitudes of the summed terms (the cancellation test of the checks, updated())
    using C = Cst<R>;
    const C om = mag(orho);
    auto M = [](auto... x) { return (mag(x) + ...); };
    L.qcmag = L.qcmag + M(t.prr_wau, t.pri_wfz, t.prr_rcw, t.prs_scw, t.prg_scw, t.prg_gcw) * om;
    L.ncmag = L.ncmag + M(t.pnc_wau, t.pnc_rcw, t.pni_wfz, t.pnc_scw, t.pnc_gcw) * om;
    L.qimag = L.qimag + M(t.pri_inu, t.pri_iha, t.pri_ihm, t.pri_wfz, t.pri_rfz, t.pri_ide, t.prs_iau,
                          t.prs_sci, t.pri_rci) * om;
    L.nimag = L.nimag + M(t.pni_inu, t.pni_iha, t.pni_ihm, t.pni_wfz, t.pni_rfz, t.pni_ide, t.pni_iau,
                          t.pni_sci, t.pni_rci) * om;
    L.qrmag = L.qrmag + M(t.prr_wau, t.prr_rcw, t.prr_sml, t.prr_gml, t.prr_rcs, t.prr_rcg, t.prg_rfz,
                          t.pri_rfz, t.prr_rci) * om;
    L.nrmag = L.nrmag + M(t.pnr_wau, t.pnr_sml, t.pnr_gml, t.pnr_rfz, t.pnr_rcr, t.pnr_rcg, t.pnr_rcs,
                          t.pnr_rci, t.pni_rfz) * om;
    L.qsmag = L.qsmag + M(t.prs_iau, t.prs_sde, t.prs_sci, t.prs_scw, t.prs_rcs, t.prs_ide, t.prs_ihm,
                          t.prr_sml) * om;
    L.qgmag = L.qgmag + M(t.prg_scw, t.prg_rfz, t.prg_gde, t.prg_rcg, t.prg_gcw, t.prg_rci, t.prg_rcs,
                          t.prg_ihm, t.prr_gml) * om;
    L.ngmag = L.ngmag + M(t.png_scw, t.png_rfz, t.png_rcg, t.png_rci, t.png_rcs, t.png_gde, t.pnr_gml) * om;
    L.qbmag = L.qbmag + (M(t.pbg_scw, t.pbg_rfz, t.pbg_gcw, t.pbg_rci, t.pbg_rcs, t.pbg_rcg, t.pbg_sml,
                           t.pbg_gml) +
                         C(meters3_to_liters) * M(t.prg_gde, t.prg_ihm) / C(rho_gd(L.idx_bg))) * om;
  }
  I ocp = I(L.ocp);
  if (L.temp < t0) {
    L.tten = L.tten + (lsub * ocp * I(t.pri_inu + t.pri_ide + t.prs_ide + t.prs_sde + t.prg_gde + t.pri_iha) +
                       lfus2 * ocp * I(t.pri_wfz + t.pri_rfz + t.prg_rfz + t.prs_scw + t.prg_scw +
                                       t.prg_gcw + t.prg_rcs + t.prs_rcs + t.prr_rci + t.prg_rcg)) * orho_d;
  } else {
    L.tten = L.tten + (L.ci->lfus * ocp * I(-t.prr_sml - t.prr_gml - t.prr_rcg - t.prr_rcs) +
                       lsub * ocp * I(t.prs_sde + t.prg_gde)) * orho_d;
  }
}

// activate_cloud_number (main:2198-2276) without the land argument
template <class C, class R>
__device__ R activate_cloud_number(const TempoConsts<C>& c, R temp, R w1d, R nwfa, const float* tnccn) {
  R n_local = nwfa * R(1.e-6);
  if (n_local >= c.ta_na[ntb_arc - 1])
    n_local = c.ta_na[ntb_arc - 1] - R(1.0);
  else if (n_local <= c.ta_na[0])
    n_local = c.ta_na[0] + R(1.0);
  int n;
  for (n = 2; n <= ntb_arc; n++)
    if (n_local >= c.ta_na[n - 2] && n_local < c.ta_na[n - 1]) break;
  n = min(n, ntb_arc);
  const int i = n;
  R x1 = c.ln_ta_na[i - 2], x2 = c.ln_ta_na[i - 1];
  R w_local = w1d;
  if (w_local >= c.ta_ww[ntb_arw - 1])
    w_local = c.ta_ww[ntb_arw - 1] - R(1.0);
  else if (w_local <= c.ta_ww[0])
    w_local = c.ta_ww[0] + R(0.001);
  for (n = 2; n <= ntb_arw; n++)
    if (w_local >= c.ta_ww[n - 2] && w_local < c.ta_ww[n - 1]) break;
  n = min(n, ntb_arw);
  const int j = n;
  R y1 = c.ln_ta_ww[j - 2], y2 = c.ln_ta_ww[j - 1];
  int k = max(1, min(Nint((temp - c.ta_tk[0]) * R(0.1)) + 1, ntb_art));
  const int l = 3, m = 2;
  auto TN = [&](int a, int b) -> R {
    return R(ld(tnccn + (a - 1) + (long)(b - 1) * ntb_arc + (long)(k - 1) * ntb_arc * ntb_arw +
                (long)(l - 1) * ntb_arc * ntb_arw * ntb_art +
                (long)(m - 1) * ntb_arc * ntb_arw * ntb_art * ntb_arr));
  };
  R a = TN(i - 1, j - 1), b = TN(i, j - 1), cc = TN(i, j), d = TN(i - 1, j);
  R nx = Log(n_local), wy = Log(w_local);
  R t = (nx - x1) / (x2 - x1), u = (wy - y1) / (y2 - y1);
  R fraction = (R(1.0) - t) * (R(1.0) - u) * a + t * (R(1.0) - u) * b + t * u * cc + (R(1.0) - t) * u * d;
  fraction = Max(fraction, R(0.));
  return nwfa * fraction;
}

// cloud_condensation (main:1980-2056).  The saturation adjustment runs in double.
template <class R>
__device__ void cloud_condensation(const Lev<R>& L, Tend<R>& t, const Tables<Cst<R>>& T, R w,
                                   uint32_t f, R ncsave, R dt, R odt) {
  const TempoConsts<Cst<R>>& c = *L.cs;
  if (Fabs(L.ssatw) < eps) return;
  using I = Isl<R>;
  R orho = R(1.0 / L.rho);
  if (L.ssatw < 0.0 && L.rc <= R(r1)) {
    // Subsaturated without cloud water: the Newton iterations below start at
    // (qv - qvs) / (1 + lvt2 qvs) < 0 and, on a convex increasing function, approach
    // its negative root from the right, so the condensed amount stays negative and
    // rc + clap rho <= r1: the branch that removes the (absent) cloud, taken here
    // without the iterations.
    t.prw_vcd = -(L.rc * orho * odt);
    t.pnc_wcd = -(L.nc * orho * odt);
    return;
  }
  I clap;
  if constexpr (std::is_same<I, df>::value) {
    // Mixed form: the cancellation sits in qv - qvs, formed once in the island type; the
    // three Newton iterations then solve in FP32 for the condensed amount c on
    // qvs (exp(lvt2 c) - 1) + c - (qv - qvs), the same function as qvs exp(lvt2 c) - qv
    // + c, with every term of the size of c (so FP32 gives c to FP32 precision).
    const float d = float(L.qv - L.qvs), qs = float(L.qvs), lv = float(L.lvt2);
    float c = d / (1.0f + lv * qs);
    for (int n = 1; n <= 3; n++) {
      const float em1 = expm1f(lv * c);
      const float fcd = qs * em1 + (c - d);
      const float dfcd = qs * lv * (em1 + 1.0f) + 1.0f;
      c = c - fcd / dfcd;
    }
    clap = I(c);
  } else {
    I lvt2 = I(L.lvt2);
    clap = (L.qv - L.qvs) / (1.0 + lvt2 * L.qvs);
    for (int n = 1; n <= 3; n++) {  // Newton on qvs exp(lvt2 c) - qv + c = 0 (main:2002-2007)
      const I ex = Exp(lvt2 * clap);
      I fcd = L.qvs * ex - L.qv + clap;
      I dfcd = L.qvs * lvt2 * ex + 1.0;
      clap = clap - fcd / dfcd;
    }
  }
  I xrc = I(L.rc) + clap * L.rho;
  if (xrc > r1) {
    t.prw_vcd = R(clap * I(odt));
    if (clap > eps) {
      R xnc;
      if (f & F_NWFA)
        xnc = Max(R(nt_c_min), activate_cloud_number(c, R(L.temp), w, L.nwfa, T.tnccn));
      else
        xnc = ncsave;  // ncsave when nc is absent, else nt_c_l (main:2018-2022)
      t.pnc_wcd = R(0.5) * (xnc - L.nc + Fabs(xnc - L.nc)) * odt * orho;
    } else if (L.l_qc && L.ssatw < -1.e-6 && clap < -eps) {
      R otemp = R(1.0 / L.temp);
      R rvs = R(L.rho * L.qvs);
      R rvs_p = rvs * otemp * (L.lvap * otemp * c.orv - R(1.0));
      R rvs_pp = rvs * (otemp * (L.lvap * otemp * c.orv - R(1.0)) * otemp * (L.lvap * otemp * c.orv - R(1.0)) +
                        (-(R(2.0) * L.lvap * otemp * otemp * otemp * c.orv)) + otemp * otemp);
      R gamsc = L.lvap * L.diffu / L.tcond * rvs_p;
      R alphsc = R(0.5) * (gamsc / (R(1.0) + gamsc)) * (gamsc / (R(1.0) + gamsc)) * rvs_pp / rvs_p * rvs / rvs_p;
      alphsc = Max(R(1.e-9), alphsc);
      R xsat = R(L.ssatw);
      if (Fabs(xsat) < R(1.e-9)) xsat = R(0.0);
      R t1_evap = R(2.0) * R(pi) *
                  (R(1.0) - alphsc * xsat + R(2.0) * alphsc * alphsc * xsat * xsat -
                   R(5.0) * alphsc * alphsc * alphsc * xsat * xsat * xsat) /
                  (R(1.0) + gamsc);
      R dc_star = Sqrt(-(R(2.0) * dt) * t1_evap / (R(2.0) * R(pi)) * R(4.0) * L.diffu * R(L.ssatw) * rvs / R(rho_w));
      int idx_d = max(1, min(Int(R(1.e6) * dc_star), nbc));
      int idx_c, idx_n;
      cloud_index(c, T.edges, L.rc, L.nc, idx_c, idx_n);
      TG_TRACE(L, TR_EVAP, idx_d | (idx_c << 8) | (idx_n << 16) | (1 << 24));
      TG_RANGE(L, RG_EVAP, idx_d, 1, nbc);
      TG_RANGE(L, RG_EVAP, idx_c, 1, ntb_c);
      TG_RANGE(L, RG_EVAP, idx_n, 1, nbc);
      R tnc = ld(T.tnc_wev + (idx_d - 1) + (long)(idx_c - 1) * nbc + (long)(idx_n - 1) * nbc * ntb_c);
      t.prw_vcd = Max(-(L.rc * R(0.99) * orho * odt), t.prw_vcd);
      t.pnc_wcd = Max(-(L.nc * R(0.99) * orho * odt), -(tnc * orho * odt));
    }
  } else {
    t.prw_vcd = -(L.rc * orho * odt);
    t.pnc_wcd = -(L.nc * orho * odt);
  }
}

// rain_evaporation (main:2059-2121)
template <class R>
__device__ void rain_evaporation(const Lev<R>& L, Tend<R>& t, R odt) {
  const TempoConsts<Cst<R>>& c = *L.cs;
  if (!L.l_qr) return;
  if (!((L.ssatw < -eps) && t.prw_vcd <= R(0.0))) return;
  R orho = R(1.0 / L.rho);
  R tempc = R(L.temp - t0);
  R otemp = R(1.0 / L.temp);
  R rvs = R(L.rho * L.qvs);
  R rvs_p = rvs * otemp * (L.lvap * otemp * c.orv - R(1.0));
  R rvs_pp = rvs * (otemp * (L.lvap * otemp * c.orv - R(1.0)) * otemp * (L.lvap * otemp * c.orv - R(1.0)) +
                    (-(R(2.0) * L.lvap * otemp * otemp * otemp * c.orv)) + otemp * otemp);
  R gamsc = L.lvap * L.diffu / L.tcond * rvs_p;
  R alphsc = R(0.5) * (gamsc / (R(1.0) + gamsc)) * (gamsc / (R(1.0) + gamsc)) * rvs_pp / rvs_p * rvs / rvs_p;
  alphsc = Max(R(1.e-9), alphsc);
  R xsat = Min(R(-1.e-9), R(L.ssatw));
  R t1_evap = R(2.0) * R(pi) *
              (R(1.0) - alphsc * xsat + R(2.0) * alphsc * alphsc * xsat * xsat -
               R(5.0) * alphsc * alphsc * alphsc * xsat * xsat * xsat) /
              (R(1.0) + gamsc);
  if (L.qv / L.qvs < 0.95 && L.rr * orho <= R(1.e-8)) {
    t.prv_rev = L.rr * orho * odt;
  } else {
    R lamr = R(1.0) / L.ilamr;
    R n0_r = L.nr * c.org2 * PowCre<1>(lamr, c.cre[1]);
    t.prv_rev = t1_evap * L.diffu * R(-L.ssatw) * n0_r * rvs *
                (c.t1_qr_ev * PowCre<9>(L.ilamr, c.cre[9]) +
                 c.t2_qr_ev * L.vsc2 * L.rhof2 * PowCre<10, -1>(lamr + R(0.5) * R(fv_r), -c.cre[10]));
    R rate_max = Min((L.rr * orho * odt), R((L.qvs - L.qv) * Isl<R>(odt)));
    t.prv_rev = Min(rate_max, t.prv_rev * orho);
    if (t.prr_gml > R(0.0)) {
      R eva_factor = Min(R(1.0), R(0.01) + R(0.99 - 0.01) * (tempc / R(20.0)));
      t.prv_rev = t.prv_rev * eva_factor;
    }
  }
  t.pnr_rev = Min(L.nr * R(0.99) * orho * odt, t.prv_rev * L.nr / L.rr);
}

// ---------------------------------------------------------------------------------
// diagnostics (diags.F90), one level
// ---------------------------------------------------------------------------------
// the three contributions to Ze without melting (diags:80-111)
template <class R>
__device__ void reflectivity_parts(const Lev<R>& L, R& ze_r, R& ze_s, R& ze_g) {
  const TempoConsts<Cst<R>>& c = *L.cs;
  ze_r = R(1.e-22);
  ze_s = R(1.e-22);
  ze_g = R(1.e-22);
  if (L.l_qr) {
    R lamr = R(1.0) / L.ilamr;
    R n0_r = L.nr * c.org2 * PowCre<1>(lamr, c.cre[1]);
    ze_r = n0_r * c.crg[3] * PowCre<3>(L.ilamr, c.cre[3]);
  }
  if (L.l_qs)
    ze_s = R(0.176 / 0.93) * (R(6.0) / R(pi)) * (R(6.0) / R(pi)) * (R(am_s) / R(900.0)) *
           (R(am_s) / R(900.0)) * L.smoz;
  if (L.l_qg) {
    const int ig = L.idx_bg;
    R n0_g = L.ng * c.ogg2 * PowCge<1>(R(1.0) / L.ilamg, c.cge[0][1]);
    ze_g = R(0.176 / 0.93) * (R(6.0) / R(pi)) * (R(6.0) / R(pi)) * (c.am_g[ig - 1] / R(900.0)) *
           (c.am_g[ig - 1] / R(900.0)) * n0_g * c.cgg[0][3] * PowCge<3>(L.ilamg, c.cge[0][3]);
  }
}
template <class R>
__device__ R reflectivity_10cm(const Lev<R>& L) {  // diags:59-121 without melting
  R ze_r, ze_s, ze_g;
  reflectivity_parts(L, ze_r, ze_s, ze_g);
  return Max(R(-35.0), R(10.0) * Log10((ze_r + ze_s + ze_g) * R(1.e18)));
}

template <class R>
__device__ R max_hail_diam(const Lev<R>& L) {  // diags:398-438
  const TempoConsts<Cst<R>>& c = *L.cs;
  const R threshold_conc = R(0.0005);
  if (!(L.rg / R(L.rho) >= R(1.e-6))) return R(0.0);
  if (rho_gd(L.idx_bg) < 350.0) return R(0.0);
  R lamg = R(1.0) / L.ilamg;
  R n0_g = L.ng * c.ogg2 * PowCge<1>(lamg, c.cge[0][1]);
  R sum_nh = R(0.0), sum_t = R(0.0), hail_max;
  int n;
  for (n = nhbins; n >= 1; n--) {
    R f_d = n0_g * Pow(c.hbins[n - 1], R(mu_g)) * Exp(-(lamg * c.hbins[n - 1])) * c.dhbins[n - 1];
    sum_nh = sum_nh + f_d;
    if (sum_nh > threshold_conc) break;
    sum_t = sum_nh;
  }
  if (n >= nhbins)
    hail_max = c.hbins[nhbins - 1];
  else if (c.hbins[n] > R(1.e-3))
    hail_max = c.hbins[n - 1] - (sum_nh - threshold_conc) / (sum_nh - sum_t) * (c.hbins[n - 1] - c.hbins[n]);
  else
    hail_max = R(1.e-4);
  return R(1000.0) * hail_max;
}

}  // namespace tg
