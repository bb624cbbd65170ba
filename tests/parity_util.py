"""Helpers shared by the parity tests: run one workload through the oracle and the
CUDA library on identical inputs, and compare field by field."""
from __future__ import annotations

import numpy as np

OUT3 = ("t", "qv", "qc", "qr", "qi", "qs", "qg", "ni", "nr", "nc", "nwfa", "nifa", "ng", "qb")
# absolute floors below which differences are judged against the floor instead of the
# value (the reference's existence thresholds r1 = 1e-12 kg/m3, r2 = 1e-6 /m3 scaled
# to per-kg mixing ratios)
FLOOR = {"t": 1.0, "qv": 1e-12, "qc": 1e-12, "qr": 1e-12, "qi": 1e-12, "qs": 1e-12, "qg": 1e-12,
         "ni": 1e-6, "nr": 1e-6, "nc": 1e-6, "nwfa": 1.0, "nifa": 1.0, "ng": 1e-6, "qb": 1e-12,
         "rain_precip": 1e-12, "ice_liquid_equiv_precip": 1e-12,
         "snow_liquid_equiv_precip": 1e-12, "graupel_liquid_equiv_precip": 1e-12,
         "frozen_fraction": 1e-12, "frz_rain_precip": 1e-12, "max_hail_diameter_sfc": 1e-6,
         "max_hail_diameter_column": 1e-6, "refl10cm": 1.0, "re_cloud": 1e-9, "re_ice": 1e-9,
         "re_snow": 1e-9, "rain_med_vol_diam": 1e-9, "graupel_med_vol_diam": 1e-9,
         "cloud_number_mixing_ratio": 1e-6}
DIAG2 = ("rain_precip", "ice_liquid_equiv_precip", "snow_liquid_equiv_precip",
         "graupel_liquid_equiv_precip", "frozen_fraction", "frz_rain_precip",
         "max_hail_diameter_sfc", "max_hail_diameter_column")
DIAG3 = ("refl10cm", "re_cloud", "re_ice", "re_snow", "rain_med_vol_diam",
         "graupel_med_vol_diam", "cloud_number_mixing_ratio")


def make_diags(shape, diag3=DIAG3, dtype=np.float64):
    nj, nk, ni = shape
    d = {n: np.full((nj, ni), np.nan, dtype=dtype) for n in DIAG2}
    d.update({n: np.full((nj, nk, ni), np.nan, dtype=dtype) for n in diag3})
    return d


def run_oracle(oracle, cfg_over: dict, wl, fields=None, itimestep=1, diag3=DIAG3, nthreads=0):
    f = {k: v.copy() for k, v in (fields or wl.fields).items()}
    d = make_diags(f["p"].shape, diag3)
    cfg = oracle.default_cfgs(**cfg_over)
    rc = oracle.run(cfg, wl.dt, itimestep, f, d, nthreads=nthreads)
    assert rc == 0, f"oracle_run returned {rc}"
    return f, d


def run_gpu(ctx, cfg_over: dict, wl, fields=None, itimestep=1, diag3=DIAG3, dtype=np.float64):
    import tempo_gb300 as tg
    f = {k: np.ascontiguousarray(v.astype(dtype)) for k, v in (fields or wl.fields).items()}
    d = make_diags(f["p"].shape, diag3, dtype)
    cfg = tg.default_cfgs(**cfg_over)
    ctx.run(f, wl.dt, itimestep, diags=d, cfgs=cfg)
    return f, d


def rel_err(a, b, floor):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


def compare(fa, da, fb, db, names3=OUT3):
    """Per-field (max, rms) relative error of a against b (b = oracle)."""
    out = {}
    for n in names3:
        if n in fa and n in fb:
            e = rel_err(fa[n], fb[n], FLOOR[n])
            out[n] = (float(e.max()), float(np.sqrt(np.mean(e * e))))
    for n in tuple(DIAG2) + tuple(DIAG3):
        if n in da and n in db:
            assert not np.isnan(db[n]).any(), f"oracle left {n} unset"
            assert not np.isnan(da[n]).any(), f"{n} not written"
            e = rel_err(da[n], db[n], FLOOR[n])
            out[n] = (float(e.max()), float(np.sqrt(np.mean(e * e))))
    return out


def worst(errs):
    k = max(errs, key=lambda n: errs[n][0])
    return k, errs[k][0]


def graupel_density_ties(qg, qb, rtol=1e-12):
    """Levels at the rounding tie of the graupel density class.

    The class is idx_bg = nint(10 * rg / rb) + 1 (module_mp_tempo_main.F90:1172, 1198).
    Where the volume rb sits at its low-density clamp rg * 1000 / rho_g(1) (main:1169-1170),
    10 * rg / rb is 0.5 up to one rounding, so a one-ulp difference in rg -- e.g. from
    the device's and the host's pow/exp -- moves the class between 1 and 2.  Those
    classes differ in am_g by rho_g(2) / rho_g(1) = 2, so the median volume diameter
    (proportional to am_g**(-1/3)) moves by exactly 2**(1/3), while mass and number
    (independent of am_g, main:1175-1196) do not.  Returns the boolean mask of such
    levels, judged on the final qg, qb."""
    qg = np.asarray(qg, dtype=np.float64)
    qb = np.asarray(qb, dtype=np.float64)
    ok = (qg > 1e-12) & (qb > 0)
    r = np.where(ok, 10.0 * qg / np.where(qb > 0, qb, 1.0), 0.0)
    return ok & (np.abs(r - 0.5) <= rtol * 0.5)


def mvd_g_tie_flips(mvd_got, mvd_want, ties, rtol=1e-12):
    """Splits graupel MVD differences at density-class ties into class flips (ratio
    exactly 2**(+-1/3)) and returns (number of flips, max relative error of the rest)."""
    a = np.asarray(mvd_got, dtype=np.float64)
    b = np.asarray(mvd_want, dtype=np.float64)
    e = np.abs(a - b) / np.maximum(np.abs(b), FLOOR["graupel_med_vol_diam"])
    ratio = np.where(b > 0, a / np.where(b > 0, b, 1.0), 1.0)
    c = 2.0 ** (1.0 / 3.0)
    flip = ties & ((np.abs(ratio - c) <= 1e-10 * c) | (np.abs(ratio - 1.0 / c) <= 1e-10 / c))
    rest = np.where(flip, 0.0, e)
    return int(flip.sum()), float(rest.max())
