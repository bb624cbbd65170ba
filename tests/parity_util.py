"""Helpers shared by the parity tests: run one workload through the oracle and the
CUDA library on identical inputs, and compare field by field."""
from __future__ import annotations

import numpy as np

OUT3 = ("t", "qv", "qc", "qr", "qi", "qs", "qg", "ni", "nr", "nc", "nwfa", "nifa", "ng", "qb")
# absolute floors below which differences are measured against the floor instead of the
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


def run_oracle(oracle, cfg_over: dict, wl, fields=None, itimestep=1, diag3=DIAG3, nthreads=0,
               ties=None):
    f = {k: v.copy() for k, v in (fields or wl.fields).items()}
    d = make_diags(f["p"].shape, diag3)
    cfg = oracle.default_cfgs(**cfg_over)
    rc = oracle.run(cfg, wl.dt, itimestep, f, d, nthreads=nthreads, ties=ties)
    assert rc == 0, f"oracle_run returned {rc}"
    return f, d


def run_gpu(ctx, cfg_over: dict, wl, fields=None, itimestep=1, diag3=DIAG3, dtype=np.float64):
    import tempo_gb300 as tg
    f = {k: np.ascontiguousarray(v.astype(dtype)) for k, v in (fields or wl.fields).items()}
    d = make_diags(f["p"].shape, diag3, dtype)
    cfg = tg.default_cfgs(**cfg_over)
    ctx.run(f, wl.dt, itimestep, diags=d, cfgs=cfg)
    return f, d


def rel_err(a, b, floor, scale=None):
    """|a - b| relative to max(|b|, floor) -- and, for a prognostic field, to the
    magnitude it had before the step (``scale``): the step computes new = old +
    tendency * dt, so where that sum cancels (a species nearly used up) the rounding
    of old and of the tendency, not of the small result, sets the attainable error."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.maximum(np.abs(b), floor)
    if scale is not None:
        den = np.maximum(den, np.abs(np.asarray(scale, dtype=np.float64)))
    return np.abs(a - b) / den


def compare(fa, da, fb, db, names3=OUT3, inputs=None):
    """Per-field (max, rms) relative error of a against b (b = oracle); ``inputs``: the
    fields before the step, the scale of the prognostic fields (see rel_err)."""
    out = {}
    for n in names3:
        if n in fa and n in fb:
            e = rel_err(fa[n], fb[n], FLOOR[n], None if inputs is None else inputs.get(n))
            out[n] = (float(e.max()), float(np.sqrt(np.mean(e * e))))
    for n in tuple(DIAG2) + tuple(DIAG3):
        if n in da and n in db:
            # a diagnostic whose flag is off stays untouched in both (driver:302-386)
            if np.isnan(db[n]).all() and np.isnan(da[n]).all():
                continue
            assert not np.isnan(db[n]).any(), f"oracle left {n} unset"
            assert not np.isnan(da[n]).any(), f"{n} not written"
            e = rel_err(da[n], db[n], FLOOR[n])
            out[n] = (float(e.max()), float(np.sqrt(np.mean(e * e))))
    return out


def worst(errs):
    k = max(errs, key=lambda n: errs[n][0])
    return k, errs[k][0]


def _col_err(a, b, floor, scale=None):
    """Per-column max relative error of a 2-D (nj, ni) or 3-D (nj, nk, ni) field."""
    e = rel_err(a, b, floor, scale)
    return e.max(axis=1) if e.ndim == 3 else e


GRAUPEL_DIAGS = ("graupel_med_vol_diam", "refl10cm", "max_hail_diameter_sfc",
                 "max_hail_diameter_column")


def compare_with_ties(fa, da, fb, db, ties, tol, names3=OUT3, inputs=None):
    """Column-wise comparison of a against the oracle b that tells rounding-tie branch
    flips from real mismatches.

    ``ties`` (int, (nj, ni)) comes from the oracle's tie sink: bit 1 = the column's
    step passed an index computation within one rounding of its discontinuity before
    or during sedimentation (the graupel density class nint(10 rg / rb) at the
    low-density clamp rb = rg * 1000 / rho_g(1), module_mp_tempo_main.F90:1169-1171,
    where 10 rg / rb = 0.5 up to one rounding; or a substep count int(dt vt / dz + 1));
    bit 2 = the same class tie in the final check (moves only that level's graupel
    diagnostics).  A last-bit difference of a libm result (the device's vs glibc's)
    can move such an index, and with it the column.

    Returns (worst error over unflagged columns, worst error of the non-graupel-
    diagnostic outputs over bit-2-only columns, number of bit-1 columns that deviate
    beyond tol, name of the field of the worst unflagged error, fraction of the
    unflagged (point, field) values beyond tol)."""
    ties = np.asarray(ties)
    b1 = (ties & 1).astype(bool)
    b2only = ((ties & 2).astype(bool)) & ~b1
    clean = ~(b1 | b2only)
    worst_clean, worst_b2, which = 0.0, 0.0, None
    n_all = n_over = 0
    dev1 = np.zeros_like(b1)
    items = [(n, fa, fb) for n in names3 if n in fa and n in fb]
    items += [(n, da, db) for n in tuple(DIAG2) + tuple(DIAG3) if n in da and n in db]
    for n, A, B in items:
        if A is da and np.isnan(B[n]).all() and np.isnan(A[n]).all():
            continue  # flag off: untouched in both
        assert not np.isnan(B[n]).any(), f"oracle left {n} unset"
        assert not np.isnan(A[n]).any(), f"{n} not written"
        sc = None if (inputs is None or A is da) else inputs.get(n)
        e = _col_err(A[n], B[n], FLOOR[n], sc)
        ep = rel_err(A[n], B[n], FLOOR[n], sc)
        ep = ep.transpose(0, 2, 1)[clean] if ep.ndim == 3 else ep[clean]
        n_all += ep.size
        n_over += int((ep > tol).sum())
        m = float(e[clean].max()) if clean.any() else 0.0
        if m > worst_clean:
            worst_clean, which = m, n
        if n not in GRAUPEL_DIAGS and b2only.any():
            worst_b2 = max(worst_b2, float(e[b2only].max()))
        dev1 |= b1 & (e > tol)
    return worst_clean, worst_b2, int(dev1.sum()), which, n_over / max(1, n_all)
