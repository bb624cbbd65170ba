"""The mixed-precision form (FP32 bulk, FP64-grade islands) against the FP64 oracle, on
the oracle's FP32-rounded inputs, over the columns whose oracle step passed no rounding
tie (graupel density class, substep count; there the reference's own result depends on
the last bit of a libm value).

Per field three measures, each against a stated bound:
  - relative RMS, ||mixed - oracle|| / ||oracle||, within the 1e-5 per-field target for
    every field;
  - normwise, max |mixed - oracle| / max |oracle|;
  - pointwise, |mixed - oracle| / max(|oracle|, floor) with the floor at 1e-7 of the
    field's largest value (the FP32 resolution of the field's scale), and the fraction
    of points beyond 1e-5 with the reference's existence floors (r1, r2).
The pointwise 1e-5 bound is not met everywhere with an FP32 bulk: where a value is the
small residue of large terms (a level that sedimentation nearly drains, the front of a
falling species, a species nearly used up) its relative error is the FP32 rounding of
the terms, and an FP32 fall speed or rate that lands on the other side of a bin edge moves
a column.  The normwise and pointwise bounds below are the measured envelope with a
margin (they catch a regression), not the 1e-5 pointwise target.  Also: the
column water budget (total water plus surface precipitation, after minus before)
against the oracle's, and 10-cm reflectivity in dBZ."""
import numpy as np
import pytest

from parity_util import DIAG2, FLOOR, make_diags, run_oracle

pytestmark = pytest.mark.gpu

PROG = ("t", "qv", "qc", "qr", "qi", "qs", "qg", "ni", "nr", "nc", "ng", "qb")
# relative RMS per field: the 1e-5 target for every field on these samples (the
# largest measured is 1.2e-6, nc of the hail-convection sample; on the 262 144 columns of the
# bench's precision study a few columns that cross a discrete step move some fields
# beyond it)
REL_RMS = {n: 1e-5 for n in PROG}
NORMWISE = {"t": 1e-5, "qv": 1e-5}           # others: 1e-4 (largest measured 4.2e-5, nc)
SCALED_MAX = {"t": 1e-5, "qv": 1e-5}          # others: 0.05 (largest 1.7e-2, qg at clamps)
FRAC_R1 = 0.05                               # points beyond 1e-5 with the reference floors
BUDGET = 1e-7                                # column water budget against the oracle's
REFL_DBZ_RMS = 1e-3


def _run_mixed_f32(ctx, over, wl, itimestep=1):
    import tempo_gb300 as tg
    f = {k: np.ascontiguousarray(v.astype(np.float32)) for k, v in wl.fields.items()}
    d = make_diags(f["p"].shape, dtype=np.float32)
    ctx.set_precision(tg.PREC_MIXED)
    try:
        ctx.run(f, wl.dt, itimestep, diags=d, cfgs=tg.default_cfgs(**over))
    finally:
        ctx.set_precision(tg.PREC_FP64)
    return f, d


def _rounded(wl):
    from copy import copy
    w2 = copy(wl)
    w2.fields = {k: v.astype(np.float32).astype(np.float64) for k, v in wl.fields.items()}
    return w2


def _metrics(fm, dm, fo, do, wl, clean):
    out = {}
    for n in PROG:
        if n not in fm or n not in fo:
            continue
        m = np.broadcast_to(clean[:, None, :], fo[n].shape)
        a = np.asarray(fm[n], np.float64)[m]
        b = fo[n][m]
        d = np.abs(a - b)
        scale = max(np.abs(b).max(), 1e-300)
        out[n] = dict(rel_rms=float(np.sqrt((d * d).sum() / max((b * b).sum(), 1e-300))),
                      normwise=float(d.max() / scale),
                      scaled_max=float((d / np.maximum(np.abs(b), 1e-7 * scale)).max()),
                      frac_r1=float((d / np.maximum(np.abs(b), FLOOR[n]) > 1e-5).mean()))
    from tempo_gb300.workloads import RD
    x = wl.fields
    rho = RD / 461.5 * x["p"] / (RD * x["t"] * (np.maximum(1e-10, x["qv"]) + RD / 461.5))

    def water(F, D):
        q = sum(np.asarray(F[n], np.float64) for n in ("qv", "qc", "qr", "qi", "qs", "qg"))
        return (q * rho * x["dz"]).sum(axis=1) + sum(np.asarray(D[n], np.float64) for n in DIAG2[:4])

    w0 = water(x, {n: 0.0 for n in DIAG2[:4]})
    out["budget"] = float((np.abs(water(fm, dm) - water(fo, do)) / w0)[clean].max())
    e = np.abs(np.asarray(dm["refl10cm"], np.float64) - do["refl10cm"])[np.broadcast_to(clean[:, None, :], do["refl10cm"].shape)]
    out["refl10cm_dbz"] = dict(max=float(e.max()), rms=float(np.sqrt((e * e).mean())))
    return out


def _check(out):
    bad = []
    for n, v in out.items():
        if n in ("budget", "refl10cm_dbz"):
            continue
        if v["rel_rms"] > REL_RMS[n]:
            bad.append((n, "rel_rms", v["rel_rms"]))
        if v["normwise"] > NORMWISE.get(n, 1e-4):
            bad.append((n, "normwise", v["normwise"]))
        if v["scaled_max"] > SCALED_MAX.get(n, 0.05):
            bad.append((n, "scaled_max", v["scaled_max"]))
        if v["frac_r1"] > FRAC_R1:
            bad.append((n, "frac_r1", v["frac_r1"]))
    if out["budget"] > BUDGET:
        bad.append(("budget", out["budget"]))
    if out["refl10cm_dbz"]["rms"] > REFL_DBZ_RMS:
        bad.append(("refl10cm_dbz", out["refl10cm_dbz"]))
    return bad


@pytest.mark.parametrize("case", ["stretched_grid", "hail_convection", "stretched_grid_dt120"])
def test_mixed_against_oracle(ctx_nohail, ctx_hail, oracle_mod, case):
    """stretched_grid_dt120: the stretched-grid columns with a 120 s step, where rain near the
    surface needs more than 8 sedimentation substeps, so the mixed form's level-by-level
    walk runs in several passes with the state stored in FP32 between them."""
    from tempo_gb300 import workloads as W
    hail = case == "hail_convection"
    if hail:
        wl = _rounded(W.hail_convection(ni=32, nj=16))
    elif case == "stretched_grid_dt120":
        wl = _rounded(W.stretched_grid(ni=64, nj=16, steps=1, dt=120.0))
    else:
        wl = _rounded(W.stretched_grid(ni=64, nj=16, steps=1))
    ctx = ctx_hail if hail else ctx_nohail
    over = dict(hailaware_flag=int(hail), rain_med_vol_diam_flag=1, graupel_med_vol_diam_flag=1,
                cloud_number_mixing_ratio_flag=1)
    oracle_mod.init(hail)
    ties = np.zeros(wl.fields["p"].shape[::2], np.int32)
    fo, do = run_oracle(oracle_mod, over, wl, ties=ties)
    fm, dm = _run_mixed_f32(ctx, over, wl)
    oracle_mod.init(True)
    clean = (ties & 1) == 0
    assert clean.mean() > 0.5
    out = _metrics(fm, dm, fo, do, wl, clean)
    print(case, "tie columns", int((~clean).sum()), "of", clean.size)
    for n, v in out.items():
        print(f"  {n:14s} {v}")
    bad = _check(out)
    assert not bad, bad
