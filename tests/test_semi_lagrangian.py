"""Semi-Lagrangian sedimentation of rain and graupel (semi_sedi_flag,
src/module_mp_tempo_main.F90:595-671, scheme :1562-1749).

The reference's tests run this path without assertions, so parity rests on the oracle's
restatement: the GPU FP64 step against the oracle to 1e-12 (with the hail-aware
density-class ties handled as in the explicit-path tests), and on the CPU the property
that the flag changes only columns where rain or graupel sediment."""
import numpy as np
import pytest

from parity_util import compare, compare_with_ties, run_gpu, run_oracle, worst

TOL64 = 1e-12
SEMI = dict(hailaware_flag=0, semi_sedi_flag=1)


def test_oracle_semi_changes_only_rain_and_graupel_columns(oracle_mod):
    from tempo_gb300 import workloads as W
    oracle_mod.init(False)
    wl = W.stretched_grid(ni=32, nj=8, steps=1, dt=60.0)
    fe, de = run_oracle(oracle_mod, dict(hailaware_flag=0), wl)
    fs, ds = run_oracle(oracle_mod, SEMI, wl)
    moving = np.zeros(wl.fields["p"].shape[::2], bool)
    for k in ("qr", "qg"):
        moving |= (fe[k] > 1e-12).any(axis=1) | (wl.fields[k] > 1e-12).any(axis=1)
    assert moving.any() and (~moving).any()
    for k in ("t", "qv", "qc", "qr", "nr", "qi", "ni", "qs", "qg"):
        a, b = fe[k].transpose(0, 2, 1)[~moving], fs[k].transpose(0, 2, 1)[~moving]
        assert np.array_equal(a, b), k
        assert np.isfinite(fs[k]).all(), k
    # the scheme moves rain: the two paths differ where rain falls
    assert not np.array_equal(fe["qr"], fs["qr"])
    assert (ds["rain_precip"] >= 0).all()
    oracle_mod.init(True)


def _fractions_over(fa, da, fb, db, tol, inputs):
    """Fraction of points (or columns, for 2-D diagnostics) above tol per field."""
    from parity_util import DIAG2, DIAG3, FLOOR, OUT3, rel_err
    out = {}
    for n in OUT3:
        if n in fa and n in fb:
            out[n] = float(np.mean(rel_err(fa[n], fb[n], FLOOR[n], inputs.get(n)) > tol))
    for n in tuple(DIAG2) + tuple(DIAG3):
        if n in da and n in db and not (np.isnan(da[n]).all() and np.isnan(db[n]).all()):
            out[n] = float(np.mean(rel_err(da[n], db[n], FLOOR[n]) > tol))
    return out


# The remap decides by comparisons of departure heights with cell edges and by the
# sign tests of its monotonicity limiter, so last-bit differences (the device's and
# glibc's pow in the fall speeds) flip some decisions and move those levels' values by
# O(1).  The oracle shows the same behaviour against itself: perturbing its inputs in
# the last bit changes a fraction of its semi-Lagrangian outputs beyond 1e-12 (and none
# of the explicit path's rain).  FP64 parity is stated against that calibration: per
# field, the fraction of points beyond 1e-12 from the oracle is at most three times the
# oracle's own last-bit fraction, or 1e-3.
def _self_fraction(oracle_mod, over, wl, state=None, itimestep=1):
    from copy import copy
    base = state if state is not None else wl.fields
    rng = np.random.default_rng(17)
    w2 = copy(wl)
    w2.fields = {k: (v * (1 + 2e-16 * rng.standard_normal(v.shape))
                     if k in ("t", "qv", "qc", "qr", "nr", "qg", "qs") else v.copy())
                 for k, v in base.items()}
    fa, da = run_oracle(oracle_mod, over, wl, fields=base, itimestep=itimestep)
    fb, db = run_oracle(oracle_mod, over, w2, itimestep=itimestep)
    return _fractions_over(fb, db, fa, da, TOL64, base)


def _check_calibrated(frac, calib):
    bad = {k: (v, calib.get(k, 0.0)) for k, v in frac.items() if v > max(3 * calib.get(k, 0.0), 1e-3)}
    assert not bad, bad


@pytest.mark.gpu
def test_semi_fp64_matches_oracle(ctx_nohail, oracle_mod):
    from tempo_gb300 import workloads as W
    oracle_mod.init(False)
    wl = W.stretched_grid(ni=64, nj=8, steps=2, dt=60.0)
    state = {k: v.copy() for k, v in wl.fields.items()}
    for step in (1, 2):
        calib = _self_fraction(oracle_mod, SEMI, wl, state, step)
        fo, do = run_oracle(oracle_mod, SEMI, wl, fields=state, itimestep=step)
        fg, dg = run_gpu(ctx_nohail, SEMI, wl, fields=state, itimestep=step)
        _check_calibrated(_fractions_over(fg, dg, fo, do, TOL64, state), calib)
        state = fo
    oracle_mod.init(True)


@pytest.mark.gpu
def test_semi_hail_fp64_matches_oracle(ctx_hail, oracle_mod):
    from tempo_gb300 import workloads as W
    oracle_mod.init(True)
    wl = W.hail_convection(ni=32, nj=16, dt=60.0)
    over = dict(hailaware_flag=1, semi_sedi_flag=1, rain_med_vol_diam_flag=1,
                graupel_med_vol_diam_flag=1)
    calib = _self_fraction(oracle_mod, over, wl)
    ties = np.zeros(wl.fields["p"].shape[::2], np.int32)
    fo, do = run_oracle(oracle_mod, over, wl, ties=ties)
    fg, dg = run_gpu(ctx_hail, over, wl)
    # columns with a density-class rounding tie (as in the explicit hail-aware test) aside
    keep = (ties & 3) == 0
    sub = lambda d: {k: (v.transpose(0, 2, 1)[keep] if v.ndim == 3 else v[keep]) for k, v in d.items()}
    _check_calibrated(_fractions_over(sub(fg), sub(dg), sub(fo), sub(do), TOL64, sub(wl.fields)), calib)
    assert keep.mean() > 0.5


@pytest.mark.gpu
def test_semi_mixed_close_to_fp64(tg, ctx_nohail):
    """The mixed form against the FP64 step on the same (FP32-representable) inputs: the
    semi-Lagrangian remap switches between reconstructions at thresholds (its
    monotonicity tests), so its pointwise error fractions may exceed the explicit
    path's, but by a bounded factor; column precipitation agrees to 1e-4."""
    from copy import copy
    from tempo_gb300 import workloads as W
    wl = copy(W.stretched_grid(ni=64, nj=8, steps=1, dt=60.0))
    wl.fields = {k: v.astype(np.float32).astype(np.float64) for k, v in wl.fields.items()}

    def fractions(over):
        f64, d64 = run_gpu(ctx_nohail, over, wl)
        ctx_nohail.set_precision(tg.PREC_MIXED)
        try:
            f32, d32 = run_gpu(ctx_nohail, over, wl, dtype=np.float32)
        finally:
            ctx_nohail.set_precision(tg.PREC_FP64)
        out = {}
        for k in ("t", "qv", "qr", "nr"):
            floor = 1e-6 if k == "nr" else 1e-12
            scale = np.maximum(np.abs(f64[k]), np.maximum(np.abs(wl.fields[k]), floor))
            out[k] = float(np.mean(np.abs(f32[k].astype(np.float64) - f64[k]) / scale > 1e-5))
        p32, p64 = d32["rain_precip"].astype(np.float64), d64["rain_precip"]
        out["precip"] = float(np.max(np.abs(p32 - p64) / np.maximum(p64, 1e-3 * p64.max() + 1e-30)))
        return out

    explicit = fractions(dict(hailaware_flag=0))
    semi = fractions(SEMI)
    for k in ("t", "qv", "qr", "nr"):
        assert semi[k] <= max(5 * explicit[k], 0.05), (k, semi, explicit)
    assert semi["precip"] < 1e-4, (semi, explicit)


@pytest.mark.gpu
def test_semi_rejected_where_unsupported(tg, ctx_nohail):
    torch = pytest.importorskip("torch")
    from tempo_gb300 import workloads as W
    wl = W.stretched_grid(ni=8, nj=4, steps=1, dt=60.0)
    f = {k: torch.tensor(v, device="cuda") for k, v in wl.fields.items()}
    cfg = tg.default_cfgs(hailaware_flag=0, semi_sedi_flag=1)
    with pytest.raises(tg.TempoError) as e:
        ctx_nohail.tl_device(f, {}, wl.dt, 1, cfgs=cfg)
    assert e.value.code == -2
    f32 = {k: v.float() for k, v in f.items()}
    ctx_nohail.set_precision(tg.PREC_MIXED)
    try:
        with pytest.raises(tg.TempoError) as e:
            ctx_nohail.run_device_noalloc(f32, wl.dt, 1, cfgs=cfg)
        assert e.value.code == -2
    finally:
        ctx_nohail.set_precision(tg.PREC_FP64)
