"""Melting-layer 10-cm reflectivity (refl10cm_from_melting_flag,
src/module_mp_tempo_diags.F90:59-395): below the column's melting level the snow and
graupel contributions come from melting particles (Maxwell-Garnett mixing, Rayleigh
backscatter over 50 radar bins).

The reference's tests do not run this path, so parity rests on the oracle's
restatement: on the CPU, the flag changes refl10cm alone and only below the melting
level; on the GPU, the FP64 step against the oracle to 1e-12 on the columns without a
graupel density-class rounding tie (as in the explicit hail-aware parity test), and the
mixed form within the dBZ bound of the mixed-precision tests."""
import numpy as np
import pytest

from parity_util import compare_with_ties, run_gpu, run_oracle

TOL64 = 1e-12
MELT = dict(hailaware_flag=1, refl10cm_from_melting_flag=1)


def test_oracle_melting_changes_only_reflectivity(oracle_mod):
    from tempo_gb300 import workloads as W
    oracle_mod.init(True)
    wl = W.hail_convection(ni=16, nj=8)
    fa, da = run_oracle(oracle_mod, dict(hailaware_flag=1), wl)
    fb, db = run_oracle(oracle_mod, MELT, wl)
    for k in fa:
        assert np.array_equal(fa[k], fb[k]), k
    for k in da:
        if k != "refl10cm":
            assert np.array_equal(da[k], db[k], equal_nan=True), k
    changed = da["refl10cm"] != db["refl10cm"]
    assert changed.any()
    assert np.isfinite(db["refl10cm"]).all() and (db["refl10cm"] >= -35.0).all()
    # a changed level lies below a level that is warmer than 0 C with rain
    t0 = 273.15
    nj, nk, ni = changed.shape
    for j in range(nj):
        for i in range(ni):
            ks = np.nonzero(changed[j, :, i])[0]
            if ks.size:
                warm = np.nonzero((fb["t"][j, :, i] > t0) & (fb["qr"][j, :, i] > 1e-12))[0]
                assert warm.size and ks.max() < warm.max() + 1, (j, i, ks, warm)
    oracle_mod.init(True)


@pytest.mark.gpu
def test_melting_fp64_matches_oracle(ctx_hail, oracle_mod):
    from tempo_gb300 import workloads as W
    oracle_mod.init(True)
    wl = W.hail_convection(ni=32, nj=16)
    over = dict(MELT, rain_med_vol_diam_flag=1, graupel_med_vol_diam_flag=1)
    ties = np.zeros(wl.fields["p"].shape[::2], np.int32)
    fo, do = run_oracle(oracle_mod, over, wl, ties=ties)
    fg, dg = run_gpu(ctx_hail, over, wl)
    clean, b2, moved, which, frac = compare_with_ties(fg, dg, fo, do, ties, TOL64,
                                                      inputs=wl.fields)
    assert clean < 1e-10, (which, clean)
    assert frac <= 1e-3, (frac, which, clean)
    # a density-class tie moves the graupel contribution, and with melting that reaches
    # every level below the melting level of the column: a few more columns than on the
    # explicit path
    assert moved <= max(1, ties.size // 50), moved
    # the melting path is exercised
    fn, dn = run_oracle(oracle_mod, dict(hailaware_flag=1), wl)
    assert (dn["refl10cm"] != do["refl10cm"]).mean() > 0.01


@pytest.mark.gpu
def test_melting_mixed_close_to_fp64(tg, ctx_hail):
    from tempo_gb300 import workloads as W
    wl = W.hail_convection(ni=32, nj=16)
    wl.fields = {k: v.astype(np.float32).astype(np.float64) for k, v in wl.fields.items()}
    f64, d64 = run_gpu(ctx_hail, MELT, wl)
    ctx_hail.set_precision(tg.PREC_MIXED)
    try:
        f32, d32 = run_gpu(ctx_hail, MELT, wl, dtype=np.float32)
    finally:
        ctx_hail.set_precision(tg.PREC_FP64)
    dz = np.abs(d32["refl10cm"].astype(np.float64) - d64["refl10cm"])
    # the bound of the mixed-precision tests: |d dBZ| > 0.1 on at most 0.2 % of points
    # (plus the points where a species' existence flips between the two forms)
    assert float(np.mean(dz > 0.1)) <= 5e-3, float(np.mean(dz > 0.1))


@pytest.mark.gpu
def test_melting_rejected_where_unsupported(tg, ctx_hail):
    torch = pytest.importorskip("torch")
    from tempo_gb300 import workloads as W
    wl = W.hail_convection(ni=8, nj=4)
    f = {k: torch.tensor(v, device="cuda") for k, v in wl.fields.items()}
    cfg = tg.default_cfgs(**MELT)
    refl = torch.zeros(f["p"].shape, dtype=torch.float64, device="cuda")
    with pytest.raises(tg.TempoError) as e:
        ctx_hail.tl_device(f, {}, wl.dt, 1, diags={"refl10cm": refl}, cfgs=cfg)
    assert e.value.code == -2
