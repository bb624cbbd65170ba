"""ML cloud number (ml_for_nc_flag with no nc array, src/module_mp_tempo_main.F90:364-371,
network src/module_mp_tempo_ml.F90:104-176): each level's single-moment cloud number is
the network's prediction from qc, qr, qi, qs, p, T and w.  The network's weights are
the reference's (tests/golden/ml_cloud_number.npz, parsed from its source by
tests/golden/make_ml_weights.py); the library ships none and takes them from the host.

Parity rests on the oracle's restatement of the network: GPU FP64 against the oracle
to 1e-12."""
from copy import copy
from pathlib import Path

import numpy as np
import pytest

from parity_util import compare, run_gpu, run_oracle, worst

TOL64 = 1e-12
ML = dict(hailaware_flag=0, ml_for_nc_flag=1)
WEIGHTS = Path(__file__).resolve().parent / "golden" / "ml_cloud_number.npz"


def _workload():
    from tempo_gb300 import workloads as W
    wl = copy(W.stretched_grid(ni=32, nj=8, steps=1))
    wl.fields = {k: v for k, v in wl.fields.items() if k != "nc"}  # single-moment cloud
    return wl


def test_oracle_ml_changes_the_step(oracle_mod):
    oracle_mod.init(False)
    oracle_mod.set_ml(dict(np.load(WEIGHTS)))
    wl = _workload()
    fa, _ = run_oracle(oracle_mod, dict(hailaware_flag=0), wl)
    fb, db = run_oracle(oracle_mod, ML, wl)
    fc, _ = run_oracle(oracle_mod, ML, wl)
    assert not np.array_equal(fa["qc"], fb["qc"])  # the predicted number acts
    for k in fb:
        assert np.array_equal(fb[k], fc[k]), k      # and deterministically
        assert np.isfinite(fb[k]).all(), k
    oracle_mod.init(True)


@pytest.mark.gpu
def test_ml_fp64_matches_oracle(tg, oracle_mod, oracle_tables):
    oracle_mod.init(False)
    weights = dict(np.load(WEIGHTS))
    oracle_mod.set_ml(weights)
    ctx = tg.TempoContext(table_dir=oracle_tables, build_tables=False,
                          cfgs=tg.default_cfgs(hailaware_flag=0))
    try:
        ctx.set_ml_cloud_number(weights)
        wl = _workload()
        over = dict(ML, cloud_number_mixing_ratio_flag=1)
        fo, do = run_oracle(oracle_mod, over, wl)
        fg, dg = run_gpu(ctx, over, wl)
        name, e = worst(compare(fg, dg, fo, do, inputs=wl.fields))
        assert e < TOL64, (name, e)
    finally:
        ctx.close()
        oracle_mod.init(True)


@pytest.mark.gpu
def test_ml_without_weights_is_an_error(tg, oracle_tables):
    ctx = tg.TempoContext(table_dir=oracle_tables, build_tables=False,
                          cfgs=tg.default_cfgs(hailaware_flag=0))
    try:
        wl = _workload()
        with pytest.raises(tg.TempoError) as e:
            run_gpu(ctx, ML, wl)
        assert e.value.code == -6
    finally:
        ctx.close()


@pytest.mark.gpu
def test_ml_mixed_close_to_fp64(tg, oracle_tables):
    ctx = tg.TempoContext(table_dir=oracle_tables, build_tables=False,
                          cfgs=tg.default_cfgs(hailaware_flag=0))
    try:
        ctx.set_ml_cloud_number(dict(np.load(WEIGHTS)))
        wl = _workload()
        wl.fields = {k: v.astype(np.float32).astype(np.float64) for k, v in wl.fields.items()}
        f64, _ = run_gpu(ctx, ML, wl)
        ctx.set_precision(tg.PREC_MIXED)
        f32, _ = run_gpu(ctx, ML, wl, dtype=np.float32)
        # the network can predict very few droplets (its exponent is clamped at -6), where
        # the warm-rain rates react strongly to the number; the mixed form evaluates the
        # network in FP32, so more rain points move beyond 1e-5 than on the constant-number
        # path (measured 2.4 %)
        bounds = {"t": 1e-2, "qv": 1e-2, "qr": 5e-2}
        for k, bound in bounds.items():
            scale = np.maximum(np.abs(f64[k]), np.maximum(np.abs(wl.fields[k]), 1e-12))
            frac = float(np.mean(np.abs(f32[k].astype(np.float64) - f64[k]) / scale > 1e-5))
            assert frac <= bound, (k, frac)
    finally:
        ctx.close()


def _with_bl(wl):
    """Boundary-layer cloud water and fraction in the lowest 12 levels (seeded)."""
    rng = np.random.default_rng(41)
    shape = wl.fields["p"].shape
    qbl = np.zeros(shape)
    fbl = np.zeros(shape)
    qbl[:, :12, :] = rng.uniform(0.0, 5e-4, (shape[0], 12, shape[2]))
    fbl[:, :12, :] = rng.uniform(0.05, 1.0, (shape[0], 12, shape[2]))
    w2 = copy(wl)
    w2.fields = dict(wl.fields, qc_bl=qbl, qcfrac_bl=fbl)
    return w2


def test_oracle_bl_changes_only_re_cloud(oracle_mod):
    oracle_mod.init(False)
    oracle_mod.set_ml(dict(np.load(WEIGHTS)))
    from tempo_gb300 import workloads as W
    wl = W.stretched_grid(ni=32, nj=8, steps=1)
    fa, da = run_oracle(oracle_mod, dict(hailaware_flag=0), wl)
    fb, db = run_oracle(oracle_mod, dict(hailaware_flag=0), _with_bl(wl))
    for k in fa:
        if k in ("qc_bl", "qcfrac_bl"):
            continue
        assert np.array_equal(fa[k], fb[k]), k
    for k in da:
        if k != "re_cloud":
            assert np.array_equal(da[k], db[k], equal_nan=True), k
    assert not np.array_equal(da["re_cloud"], db["re_cloud"])
    oracle_mod.init(True)


@pytest.mark.gpu
def test_bl_fp64_matches_oracle(tg, oracle_mod, oracle_tables):
    from tempo_gb300 import workloads as W
    oracle_mod.init(False)
    weights = dict(np.load(WEIGHTS))
    oracle_mod.set_ml(weights)
    ctx = tg.TempoContext(table_dir=oracle_tables, build_tables=False,
                          cfgs=tg.default_cfgs(hailaware_flag=0))
    try:
        ctx.set_ml_cloud_number(weights)
        wl = _with_bl(W.stretched_grid(ni=32, nj=8, steps=1))
        fo, do = run_oracle(oracle_mod, dict(hailaware_flag=0), wl)
        fg, dg = run_gpu(ctx, dict(hailaware_flag=0), wl)
        name, e = worst(compare(fg, dg, fo, do, inputs=wl.fields))
        assert e < TOL64, (name, e)
    finally:
        ctx.close()
        oracle_mod.init(True)
