"""Conditioning of the reference step at FP32 resolution, on the oracle (CPU).

The FP64 oracle is stepped twice from the same FP32-representable state, once with
every nonzero input value (t, p, w and the prognostic fields) moved by at most one FP32
unit in the last place (a relative change of at most 6e-8).  The step amplifies that
change: cloud water condenses from the difference qv - qvs, and number concentrations,
clamped diameters and table bins react to it.  So a relative error bound of 1e-5 per
point against the FP64 oracle is finer than the step's own response to an FP32 rounding
of its inputs; these tests pin that response, the yardstick for the mixed form's
pointwise errors.
"""
from copy import copy

import numpy as np
import pytest

from parity_util import FLOOR, run_oracle

PERTURB = ("t", "p", "w", "qv", "qc", "qr", "qi", "qs", "qg", "ni", "nr", "nc", "ng", "qb")


def _fp32(wl):
    w2 = copy(wl)
    w2.fields = {k: (v.astype(np.float32).astype(np.float64) if v.dtype == np.float64 else v)
                 for k, v in wl.fields.items()}
    return w2


def _one_ulp(wl, seed):
    """Each nonzero input value moved by -1, 0 or +1 FP32 ulp (zeros stay zero, so
    no species appears or disappears)."""
    rng = np.random.default_rng(seed)
    w2 = _fp32(wl)
    f = dict(w2.fields)
    for k in PERTURB:
        if k not in f:
            continue
        v = f[k].astype(np.float32)
        s = rng.integers(-1, 2, size=v.shape)
        up = np.nextafter(v, np.float32(np.inf))
        dn = np.nextafter(v, np.float32(-np.inf))
        p = np.where(s > 0, up, np.where(s < 0, dn, v))
        f[k] = np.where(v == 0, v, p).astype(np.float64)
    w2.fields = f
    return w2


def _response(oracle_mod, wl, hail):
    nj, _, ni = wl.fields["p"].shape
    over = dict(hailaware_flag=int(hail))
    oracle_mod.init(hail)
    try:
        t0 = np.zeros((nj, ni), np.int32)
        t1 = np.zeros((nj, ni), np.int32)
        fa, _ = run_oracle(oracle_mod, over, _fp32(wl), ties=t0)
        fb, _ = run_oracle(oracle_mod, over, _one_ulp(wl, 1), ties=t1)
    finally:
        oracle_mod.init(True)
    clean = (t0 == 0) & (t1 == 0)   # no rounding tie in either step
    out = {}
    for n in ("t", "qv", "qc", "qr", "qg", "nc"):
        if n not in fa:
            continue
        m = np.broadcast_to(clean[:, None, :], fa[n].shape)
        a, b = fb[n][m], fa[n][m]
        d = np.abs(a - b)
        out[n] = dict(rel_rms=float(np.sqrt((d * d).sum() / (b * b).sum())),
                      frac=float((d / np.maximum(np.abs(b), FLOOR[n]) > 1e-5).mean()))
    return out


@pytest.mark.parametrize("case", ["stretched_grid", "hail_convection"])
def test_one_fp32_ulp_of_input_moves_outputs_beyond_1e5(oracle_mod, oracle_tables, case):
    """Measured on these samples (and on 262 144 hail-convection columns): t and qv
    follow the perturbation (relative RMS below 1e-6, no point beyond 1e-5), while 15-17 %
    of cloud-water points, 0.3-1 % of graupel points and 0.3-0.4 % of cloud-number
    points move by more than 1e-5, and the cloud number's relative RMS exceeds 1e-5."""
    from tempo_gb300 import workloads as W
    hail = case == "hail_convection"
    wl = W.hail_convection(ni=32, nj=16) if hail else W.stretched_grid(ni=64, nj=16, steps=1)
    r = _response(oracle_mod, wl, hail)
    assert r["t"]["rel_rms"] < 1e-6 and r["t"]["frac"] == 0.0, r["t"]
    assert r["qv"]["rel_rms"] < 1e-6 and r["qv"]["frac"] == 0.0, r["qv"]
    assert r["qc"]["frac"] > 0.05, r["qc"]
    assert r["qg"]["frac"] > 1e-3, r["qg"]
    assert r["nc"]["frac"] > 1e-3 and r["nc"]["rel_rms"] > 1e-5, r["nc"]


def test_one_fp32_ulp_of_input_flips_decisions(oracle_mod, oracle_tables):
    """The same change flips table bins and branches of the FP64 step itself: 9.0e-5 of
    the stretched-grid sample's points (droplet-evaporation bins, condensation and final
    existence checks), 1.9e-4 on 65 536 hail-convection columns -- the yardstick for
    the mixed form's decision flips against the oracle."""
    from parity_util import make_diags
    from tempo_gb300 import workloads as W
    from trace_util import mismatches
    wl = W.stretched_grid(ni=64, nj=16, steps=1)
    over = dict(rain_med_vol_diam_flag=1, graupel_med_vol_diam_flag=1,
                cloud_number_mixing_ratio_flag=1, hailaware_flag=0)
    nj, nz, ni = wl.fields["p"].shape

    def trace(w):
        f = {k: v.copy() for k, v in w.fields.items()}
        tr = np.zeros(oracle_mod.trace_size(ni * nj, nz), np.int32)
        ties = np.zeros((nj, ni), np.int32)
        rc = oracle_mod.run(oracle_mod.default_cfgs(**over), w.dt, 1, f, make_diags(f["p"].shape),
                            ties=ties, trace=tr)
        assert rc == 0
        return tr, ties

    oracle_mod.init(False)
    try:
        a, ta = trace(_fp32(wl))
        b, tb = trace(_one_ulp(wl, 1))
    finally:
        oracle_mod.init(True)
    clean = ((ta.ravel() | tb.ravel()) & 1) == 0
    flips = sum(mismatches(b, a, ni * nj, nz, clean).values()) / (int(clean.sum()) * nz)
    assert 1e-5 < flips < 1e-3, flips
