"""Table indices and branch decisions of the GPU step, compared exactly with the oracle's.

A test-only build of the library (TEMPO_TRACE) and the oracle record, for every point of
a step, each table index a rate routine uses (efficiency bins of rain-cloud and
snow-cloud collection, the rain-snow, rain-graupel, freezing and ice-autoconversion
table indices, the droplet-evaporation bins), the existence and limit decisions of
each pass of the check routines (with the graupel density class and the cloud shape
parameter), the over-depletion limiter's branches, and per column the sedimentation
substep counts and top levels.  The FP64 drop-in must take every decision the oracle
takes (src/module_mp_tempo_main.F90:891-1231 checks, :2279-2858 rates and indices,
:1313-1438 limiter, :593-727 sedimentation).  Columns whose oracle step passed a
rounding tie of an index (the graupel density class nint(10 rg / rb) at its clamp,
main:1171/1200, or a substep count int(dt vt / dz + 1)) are excluded: there the
result of the reference itself depends on the last bit of a libm result.

The mixed form's decisions are counted against the oracle's (the precision study):
its FP32 values can land on the other side of a bin edge or threshold.

The same build checks every table index against its table's bounds before the read
(TR_RANGE): a bad index sets its site's bit and is clamped.  No point of any case, in
either form, may set one."""
import numpy as np
import pytest

from parity_util import make_diags
from trace_util import TRACE_COLUMN, TRACE_POINT, mismatches, trace_library

pytestmark = pytest.mark.gpu

# mixed form: decisions that differ from the oracle's, per point and over all slots
MIXED_FLIP_BOUND = 5e-4
TR_RANGE = 14  # TraceSlot::TR_RANGE


def _oracle_trace(oracle_mod, wl, over, hail):
    oracle_mod.init(hail)
    f = {k: v.copy() for k, v in wl.fields.items()}
    d = make_diags(f["p"].shape)
    nj, nz, ni = f["p"].shape
    tr = np.zeros(oracle_mod.trace_size(ni * nj, nz), np.int32)
    ties = np.zeros((nj, ni), np.int32)
    assert oracle_mod.run(oracle_mod.default_cfgs(**over), wl.dt, 1, f, d, ties=ties, trace=tr) == 0
    return tr, ties


def _gpu_trace(tg, lib, ctx, wl, over, mixed):
    torch = pytest.importorskip("torch")
    dtype = torch.float32 if mixed else torch.float64
    f = {k: torch.tensor(v, device="cuda", dtype=dtype) for k, v in wl.fields.items()}
    nj, nz, ni = f["p"].shape
    d = {n: torch.zeros((nj, ni), device="cuda", dtype=dtype) for n in tg.DIAG2}
    d.update({n: torch.zeros((nj, nz, ni), device="cuda", dtype=dtype) for n in tg.DIAG3})
    tr = torch.zeros(ni * nj * nz * TRACE_POINT + ni * nj * TRACE_COLUMN, device="cuda",
                     dtype=torch.int32)
    assert lib.tempo_set_trace_c(ctx._h, tr.data_ptr()) == 0
    ctx.set_precision(tg.PREC_MIXED if mixed else tg.PREC_FP64)
    try:
        ctx.run_device(f, wl.dt, 1, diags=d, cfgs=tg.default_cfgs(**over))
        torch.cuda.synchronize()
    finally:
        ctx.set_precision(tg.PREC_FP64)
        lib.tempo_set_trace_c(ctx._h, None)
    return tr.cpu().numpy()


def _workloads():
    from tempo_gb300 import workloads as W
    diag = dict(rain_med_vol_diam_flag=1, graupel_med_vol_diam_flag=1,
                cloud_number_mixing_ratio_flag=1)
    return [
        ("uniform_grid", W.uniform_grid(ncol=256), dict(diag, hailaware_flag=0), False),
        ("stretched_grid", W.stretched_grid(ni=64, nj=16, steps=1), dict(diag, hailaware_flag=0), False),
        ("hail_convection", W.hail_convection(ni=32, nj=16), dict(diag, hailaware_flag=1), True),
    ]


def _rounded(wl):
    from copy import copy
    w2 = copy(wl)
    w2.fields = {k: v.astype(np.float32).astype(np.float64) for k, v in wl.fields.items()}
    return w2


def _run(tg, oracle_mod, oracle_tables, case, mixed):
    name, wl, over, hail = _workloads()[case]
    if mixed:
        wl = _rounded(wl)
    nj, nz, ni = wl.fields["p"].shape
    ref, ties = _oracle_trace(oracle_mod, wl, over, hail)
    with trace_library(tg) as lib:
        ctx = tg.TempoContext(table_dir=oracle_tables, build_tables=False,
                              cfgs=tg.default_cfgs(hailaware_flag=int(hail)))
        try:
            got = _gpu_trace(tg, lib, ctx, wl, over, mixed=mixed)
        finally:
            ctx.close()
    oracle_mod.init(True)
    clean = (ties.ravel() & 1) == 0
    return name, ref, got, clean, ni * nj, nz


@pytest.mark.parametrize("case", [0, 1, 2], ids=["uniform_grid", "stretched_grid", "hail_convection"])
def test_fp64_decisions_equal_the_oracle(tg, oracle_mod, oracle_tables, case):
    name, ref, got, clean, ncol, nz = _run(tg, oracle_mod, oracle_tables, case, mixed=False)
    assert clean.mean() > 0.5
    ncheck = int(np.count_nonzero(ref))
    assert ncheck > 1000, ncheck  # the trace recorded decisions
    bad = {k: v for k, v in mismatches(got, ref, ncol, nz, clean).items() if v}
    print(name, "decisions recorded", ncheck, "tie columns", int((~clean).sum()), "mismatches", bad)
    assert not bad, (name, bad)
    _assert_indices_in_range(got, ncol, nz)


def _assert_indices_in_range(got, ncol, nz):
    pts = got[: ncol * nz * TRACE_POINT].reshape(ncol, nz, TRACE_POINT)
    rng = pts[:, :, TR_RANGE]
    sites = int(np.bitwise_or.reduce(rng.ravel()))
    assert not rng.any(), ("table index out of range", int(np.count_nonzero(rng)), hex(sites))


@pytest.mark.parametrize("case", [1, 2], ids=["stretched_grid", "hail_convection"])
def test_mixed_decision_census(tg, oracle_mod, oracle_tables, case):
    """The mixed form against the oracle on the same FP32-rounded inputs: per slot, the
    number of points (columns) where an FP32 value took another table bin or branch.
    Printed for the precision study; bounded so that a regression shows."""
    name, ref, got, clean, ncol, nz = _run(tg, oracle_mod, oracle_tables, case, mixed=True)
    mm = mismatches(got, ref, ncol, nz, clean)
    npts = int(clean.sum()) * nz
    frac = {k: v / npts for k, v in mm.items() if v}
    print(name, "points", npts, "mixed-form decision flips per point", frac)
    assert sum(mm.values()) / npts < MIXED_FLIP_BOUND, frac
    _assert_indices_in_range(got, ncol, nz)
