"""The autotuner of the mixed form (tempo_autotune_dev_f32_c): it leaves the caller's
state untouched, reports a time for every per-level kernel variant in both point
orders, keeps the fastest, and every variant and order computes the same step."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fields(W, torch):
    f = W.stretched_grid_torch(seed=3, ni=128, nj=64, nz=65, device="cuda", dtype=torch.float32)
    d = {n: torch.zeros((64, 128), device="cuda") for n in ("rain_precip", "snow_liquid_equiv_precip")}
    d["refl10cm"] = torch.zeros((64, 65, 128), device="cuda")
    return f, d


def test_autotune_picks_fastest_and_keeps_state(tg):
    torch = pytest.importorskip("torch")
    from tempo_gb300 import workloads as W
    ctx = tg.TempoContext(build_tables=True, cfgs=tg.default_cfgs(hailaware_flag=0))
    ctx.set_precision(tg.PREC_MIXED)
    f, d = _fields(W, torch)
    before = {k: v.clone() for k, v in f.items()}
    chosen, times = ctx.autotune_device(f, 30.0, 1, diags=d, reps=1)
    torch.cuda.synchronize()
    for k in f:
        assert torch.equal(f[k], before[k]), k
    assert 0 <= chosen < 16
    assert len(times) == 28 and all(t > 0 for t in times)
    assert times[chosen] == min(times[:16])
    tun = ctx.tuning()
    assert (tun["points_variant"], tun["points_order"]) == (chosen % 8, chosen // 8)
    assert times[16 + tun["sedim_variant"]] == min(times[16:])


def test_every_variant_computes_the_same_step(tg):
    torch = pytest.importorskip("torch")
    from tempo_gb300 import workloads as W
    ctx = tg.TempoContext(build_tables=True, cfgs=tg.default_cfgs(hailaware_flag=0))
    ctx.set_precision(tg.PREC_MIXED)
    ref = None
    for v in range(8):
        ctx.set_points_variant(v)
        f, d = _fields(W, torch)
        ctx.run_device(f, 30.0, 1, diags=d)
        torch.cuda.synchronize()
        out = {k: x.double().cpu().numpy() for k, x in list(f.items()) + list(d.items())}
        if ref is None:
            ref = out
            continue
        for k in ref:
            a, b = out[k], ref[k]
            # same arithmetic; only the register allocation differs
            assert np.allclose(a, b, rtol=1e-6, atol=1e-30), (v, k, float(np.abs(a - b).max()))


@pytest.mark.parametrize("precision,variant", [("mixed", 4), ("mixed", 5), ("fp64", 0)])
def test_regime_order_is_bit_identical(tg, precision, variant):
    """The regime order changes only which thread computes a point: two steps in
    regime order and in level-major order give identical bits in every field (variant 5
    runs its blocks in lockstep)."""
    torch = pytest.importorskip("torch")
    from tempo_gb300 import workloads as W
    outs = []
    for order in (0, 1):
        ctx = tg.TempoContext(build_tables=True, cfgs=tg.default_cfgs(hailaware_flag=0))
        if precision == "mixed":
            ctx.set_precision(tg.PREC_MIXED)
            ctx.set_points_variant(variant)
            f, d = _fields(W, torch)
        else:
            f, d = _fields(W, torch)
            f = {k: v.double() for k, v in f.items()}
            d = {k: v.double() for k, v in d.items()}
        ctx.set_points_order(order)
        ctx.set_kernel_timing(True)
        for it in (1, 2):
            ctx.run_device(f, 30.0, it, diags=d)
        times = ctx.kernel_times()
        stats = ctx.stats()
        torch.cuda.synchronize()
        if order:
            assert times["order"] > 0
        assert stats["launches"] == 4 + order
        outs.append({k: x.cpu().numpy() for k, x in list(f.items()) + list(d.items())})
    for k in outs[0]:
        assert np.array_equal(outs[0][k], outs[1][k], equal_nan=True), k


def test_graph_replay_matches_direct_launches(tg):
    """Three steps replayed from captured CUDA graphs give the same state as three
    directly launched steps."""
    torch = pytest.importorskip("torch")
    from tempo_gb300 import workloads as W
    outs = []
    for graphs in (False, True):
        ctx = tg.TempoContext(build_tables=True, cfgs=tg.default_cfgs(hailaware_flag=0))
        ctx.set_precision(tg.PREC_MIXED)
        ctx.set_graphs(graphs)
        f, d = _fields(W, torch)
        for it in (1, 2, 3):
            ctx.run_device(f, 30.0, it, diags=d)
        torch.cuda.synchronize()
        outs.append({k: x.cpu().numpy() for k, x in list(f.items()) + list(d.items())})
    for k in outs[0]:
        assert np.array_equal(outs[0][k], outs[1][k]), k


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_sedim_variants_are_bit_identical(tg, precision):
    """The sedimentation variants change only how many levels' loads a sweep issues
    together, how a column's species map to threads and whether a species' substeps run
    level by level or substep by substep: two steps with each give identical bits in
    every field."""
    torch = pytest.importorskip("torch")
    from tempo_gb300 import workloads as W
    outs = []
    for sv in range(12):
        ctx = tg.TempoContext(build_tables=True, cfgs=tg.default_cfgs(hailaware_flag=0))
        f, d = _fields(W, torch)
        if precision == "mixed":
            ctx.set_precision(tg.PREC_MIXED)
        else:
            f = {k: v.double() for k, v in f.items()}
            d = {k: v.double() for k, v in d.items()}
        ctx.set_sedim_variant(sv)
        assert ctx.tuning()["sedim_variant"] == sv
        for it in (1, 2):
            ctx.run_device(f, 30.0, it, diags=d)
        torch.cuda.synchronize()
        outs.append({k: x.cpu().numpy() for k, x in list(f.items()) + list(d.items())})
    for o in outs[1:]:
        for k in outs[0]:
            assert np.array_equal(outs[0][k], o[k], equal_nan=True), k
