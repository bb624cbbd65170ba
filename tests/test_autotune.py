"""The autotuner of the mixed form (tempo_autotune_dev_f32_c): it leaves the caller's
state untouched, reports a time for every per-level kernel variant, keeps the fastest,
and every variant computes the same step."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fields(W, torch):
    f = W.config1_torch(seed=3, ni=128, nj=64, nz=65, device="cuda", dtype=torch.float32)
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
    assert 0 <= chosen < 8
    assert all(t > 0 for t in times)
    assert times[chosen] == min(times)


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
