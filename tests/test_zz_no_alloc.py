"""tempo_run_dev_f32_noalloc_c (the mixed step with its scratch in the library's fixed
device array) against tempo_run_dev_f32_c (scratch grown with cudaMalloc), through the
C ABI on the same inputs, two steps in a row.  Both run the same kernels, so the
outputs agree to 1e-6 relative (in practice bit for bit).  Collected last so that it
runs both alone and after every other GPU test in one process."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OUT3 = ("t", "qv", "qc", "qr", "qi", "qs", "qg", "ni", "nr", "nc", "nwfa", "nifa")


def _diags(torch, nj, nk, ni, tg):
    d = {n: torch.zeros((nj, ni), device="cuda") for n in tg.DIAG2}
    d.update({n: torch.zeros((nj, nk, ni), device="cuda")
              for n in ("refl10cm", "re_cloud", "re_ice", "re_snow")})
    return d


def test_noalloc_step_matches_allocating_step(tg, ctx_nohail):
    torch = pytest.importorskip("torch")
    from tempo_gb300 import workloads as W
    ctx = ctx_nohail
    wl = W.stretched_grid(seed=5, ni=40, nj=25, steps=2, dt=30.0)      # 1000 columns x 65 levels
    f = {k: torch.tensor(v.astype(np.float32), device="cuda") for k, v in wl.fields.items()}
    nj, nk, ni = f["p"].shape
    a = {k: v.clone() for k, v in f.items()}
    b = {k: v.clone() for k, v in f.items()}
    da, db = _diags(torch, nj, nk, ni, tg), _diags(torch, nj, nk, ni, tg)
    ctx.set_precision(tg.PREC_MIXED)
    try:
        for it in (1, 2):
            ctx.run_device(a, wl.dt, it, diags=da)           # tempo_run_dev_f32_c
            ctx.run_device_noalloc(b, wl.dt, it, diags=db)   # tempo_run_dev_f32_noalloc_c
            torch.cuda.synchronize()
            for k in OUT3:
                torch.testing.assert_close(b[k], a[k], rtol=1e-6, atol=0.0, msg=f"{k} step {it}")
            for k in da:
                torch.testing.assert_close(db[k], da[k], rtol=1e-6, atol=1e-30, msg=f"{k} step {it}")
    finally:
        ctx.set_precision(tg.PREC_FP64)


def test_noalloc_rejects_tiles_beyond_its_scratch(tg, ctx_nohail):
    torch = pytest.importorskip("torch")
    from tempo_gb300 import workloads as W
    ctx = ctx_nohail
    wl = W.stretched_grid(seed=6, ni=128, nj=64, steps=1, dt=30.0)     # 8192 columns > ~4200
    f = {k: torch.tensor(v.astype(np.float32), device="cuda") for k, v in wl.fields.items()}
    before = {k: v.clone() for k, v in f.items()}
    ctx.set_precision(tg.PREC_MIXED)
    try:
        with pytest.raises(tg.TempoError) as e:
            ctx.run_device_noalloc(f, wl.dt, 1)
        assert e.value.code == -1 and "fixed scratch" in str(e.value)
    finally:
        ctx.set_precision(tg.PREC_FP64)
    torch.cuda.synchronize()
    for k in f:   # rejected before any work: the state is untouched
        assert torch.equal(f[k], before[k]), k


def test_noalloc_allocates_nothing_and_records_no_kernel_times(tg, ctx_nohail):
    """After a first call (which looks up the fixed array), further steps leave the
    device's free memory unchanged; and since the call records no timing events, the
    kernel-times query refuses to report an earlier run's times as this step's."""
    torch = pytest.importorskip("torch")
    from tempo_gb300 import workloads as W
    ctx = ctx_nohail
    wl = W.stretched_grid(seed=7, ni=32, nj=20, steps=4, dt=30.0)       # 640 columns
    f = {k: torch.tensor(v.astype(np.float32), device="cuda") for k, v in wl.fields.items()}
    nj, nk, ni = f["p"].shape
    d = _diags(torch, nj, nk, ni, tg)
    ctx.set_precision(tg.PREC_MIXED)
    try:
        ctx.run_device_noalloc(f, wl.dt, 1, diags=d)
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        for it in (2, 3, 4):
            ctx.run_device_noalloc(f, wl.dt, it, diags=d)
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0, (free0, free1)
        ctx.set_kernel_timing(True)
        try:
            g = {k: v.clone() for k, v in f.items()}
            ctx.run_device(g, wl.dt, 5, diags=d)
            assert ctx.kernel_times()["points"] > 0
            ctx.run_device_noalloc(f, wl.dt, 5, diags=d)
            with pytest.raises(tg.TempoError) as e:
                ctx.kernel_times()
            assert e.value.code == -6
        finally:
            ctx.set_kernel_timing(False)
    finally:
        ctx.set_precision(tg.PREC_FP64)
