"""The multi-domain batch step (tempo_run_batch_dev_f32_c) against one
tempo_run_dev_f32_c call per domain: domains of different columns, levels (50 to 128) and
time steps stepped by one launch sequence give, domain by domain, the same arrays and
diagnostics bit for bit, over two consecutive steps, in level-major and in regime
order of the points."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DOMAINS = [(300, 50, 10.0, 11), (1200, 65, 30.0, 12), (77, 90, 60.0, 13), (2000, 128, 20.0, 14),
           (1, 65, 30.0, 15)]
OUT = ("t", "qv", "qc", "qr", "qi", "qs", "qg", "ni", "nr", "nc", "nwfa", "nifa")


def _domain(torch, tg, ncol, nz, dt, seed):
    from tempo_gb300 import workloads as W
    wl = W.domain_set_member(ncol, nz, dt, seed)
    f = {k: torch.tensor(v.astype(np.float32), device="cuda") for k, v in wl.fields.items()}
    nj, nk, ni = f["p"].shape
    d = {n: torch.zeros((nj, ni), device="cuda") for n in tg.DIAG2}
    d.update({n: torch.zeros((nj, nk, ni), device="cuda") for n in ("refl10cm", "re_cloud", "re_ice", "re_snow")})
    return f, d, dt


@pytest.mark.parametrize("order", [0, 1], ids=["level-major", "regime"])
def test_batch_equals_per_domain_steps(tg, ctx_nohail, order):
    torch = pytest.importorskip("torch")
    ctx = ctx_nohail
    doms = [_domain(torch, tg, *x) for x in DOMAINS]
    single = [({k: v.clone() for k, v in f.items()}, {k: v.clone() for k, v in d.items()}, dt)
              for f, d, dt in doms]
    batch = [({k: v.clone() for k, v in f.items()}, {k: v.clone() for k, v in d.items()}, dt)
             for f, d, dt in doms]
    ctx.set_precision(tg.PREC_MIXED)
    ctx.set_points_order(order)
    try:
        for it in (1, 2):
            for f, d, dt in single:
                ctx.run_device(f, dt, it, diags=d)
            ctx.run_batch_device([dict(fields=f, diags=d, dt=dt, itimestep=it) for f, d, dt in batch])
            torch.cuda.synchronize()
            for n, ((fs, ds, _), (fb, db, _)) in enumerate(zip(single, batch)):
                for k in OUT:
                    assert torch.equal(fs[k], fb[k]), (n, k, it)
                for k in ds:
                    assert torch.equal(ds[k], db[k]), (n, k, it)
        st = ctx.stats()
        assert st["columns"] == sum(x[0] for x in DOMAINS)
    finally:
        ctx.set_points_order(0)
        ctx.set_precision(tg.PREC_FP64)


def test_batch_rejects_bad_arguments(tg, ctx_nohail):
    torch = pytest.importorskip("torch")
    ctx = ctx_nohail
    f, d, dt = _domain(torch, tg, 64, 65, 30.0, 3)
    ctx.set_precision(tg.PREC_FP64)
    with pytest.raises(tg.TempoError) as e:   # the batch runs the mixed form only
        ctx.run_batch_device([dict(fields=f, diags=d, dt=dt, itimestep=1)])
    assert e.value.code == -6
    ctx.set_precision(tg.PREC_MIXED)
    try:
        with pytest.raises(tg.TempoError) as e:
            ctx.run_batch_device([dict(fields=f, diags=d, dt=-1.0, itimestep=1)])
        assert e.value.code == -1 and "domain 0" in str(e.value)
        with pytest.raises(tg.TempoError) as e:
            ctx.run_batch_device([dict(fields=f, diags=d, dt=dt, itimestep=1)],
                                 cfgs=tg.default_cfgs(hailaware_flag=0, semi_sedi_flag=1))
        assert e.value.code == -2
    finally:
        ctx.set_precision(tg.PREC_FP64)
