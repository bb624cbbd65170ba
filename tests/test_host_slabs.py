"""Host-array runs of large tiles go in slabs of rows whose copies overlap the other
slabs' steps (tempo_run_f32_c).  The result is the device-array step's, bit for bit,
and memory rows outside the tile stay untouched."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_slabbed_host_run_matches_device_run(tg):
    torch = pytest.importorskip("torch")
    from tempo_gb300 import workloads as W
    ni, nj, nz = 1024, 520, 65
    f = W.stretched_grid_torch(seed=11, ni=ni, nj=nj, nz=nz, device="cuda", dtype=torch.float32)
    # tile rows 5..516 (512 rows = 2 slabs of 262 144 columns) inside memory rows 1..520
    b = [1, ni, 1, nj, 1, nz, 1, ni, 1, nj, 1, nz, 1, ni, 5, 516, 1, nz]
    tj = 516 - 5 + 1
    d = {n: torch.zeros((tj, ni), device="cuda") for n in ("rain_precip", "snow_liquid_equiv_precip")}
    d["refl10cm"] = torch.zeros((tj, nz, ni), device="cuda")
    host = {k: v.cpu().numpy().copy() for k, v in f.items()}
    hdiag = {k: v.cpu().numpy().copy() for k, v in d.items()}
    before = {k: v.copy() for k, v in host.items()}
    ctx = tg.TempoContext(build_tables=True, cfgs=tg.default_cfgs(hailaware_flag=0))
    ctx.set_precision(tg.PREC_MIXED)
    ctx.run(host, 30.0, 1, diags=hdiag, bounds=b)
    st_host = ctx.stats()
    ctx.run_device(f, 30.0, 1, diags=d, bounds=b)
    torch.cuda.synchronize()
    st_dev = ctx.stats()
    assert st_host["columns"] == st_dev["columns"] == ni * tj
    assert st_host["early_exit"] == st_dev["early_exit"]
    # one step per slab: 4 slabs of 131 072 columns
    assert st_host["launches"] == 4 * st_dev["launches"]
    for k in ("substeps_rain", "substeps_graupel", "substeps_snow", "substeps_ice", "substeps_cloud"):
        assert st_host[k] == st_dev[k], k
    for k in host:
        dev = f[k].cpu().numpy()
        assert np.array_equal(host[k], dev, equal_nan=True), k
        for rows in (slice(0, 4), slice(516, nj)):  # memory rows outside the tile
            assert np.array_equal(host[k][rows], before[k][rows]), k
    for k in hdiag:
        assert np.array_equal(hdiag[k], d[k].cpu().numpy(), equal_nan=True), k
