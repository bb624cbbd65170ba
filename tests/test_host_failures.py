"""Failure paths of the host side on a GPU context, and the table writer.

- tempo_set_validation: a non-finite or non-physical input is refused with
  TEMPO_ERR_NONFINITE naming the field and the (i, k, j) index, before any array is
  modified (host arrays and device arrays).
- tempo_write_table_c writes the context's tables back in the reference's big-endian
  stream format (src/module_mp_tempo_tables.F90:96-129, 271-311, 412-444), byte for
  byte the files the oracle wrote and the context read.
- tempo_aerosol_surface_emissions_dev_c: nwfa(i, kts, j) += nwfa2d(i, j) * dt over the
  memory range (src/module_mp_tempo_driver.F90:516-529)."""
import filecmp

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fields(dtype=np.float64):
    from tempo_gb300 import workloads as W
    wl = W.uniform_grid(ncol=48)
    return wl, {k: np.ascontiguousarray(v.astype(dtype)) for k, v in wl.fields.items()}


@pytest.mark.parametrize("field,index,value,word", [
    ("qr", (0, 7, 11), np.nan, "qr(12, 8, 1)"),
    ("t", (0, 3, 40), np.inf, "t(41, 4, 1)"),
    ("p", (0, 50, 2), -1.0, "p(3, 51, 1)"),
    ("dz", (0, 0, 0), 0.0, "dz(1, 1, 1)"),
])
def test_validation_refuses_bad_host_input(ctx_nohail, tg, field, index, value, word):
    wl, f = _fields()
    f[field][index] = value
    before = {k: v.copy() for k, v in f.items()}
    ctx_nohail.set_validation(True)
    try:
        with pytest.raises(tg.TempoError) as e:
            ctx_nohail.run(f, wl.dt, 1, cfgs=tg.default_cfgs(hailaware_flag=0))
    finally:
        ctx_nohail.set_validation(False)
    assert e.value.code == -8 and word in str(e.value), str(e.value)
    for k in f:
        np.testing.assert_array_equal(f[k], before[k], err_msg=k)


def test_validation_passes_good_input_and_changes_nothing(ctx_nohail, tg):
    wl, f = _fields()
    g = {k: v.copy() for k, v in f.items()}
    ctx_nohail.run(f, wl.dt, 1, cfgs=tg.default_cfgs(hailaware_flag=0))
    ctx_nohail.set_validation(True)
    try:
        ctx_nohail.run(g, wl.dt, 1, cfgs=tg.default_cfgs(hailaware_flag=0))
    finally:
        ctx_nohail.set_validation(False)
    for k in f:
        np.testing.assert_array_equal(f[k], g[k], err_msg=k)


def test_validation_refuses_bad_device_input(ctx_nohail, tg):
    torch = pytest.importorskip("torch")
    wl, f = _fields()
    d = {k: torch.tensor(v, device="cuda") for k, v in f.items()}
    d["qg"][0, 20, 5] = float("nan")
    before = {k: v.clone() for k, v in d.items()}
    ctx_nohail.set_validation(True)
    try:
        with pytest.raises(tg.TempoError) as e:
            ctx_nohail.run_device(d, wl.dt, 1, cfgs=tg.default_cfgs(hailaware_flag=0))
    finally:
        ctx_nohail.set_validation(False)
    assert e.value.code == -8 and "qg(6, 21, 1)" in str(e.value), str(e.value)
    torch.cuda.synchronize()
    for k in d:
        assert torch.equal(torch.nan_to_num(d[k]), torch.nan_to_num(before[k])), k


@pytest.mark.parametrize("family,fname", [
    ("qr_acr_qs", "qr_acr_qs_data_tempo_v3"),
    ("qr_acr_qg", "qr_acr_qg_data_tempo_v3"),
    ("freezewater", "freeze_water_data_tempo_v3"),
])
def test_table_writer_round_trip(ctx_hail, tg, oracle_tables, tmp_path, family, fname):
    out = tmp_path / fname
    ctx_hail.write_table(family, out)
    assert filecmp.cmp(out, oracle_tables / fname, shallow=False)
    tg.check_table(family, out)


def test_table_writer_output_reloads(tg, ctx_hail, oracle_tables, tmp_path):
    """Tables written by one context and read by a new one give the same step."""
    for family, fname in (("qr_acr_qs", "qr_acr_qs_data_tempo_v3"), ("qr_acr_qg", "qr_acr_qg_data_tempo_v3"),
                          ("freezewater", "freeze_water_data_tempo_v3")):
        ctx_hail.write_table(family, tmp_path / fname)
    (tmp_path / "ccn_activate.bin").write_bytes((oracle_tables / "ccn_activate.bin").read_bytes())
    ctx2 = tg.TempoContext(table_dir=tmp_path, build_tables=False, cfgs=tg.default_cfgs(hailaware_flag=1))
    try:
        for name in ("tcg_racg", "tcs_racs1", "tpi_qrfz", "tni_qcfz"):
            assert np.array_equal(ctx2.get_table(name), ctx_hail.get_table(name)), name
    finally:
        ctx2.close()


def test_aerosol_surface_emissions(ctx_nohail):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    nwfa = rng.uniform(1e8, 1e9, (5, 7, 9))
    nwfa2d = rng.uniform(0.0, 1e4, (5, 9))
    want = nwfa.copy()
    want[:, 1, :] += nwfa2d * 30.0          # kts = 2 (1-based)
    d = torch.tensor(nwfa, device="cuda")
    ctx_nohail.aerosol_surface_emissions(30.0, d, torch.tensor(nwfa2d, device="cuda"), kts=2)
    torch.cuda.synchronize()
    np.testing.assert_allclose(d.cpu().numpy(), want, rtol=1e-15, atol=0)
