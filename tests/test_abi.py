"""The C ABI without a GPU: the library loads, exports every function that
include/tempo_gb300.h declares, and its GPU-free entry points behave as documented
(defaults of ty_tempo_cfgs, argument checks, a clean error when no device exists)."""
import ctypes
import re
from pathlib import Path

import pytest

HEADER = Path(__file__).resolve().parents[1] / "include" / "tempo_gb300.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\**\s*(tempo_\w+)\s*\(", text, re.M)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for n in ("tempo_init_c", "tempo_run_c", "tempo_run_f32_c", "tempo_run_dev_c",
              "tempo_run_dev_f32_c", "tempo_ctx_destroy", "tempo_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol(tg):
    lib = tg.load_library()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_empty_error(tg):
    lib = tg.load_library()
    assert lib.tempo_version().decode().startswith("tempo_gb300")
    assert isinstance(lib.tempo_last_error(), bytes)


def test_default_cfgs_match_reference(tg):
    # ty_tempo_cfgs defaults, src/module_mp_tempo_cfgs.F90:15-34
    c = tg.default_cfgs().as_dict()
    assert c["aerosolaware_flag"] == 1 and c["hailaware_flag"] == 1
    assert c["ml_for_bl_nc_flag"] == 0 and c["ml_for_nc_flag"] == 0
    assert c["semi_sedi_flag"] == 0 and c["refl10cm_from_melting_flag"] == 0
    assert c["turn_off_micro_flag"] == 0 and c["cloud_condensation_flag"] == 1
    assert c["refl10cm_flag"] == 1 and c["re_cloud_flag"] == 1 and c["re_ice_flag"] == 1
    assert c["re_snow_flag"] == 1 and c["max_hail_diameter_flag"] == 1
    assert c["rain_med_vol_diam_flag"] == 0 and c["graupel_med_vol_diam_flag"] == 0
    assert c["cloud_number_mixing_ratio_flag"] == 0


def test_null_arguments_are_rejected(tg):
    lib = tg.load_library()
    assert lib.tempo_default_cfgs(None) == -1
    assert lib.tempo_ctx_destroy(None) == 0
    assert lib.tempo_set_precision(None, 0) in (-1, -6)
    out = (ctypes.c_long * 8)()
    assert lib.tempo_last_stats_c(None, out) in (-1, -6)
    cfg = tg.default_cfgs()
    rc = lib.tempo_run_c(None, ctypes.byref(cfg), 20.0, 1, *([None] * 29), None,
                         *([1] * 18), None)
    assert rc in (-1, -6)
    assert lib.tempo_last_error().decode()


def test_init_without_gpu_fails_cleanly(tg):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(tg.TempoError) as e:
        tg.TempoContext(build_tables=True)
    assert "TEMPO_ERR_CUDA" in str(e.value)


def test_missing_library_fails_loudly(tg, tmp_path):
    saved = tg._lib
    tg._lib = None
    try:
        with pytest.raises(tg.TempoError):
            tg.load_library(tmp_path / "missing.so")
    finally:
        tg._lib = saved
