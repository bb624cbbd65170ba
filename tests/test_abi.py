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


def _bounds(ni=4, nk=5, nj=3):
    # ids..kde, ims..kme, its..kte
    return [1, ni, 1, nj, 1, nk] * 3


def _run_args(tg, dt=20.0, bounds=None, drop=(), nk=5):
    """tempo_run_c arguments with host arrays for every required input."""
    import numpy as np
    shape = (3, nk, 4)
    keep = {}
    ptrs = []
    for n in tg.FIELDS:
        if n in ("th", "pii", "nc", "nwfa", "nifa", "ng", "qb") or n in drop:
            ptrs.append(None)
            continue
        a = np.full(shape, 280.0 if n == "t" else 1e5 if n == "p" else 100.0 if n == "dz" else 0.0)
        keep[n] = a
        ptrs.append(a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return keep, [ctypes.byref(tg.default_cfgs()), dt, 1, *ptrs, *([None] * 10), None,
                  *(bounds or _bounds(nk=nk)), None]


@pytest.mark.parametrize("case,expect", [
    ("ok_args_no_context", -6),
    ("dt_zero", -1),
    ("dt_negative", -1),
    ("kte_below_kts", -1),
    ("single_level", -1),
    ("tile_outside_memory", -1),
    ("no_pressure", -1),
    ("no_temperature", -1),
])
def test_run_argument_checks_precede_the_context(tg, case, expect):
    """tempo_run's argument list is validated before the context is looked at, so a
    bad list reads TEMPO_ERR_ARG on any machine; a good list with no context reads
    TEMPO_ERR_STATE."""
    lib = tg.load_library()
    b = _bounds()
    dt, drop = 20.0, ()
    if case == "dt_zero":
        dt = 0.0
    elif case == "dt_negative":
        dt = -30.0
    elif case == "kte_below_kts":
        b[-2], b[-1] = 5, 4            # kts = 5, kte = 4
    elif case == "single_level":
        b[-2], b[-1] = 2, 2
    elif case == "tile_outside_memory":
        b[13] = 9                      # ite beyond ime = 4
    elif case == "no_pressure":
        drop = ("p",)
    elif case == "no_temperature":
        drop = ("t",)
    keep, args = _run_args(tg, dt=dt, bounds=b, drop=drop)
    for fn in (lib.tempo_run_c,):
        rc = fn(None, *args)
        assert rc == expect, (case, rc, lib.tempo_last_error())
        assert lib.tempo_last_error().decode()


def test_removed_status_code_is_not_declared():
    text = HEADER.read_text()
    assert "TEMPO_ERR_TIMEOUT" not in text


def test_f32_host_entry_takes_the_full_tempo_run_list():
    """tempo_run_f32_c and tempo_run_c declare the same parameter names in the same
    order (a -DSINGLE_PREC reference build keeps tempo_run's list, machine.F90:13-17)."""
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)

    def params(fn):
        m = re.search(fn + r"\s*\((.*?)\);", text, re.S)
        return [re.split(r"[\s*]+", p.strip())[-1] for p in m.group(1).split(",")]

    assert params("tempo_run_f32_c") == params("tempo_run_c")
