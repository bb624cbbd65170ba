"""CPU FP64 restatement of NCAR/TEMPO's column step -- test infrastructure only.

This package is the oracle, not the product.  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py`` (its ``cpu_baseline`` leg and ``--impl reference``) may import it, and
only to compare against or time beside the CUDA product.  The product
(``tempo_gb300``) never loads it.

The C sources restate the Fortran reference line by line (see ``tempo_oracle.h``
for the file:line map).  :func:`build` compiles them with gcc into
``oracle/_build/libtempo_oracle.so``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libtempo_oracle.so"
SOURCES = [HERE / "oracle_init.c", HERE / "oracle_main.c"]
HEADERS = [HERE / "tempo_oracle.h", HERE / "oracle_common.h"]
# -ffp-contract=off: no fused multiply-add (gfortran -O0 on x86-64 uses none, and
# GCC's default in GNU mode would fuse on aarch64).
CFLAGS = ["-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-fno-fast-math",
          "-ffp-contract=off", "-fno-strict-aliasing"]


def build(force: bool = False) -> Path:
    """Compile the restatement; returns the path of the shared library."""
    BUILD.mkdir(exist_ok=True)
    newest = max(p.stat().st_mtime for p in SOURCES + HEADERS)
    if LIB.exists() and not force and LIB.stat().st_mtime >= newest:
        return LIB
    tmp = LIB.with_suffix(f".so.tmp{os.getpid()}")
    cmd = ["gcc", *CFLAGS, "-o", str(tmp), *map(str, SOURCES), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


class OCfg(ctypes.Structure):
    """ty_tempo_cfgs (module_mp_tempo_cfgs.F90:14-35)."""
    _fields_ = [(n, ctypes.c_int) for n in (
        "aerosolaware_flag", "hailaware_flag", "ml_for_bl_nc_flag", "ml_for_nc_flag",
        "semi_sedi_flag", "refl10cm_from_melting_flag", "turn_off_micro_flag",
        "cloud_condensation_flag", "verbose", "check_tables")] + [
        ("single_moment_nc_opt", ctypes.c_char * 32)] + [(n, ctypes.c_int) for n in (
        "refl10cm_flag", "re_cloud_flag", "re_ice_flag", "re_snow_flag",
        "max_hail_diameter_flag", "rain_med_vol_diam_flag", "graupel_med_vol_diam_flag",
        "cloud_number_mixing_ratio_flag")]


DIAG2 = ("rain_precip", "ice_liquid_equiv_precip", "snow_liquid_equiv_precip",
         "graupel_liquid_equiv_precip", "frozen_fraction", "frz_rain_precip",
         "max_hail_diameter_sfc", "max_hail_diameter_column")
DIAG3 = ("refl10cm", "re_cloud", "re_ice", "re_snow", "rain_med_vol_diam",
         "graupel_med_vol_diam", "cloud_number_mixing_ratio")


class ODiag(ctypes.Structure):
    _fields_ = [(n, ctypes.POINTER(ctypes.c_double)) for n in DIAG2 + DIAG3]


_lib = None
_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(str(build()))
        lib.oracle_init.argtypes = [ctypes.c_int]
        for fn in ("oracle_read_ccn", "oracle_read_freezewater", "oracle_read_qr_acr_qs",
                   "oracle_read_qr_acr_qg", "oracle_write_freezewater",
                   "oracle_write_qr_acr_qs", "oracle_write_qr_acr_qg"):
            getattr(lib, fn).argtypes = [ctypes.c_char_p]
        lib.oracle_build_freezewater.argtypes = [ctypes.c_int]
        lib.oracle_build_qr_acr_qs.argtypes = [ctypes.c_int, ctypes.c_int]
        lib.oracle_build_qr_acr_qg.argtypes = [ctypes.c_int, ctypes.c_int]
        lib.oracle_qr_acr_qg_entry.argtypes = [ctypes.c_int] * 5 + [_DP]
        lib.oracle_qr_acr_qs_entry.argtypes = [ctypes.c_int] * 4 + [_DP]
        lib.oracle_table_ptr.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_long)]
        lib.oracle_table_ptr.restype = _DP
        lib.oracle_ccn_ptr.argtypes = [ctypes.POINTER(ctypes.c_long)]
        lib.oracle_ccn_ptr.restype = ctypes.POINTER(ctypes.c_float)
        lib.oracle_set_tie_sink.argtypes = [_IP]
        lib.oracle_set_trace.argtypes = [_IP]
        lib.oracle_set_ml.argtypes = [_DP] * 6
        lib.oracle_param.argtypes = [ctypes.c_char_p, ctypes.c_int]
        lib.oracle_param.restype = ctypes.c_double
        lib.oracle_calc_gamma_p.argtypes = [ctypes.c_double, ctypes.c_double]
        lib.oracle_calc_gamma_p.restype = ctypes.c_double
        lib.oracle_calc_rslf.argtypes = [ctypes.c_double, ctypes.c_double]
        lib.oracle_calc_rslf.restype = ctypes.c_double
        lib.oracle_calc_rsif.argtypes = [ctypes.c_double, ctypes.c_double]
        lib.oracle_calc_rsif.restype = ctypes.c_double
        lib.oracle_snow_moments.argtypes = [ctypes.c_double, ctypes.c_double, _DP]
        lib.oracle_get_cloud_table_index.argtypes = [ctypes.c_double, ctypes.c_double, _IP, _IP]
        lib.oracle_get_snow_table_index.argtypes = [ctypes.c_double, _IP]
        lib.oracle_get_temperature_table_index.argtypes = [ctypes.c_double, _IP]
        lib.oracle_get_rain_table_index.argtypes = [ctypes.c_double, ctypes.c_double, _IP, _IP]
        lib.oracle_get_graupel_table_index.argtypes = [ctypes.c_double, ctypes.c_double,
                                                       ctypes.c_int, _IP, _IP]
        lib.oracle_get_ice_table_index.argtypes = [ctypes.c_double, ctypes.c_double, _IP, _IP]
        lib.oracle_default_cfgs.argtypes = [ctypes.POINTER(OCfg)]
        lib.oracle_run.argtypes = ([ctypes.POINTER(OCfg), ctypes.c_double, ctypes.c_int]
                                   + [_DP] * 21 + [_IP, _IP, ctypes.POINTER(ODiag), ctypes.c_int])
        lib.oracle_last_stats.argtypes = [ctypes.POINTER(ctypes.c_long)]
        _lib = lib
    return _lib


def default_cfgs(**over) -> OCfg:
    cfg = OCfg()
    load().oracle_default_cfgs(ctypes.byref(cfg))
    for k, v in over.items():
        if k == "single_moment_nc_opt":
            cfg.single_moment_nc_opt = v.encode()
        else:
            setattr(cfg, k, int(v))
    return cfg


def init(hailaware: bool = True, ccn_path: str | os.PathLike | None = None) -> None:
    """tempo_init's parameter/bin/small-table part plus the CCN table read."""
    lib = load()
    lib.oracle_init(int(bool(hailaware)))
    if ccn_path is not None:
        rc = lib.oracle_read_ccn(str(ccn_path).encode())
        if rc:
            raise IOError(f"oracle: cannot read CCN table {ccn_path} (code {rc})")


def set_ml(weights: dict) -> None:
    """Weights of the cloud-number network (keys of tests/golden/ml_cloud_number.npz)."""
    arrs = [np.ascontiguousarray(np.asarray(weights[k], dtype=np.float64))
            for k in ("nc_ml_trans_mean", "nc_ml_trans_var", "nc_ml_w00", "nc_ml_b00",
                      "nc_ml_w01", "nc_ml_b01")]
    load().oracle_set_ml(*[a.ctypes.data_as(_DP) for a in arrs])


def param(name: str, idx: int = 0) -> float:
    return load().oracle_param(name.encode(), idx)


def table(name: str) -> np.ndarray:
    """Live view of a module table (Fortran order, flattened)."""
    n = ctypes.c_long()
    p = load().oracle_table_ptr(name.encode(), ctypes.byref(n))
    if not p:
        raise KeyError(name)
    return np.ctypeslib.as_array(p, shape=(n.value,))


def ccn_table() -> np.ndarray:
    n = ctypes.c_long()
    p = load().oracle_ccn_ptr(ctypes.byref(n))
    return np.ctypeslib.as_array(p, shape=(n.value,))


def build_big_tables(naive: bool = False, nthreads: int = 0) -> None:
    lib = load()
    lib.oracle_build_freezewater(nthreads)
    lib.oracle_build_qr_acr_qs(int(naive), nthreads)
    lib.oracle_build_qr_acr_qg(int(naive), nthreads)


def _dp(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_DP)


def run(cfg: OCfg, dt: float, itimestep: int, fields: dict, diags: dict | None = None,
        bounds=None, nthreads: int = 0, ties: np.ndarray | None = None,
        trace: np.ndarray | None = None) -> int:
    """tempo_run over 3-D fields shaped (nj, nk, ni) (Fortran (i,k,j), i fastest).

    ``fields`` maps argument names (t, th, pii, p, w, dz, qv, qc, qr, qi, qs, qg, ni,
    nr, nc, nwfa, nifa, ng, qb, land_input) to arrays; missing = not present.  Arrays
    with intent(inout) are updated in place.  ``diags`` maps diagnostic names to
    preallocated float64 arrays (2-D (nj, ni), 3-D (nj, nk, ni)).  ``ties``: optional
    int32 array of the 2-D tile shape that receives, per column, 1 if the step passed
    an index computation within one rounding of its discontinuity (see
    ``oracle_set_tie_sink``).  ``trace``: optional zeroed int32 array of
    TRACE_POINT * ncol * nz + TRACE_COLUMN * ncol entries that receives every table index
    and branch decision of the step (``trace_size``, ``oracle_set_trace``).
    """
    lib = load()
    ref = fields.get("p")
    nj, nk, ni = ref.shape
    if bounds is None:
        bounds = [1, ni, 1, nj, 1, nk] * 3
    b = (ctypes.c_int * 18)(*bounds)
    d = ODiag()
    for n in DIAG2 + DIAG3:
        a = (diags or {}).get(n)
        if a is not None:
            setattr(d, n, _dp(a))
    land = fields.get("land_input")
    land_p = None
    if land is not None:
        assert land.dtype == np.int32
        land_p = land.ctypes.data_as(_IP)
    args = [fields.get(n) for n in ("t", "th", "pii", "p", "w", "dz", "qv", "qc", "qr", "qi",
                                    "qs", "qg", "ni", "nr", "nc", "nwfa", "nifa", "ng", "qb",
                                    "qc_bl", "qcfrac_bl")]
    if ties is not None:
        assert ties.dtype == np.int32 and ties.flags.c_contiguous
        lib.oracle_set_tie_sink(ties.ctypes.data_as(_IP))
    if trace is not None:
        ncol = (bounds[13] - bounds[12] + 1) * (bounds[15] - bounds[14] + 1)
        assert trace.dtype == np.int32 and trace.flags.c_contiguous
        assert trace.size == trace_size(ncol, bounds[17] - bounds[16] + 1)
        lib.oracle_set_trace(trace.ctypes.data_as(_IP))
    try:
        rc = lib.oracle_run(ctypes.byref(cfg), float(dt), int(itimestep),
                            *[_dp(a) for a in args], land_p, b, ctypes.byref(d), int(nthreads))
    finally:
        if ties is not None:
            lib.oracle_set_tie_sink(None)
        if trace is not None:
            lib.oracle_set_trace(None)
    return rc


# decision trace layout (oracle_main.c TRP / TRC, the GPU library's TraceSlot)
TRACE_POINT, TRACE_COLUMN = 16, 10


def trace_size(ncol: int, nz: int) -> int:
    return ncol * nz * TRACE_POINT + ncol * TRACE_COLUMN


def last_stats() -> list[int]:
    out = (ctypes.c_long * 8)()
    load().oracle_last_stats(out)
    return list(out)
