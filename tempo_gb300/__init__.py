"""tempo_gb300 -- GB300 (sm_103a) TEMPO column-microphysics step.

Python mirror of the reference's driver interface (src/module_mp_tempo_driver.F90):
:func:`tempo_init` and :func:`tempo_run` keep the Fortran argument names and meaning
and call the C ABI of ``libtempo_gb300.so`` (``include/tempo_gb300.h``) through
ctypes.  Arrays are ``(jms:jme, kms:kme, ims:ime)``-shaped NumPy arrays in C order,
i.e. the Fortran ``(i, k, j)`` memory layout with i fastest.

:class:`TempoContext` is the object-level API; :func:`run_device` runs the step on
torch CUDA tensors that already live in HBM.  The library must be built
(:func:`tempo_gb300.build.build`); there is no CPU fallback -- every call fails loudly
if the CUDA library is missing.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path
from typing import Optional

import numpy as np

from . import build as _build

__all__ = ["TempoError", "TempoContext", "tempo_init", "tempo_run", "default_cfgs", "DIFF_FIELDS",
           "check_table", "EXTRA_FIELDS",
           "PREC_FP64", "PREC_MIXED", "DIAG2", "DIAG3", "load_library", "REPO_TABLES"]

PKG = Path(__file__).resolve().parent
REPO_TABLES = PKG.parent / "tables"
PREC_FP64, PREC_MIXED = 0, 1

DIAG2 = ("rain_precip", "ice_liquid_equiv_precip", "snow_liquid_equiv_precip",
         "graupel_liquid_equiv_precip", "frozen_fraction", "frz_rain_precip",
         "max_hail_diameter_sfc", "max_hail_diameter_column")
DIAG3 = ("refl10cm", "re_cloud", "re_ice", "re_snow", "rain_med_vol_diam",
         "graupel_med_vol_diam", "cloud_number_mixing_ratio")
FIELDS = ("t", "th", "pii", "p", "w", "dz", "qv", "qc", "qr", "qi", "qs", "qg", "ni", "nr",
          "nc", "nwfa", "nifa", "ng", "qb")
# the optional inputs of tempo_run between qb and land_input (driver:191-195)
EXTRA_FIELDS = ("qc_bl", "qcfrac_bl", "qcfrac", "qifrac", "thten_bl", "qvten_bl", "qcten_bl",
                "qiten_bl", "thten_lwrad", "thten_swrad")
CFG_FLAGS = ("aerosolaware_flag", "hailaware_flag", "ml_for_bl_nc_flag", "ml_for_nc_flag",
             "semi_sedi_flag", "refl10cm_from_melting_flag", "turn_off_micro_flag",
             "cloud_condensation_flag", "verbose", "check_tables")
DIAG_FLAGS = ("refl10cm_flag", "re_cloud_flag", "re_ice_flag", "re_snow_flag",
              "max_hail_diameter_flag", "rain_med_vol_diam_flag", "graupel_med_vol_diam_flag",
              "cloud_number_mixing_ratio_flag")
STATUS = {0: "TEMPO_OK", -1: "TEMPO_ERR_ARG", -2: "TEMPO_ERR_UNSUPPORTED",
          -3: "TEMPO_ERR_TABLE", -4: "TEMPO_ERR_CUDA", -5: "TEMPO_ERR_NOMEM",
          -6: "TEMPO_ERR_STATE", -8: "TEMPO_ERR_NONFINITE"}


class TempoError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class TempoCfgs(ctypes.Structure):
    """tempo_cfgs_t = ty_tempo_cfgs (src/module_mp_tempo_cfgs.F90:14-35)."""
    _fields_ = [(n, ctypes.c_int) for n in CFG_FLAGS] + \
               [("single_moment_nc_opt", ctypes.c_char * 32)] + \
               [(n, ctypes.c_int) for n in DIAG_FLAGS]

    def as_dict(self):
        d = {n: bool(getattr(self, n)) for n in CFG_FLAGS + DIAG_FLAGS}
        d["single_moment_nc_opt"] = self.single_moment_nc_opt.decode()
        return d


class TempoState(ctypes.Structure):
    """tempo_state_t: device pointers to one state (include/tempo_gb300.h)."""
    _fields_ = [(n, ctypes.c_void_p) for n in (
        "t", "th", "pii", "p", "w", "dz", "qv", "qc", "qr", "qi", "qs", "qg", "ni", "nr", "nc",
        "nwfa", "nifa", "ng", "qb", "land_input")]


# inputs of the step that the tangent-linear and adjoint steps differentiate
DIFF_FIELDS = ("t", "th", "qv", "qc", "nc", "qr", "nr", "qi", "ni", "qs", "qg", "ng", "qb")


def _state_of(fields: dict) -> TempoState:
    st = TempoState()
    for n, _ in TempoState._fields_:
        v = fields.get(n)
        if v is not None:
            setattr(st, n, v.data_ptr())
    return st


class TempoDiags(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in DIAG2 + DIAG3]


class TempoDomain(ctypes.Structure):
    """tempo_domain_t: one domain of a multi-domain batch (include/tempo_gb300.h)."""
    _fields_ = [("dt", ctypes.c_float), ("itimestep", ctypes.c_int), ("state", TempoState),
                ("diags", TempoDiags)] + [(n, ctypes.c_int) for n in (
                    "ims", "ime", "jms", "jme", "kms", "kme", "its", "ite", "jts", "jte", "kts", "kte")]


_lib = None
_DP = ctypes.POINTER(ctypes.c_double)
_FP = ctypes.POINTER(ctypes.c_float)
_IP = ctypes.POINTER(ctypes.c_int)
_VP = ctypes.c_void_p


def load_library(path: Optional[os.PathLike] = None) -> ctypes.CDLL:
    """Loads libtempo_gb300.so (built in-tree); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    lib_path = Path(path) if path else _build.LIB
    if not lib_path.exists():
        raise TempoError(-6, f"{lib_path} not built; run tempo_gb300.build.build() "
                             "(there is no CPU fallback)")
    lib = ctypes.CDLL(str(lib_path))
    i = ctypes.c_int
    lib.tempo_version.restype = ctypes.c_char_p
    lib.tempo_last_error.restype = ctypes.c_char_p
    lib.tempo_default_cfgs.argtypes = [ctypes.POINTER(TempoCfgs)]
    lib.tempo_init_c.argtypes = [_IP] * 8 + [ctypes.POINTER(TempoCfgs), ctypes.c_char_p, i, i,
                                             ctypes.POINTER(ctypes.c_void_p)]
    lib.tempo_ctx_destroy.argtypes = [_VP]
    lib.tempo_set_precision.argtypes = [_VP, i]
    lib.tempo_run_c.argtypes = ([_VP, ctypes.POINTER(TempoCfgs), ctypes.c_double, i]
                                + [_DP] * 19 + [_DP] * 10 + [_IP] + [i] * 18
                                + [ctypes.POINTER(TempoDiags)])
    lib.tempo_run_f32_c.argtypes = ([_VP, ctypes.POINTER(TempoCfgs), ctypes.c_float, i]
                                    + [_FP] * 19 + [_FP] * 10 + [_IP] + [i] * 18
                                    + [ctypes.POINTER(TempoDiags)])
    lib.tempo_run_dev_c.argtypes = ([_VP, ctypes.POINTER(TempoCfgs), ctypes.c_double, i]
                                    + [_VP] * 19 + [_VP] + [i] * 12
                                    + [ctypes.POINTER(TempoDiags), _VP])
    lib.tempo_run_dev_f32_c.argtypes = ([_VP, ctypes.POINTER(TempoCfgs), ctypes.c_float, i]
                                        + [_VP] * 19 + [_VP] + [i] * 12
                                        + [ctypes.POINTER(TempoDiags), _VP])
    lib.tempo_run_dev_f32_noalloc_c.argtypes = lib.tempo_run_dev_f32_c.argtypes
    lib.tempo_aerosol_surface_emissions_dev_c.argtypes = [_VP, ctypes.c_double, _VP, _VP] + [i] * 7 + [_VP]
    lib.tempo_write_table_c.argtypes = [_VP, ctypes.c_char_p, ctypes.c_char_p]
    lib.tempo_get_table_c.argtypes = [_VP, ctypes.c_char_p, _DP, ctypes.c_long,
                                      ctypes.POINTER(ctypes.c_long)]
    lib.tempo_build_tables_c.argtypes = [_VP, ctypes.POINTER(ctypes.c_float)]
    lib.tempo_last_stats_c.argtypes = [_VP, ctypes.POINTER(ctypes.c_long)]
    lib.tempo_set_kernel_timing.argtypes = [_VP, i]
    lib.tempo_autotune_dev_f32_c.argtypes = ([_VP, ctypes.POINTER(TempoCfgs), ctypes.c_float, i]
                                             + [_VP] * 19 + [_VP] + [i] * 12
                                             + [ctypes.POINTER(TempoDiags), _VP, i,
                                                ctypes.POINTER(ctypes.c_float), i,
                                                ctypes.POINTER(ctypes.c_int)])
    lib.tempo_set_points_variant.argtypes = [_VP, i]
    lib.tempo_set_points_order.argtypes = [_VP, i]
    lib.tempo_set_sedim_variant.argtypes = [_VP, i]
    lib.tempo_tuning_c.argtypes = [_VP, ctypes.POINTER(ctypes.c_int)]
    lib.tempo_set_host_slabs.argtypes = [_VP, i]
    lib.tempo_set_graphs.argtypes = [_VP, i]
    lib.tempo_tl_dev_c.argtypes = ([_VP, ctypes.POINTER(TempoCfgs), ctypes.c_double, i, i,
                                    ctypes.POINTER(TempoState), ctypes.POINTER(TempoState),
                                    ctypes.POINTER(TempoDiags), ctypes.POINTER(TempoDiags)]
                                   + [i] * 12 + [_VP])
    lib.tempo_adjoint_dev_c.argtypes = ([_VP, ctypes.POINTER(TempoCfgs), ctypes.c_double, i, i,
                                         ctypes.POINTER(TempoState), ctypes.POINTER(TempoState),
                                         ctypes.POINTER(TempoDiags)] + [i] * 12 + [_VP])
    lib.tempo_kernel_times_c.argtypes = [_VP, ctypes.POINTER(ctypes.c_float)]
    lib.tempo_check_table_c.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    lib.tempo_run_batch_dev_f32_c.argtypes = [_VP, ctypes.POINTER(TempoCfgs), i,
                                              ctypes.POINTER(TempoDomain), _VP]
    lib.tempo_set_validation.argtypes = [_VP, i]
    _lib = lib
    return lib


def _check(rc: int):
    if rc != 0:
        raise TempoError(rc, load_library().tempo_last_error().decode())


def check_table(name: str, path: os.PathLike) -> None:
    """tempo_check_table_c: validates one table file on the host (no GPU); raises
    TempoError (TEMPO_ERR_TABLE) with the reason for a missing, truncated, byte-swapped
    or otherwise malformed file."""
    _check(load_library().tempo_check_table_c(name.encode(), str(path).encode()))


def default_cfgs(**over) -> TempoCfgs:
    cfg = TempoCfgs()
    _check(load_library().tempo_default_cfgs(ctypes.byref(cfg)))
    for k, v in over.items():
        if k == "single_moment_nc_opt":
            cfg.single_moment_nc_opt = str(v).encode()
        else:
            setattr(cfg, k, int(bool(v)))
    return cfg


def _int_ptr(v):
    return None if v is None else ctypes.pointer(ctypes.c_int(int(bool(v))))


def _np_ptr(a, ctype):
    if a is None:
        return None
    if not (a.flags.c_contiguous and a.dtype == np.dtype(ctype)):
        raise TempoError(-1, f"array must be C-contiguous {np.dtype(ctype)}")
    return a.ctypes.data_as(ctypes.POINTER(ctype))


class TempoContext:
    """A tempo_init context: device tables plus reusable buffers on one GPU."""

    def __init__(self, table_dir: Optional[os.PathLike] = None, build_tables: Optional[bool] = None,
                 device: int = 0, cfgs: Optional[TempoCfgs] = None, **flags):
        lib = load_library()
        self.cfgs = cfgs if cfgs is not None else default_cfgs()
        table_dir = Path(table_dir) if table_dir else REPO_TABLES
        if build_tables is None:
            build_tables = not (table_dir / "qr_acr_qg_data_tempo_v3").exists()
        names = ("aerosolaware_flag", "hailaware_flag", "semi_sedi_flag",
                 "cloud_condensation_flag", "refl10cm_from_melting_flag", "ml_for_bl_nc_flag",
                 "ml_for_nc_flag", "force_init_flag")
        ptrs = [_int_ptr(flags.get(n)) for n in names]
        handle = ctypes.c_void_p()
        _check(lib.tempo_init_c(*ptrs, ctypes.byref(self.cfgs), str(table_dir).encode(),
                                int(bool(build_tables)), int(device), ctypes.byref(handle)))
        self._h = handle
        self.device = device

    def close(self):
        if getattr(self, "_h", None):
            load_library().tempo_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_precision(self, mode: int):
        _check(load_library().tempo_set_precision(self._h, int(mode)))

    def set_validation(self, on: bool = True):
        """tempo_set_validation: scan the inputs of later runs for non-finite values."""
        _check(load_library().tempo_set_validation(self._h, int(bool(on))))

    # ---- host arrays -----------------------------------------------------------------
    def run(self, fields: dict, dt: float, itimestep: int, diags: Optional[dict] = None,
            bounds=None, cfgs: Optional[TempoCfgs] = None):
        """tempo_run on host NumPy arrays (float64 -> FP64 ABI, float32 -> *_f32 ABI)."""
        lib = load_library()
        cfg = cfgs if cfgs is not None else self.cfgs
        p = fields["p"]
        nj, nk, ni = p.shape
        b = list(bounds) if bounds is not None else [1, ni, 1, nj, 1, nk] * 3
        d = TempoDiags()
        for n in DIAG2 + DIAG3:
            a = (diags or {}).get(n)
            if a is not None:
                setattr(d, n, a.ctypes.data)
        land = fields.get("land_input")
        land_p = _np_ptr(land, ctypes.c_int) if land is not None else None
        ct = ctypes.c_double if p.dtype == np.float64 else ctypes.c_float
        ptrs = [_np_ptr(fields.get(n), ct) for n in FIELDS]
        extra = [_np_ptr(fields.get(n), ct) for n in EXTRA_FIELDS]
        fn = lib.tempo_run_c if p.dtype == np.float64 else lib.tempo_run_f32_c
        _check(fn(self._h, ctypes.byref(cfg), float(dt), int(itimestep), *ptrs, *extra, land_p,
                  *b, ctypes.byref(d)))

    # ---- device tensors --------------------------------------------------------------
    def run_device(self, fields: dict, dt: float, itimestep: int, diags: Optional[dict] = None,
                   bounds=None, stream=None, cfgs: Optional[TempoCfgs] = None):
        """tempo_run on torch CUDA tensors already in HBM (float64 or float32);
        enqueued on ``stream`` (a torch.cuda.Stream, default: the current stream)."""
        import torch
        lib = load_library()
        cfg = cfgs if cfgs is not None else self.cfgs
        p = fields["p"]
        nj, nk, ni = p.shape
        b = list(bounds) if bounds is not None else [1, ni, 1, nj, 1, nk] * 3
        ims, ime, jms, jme, kms, kme, its, ite, jts, jte, kts, kte = b[6:]
        for n, tns in fields.items():
            if tns is not None and not (tns.is_cuda and tns.is_contiguous()):
                raise TempoError(-1, f"{n} must be a contiguous CUDA tensor")
        ptrs = [(fields[n].data_ptr() if fields.get(n) is not None else None) for n in FIELDS]
        land = fields.get("land_input")
        d = TempoDiags()
        for n in DIAG2 + DIAG3:
            a = (diags or {}).get(n)
            if a is not None:
                setattr(d, n, a.data_ptr())
        s = stream if stream is not None else torch.cuda.current_stream(p.device)
        sptr = ctypes.c_void_p(s.cuda_stream)
        fn = lib.tempo_run_dev_c if p.dtype == torch.float64 else lib.tempo_run_dev_f32_c
        _check(fn(self._h, ctypes.byref(cfg), float(dt), int(itimestep), *ptrs,
                  land.data_ptr() if land is not None else None,
                  ims, ime, jms, jme, kms, kme, its, ite, jts, jte, kts, kte, ctypes.byref(d), sptr))

    def run_device_noalloc(self, fields: dict, dt: float, itimestep: int,
                           diags: Optional[dict] = None, bounds=None, stream=None,
                           cfgs: Optional[TempoCfgs] = None):
        """tempo_run_dev_f32_noalloc_c on float32 CUDA tensors (TEMPO_PREC_MIXED): the
        step with its scratch in the library's fixed device array, allocating nothing.
        Calls on one device must not overlap; tiles beyond the fixed scratch raise."""
        import torch
        lib = load_library()
        cfg = cfgs if cfgs is not None else self.cfgs
        p = fields["p"]
        if p.dtype != torch.float32:
            raise TempoError(-1, "the no-allocation step works on float32 device arrays")
        nj, nk, ni = p.shape
        b = list(bounds) if bounds is not None else [1, ni, 1, nj, 1, nk] * 3
        for n, tns in fields.items():
            if tns is not None and not (tns.is_cuda and tns.is_contiguous()):
                raise TempoError(-1, f"{n} must be a contiguous CUDA tensor")
        ptrs = [(fields[n].data_ptr() if fields.get(n) is not None else None) for n in FIELDS]
        land = fields.get("land_input")
        d = TempoDiags()
        for n in DIAG2 + DIAG3:
            a = (diags or {}).get(n)
            if a is not None:
                setattr(d, n, a.data_ptr())
        s = stream if stream is not None else torch.cuda.current_stream(p.device)
        _check(lib.tempo_run_dev_f32_noalloc_c(
            self._h, ctypes.byref(cfg), float(dt), int(itimestep), *ptrs,
            land.data_ptr() if land is not None else None, *b[6:], ctypes.byref(d),
            ctypes.c_void_p(s.cuda_stream)))

    def run_batch_device(self, domains: list, stream=None, cfgs: Optional[TempoCfgs] = None):
        """tempo_run_batch_dev_f32_c: the mixed step of several domains (float32 CUDA
        tensors) as one launch sequence.  ``domains``: dicts with ``fields`` (as for
        run_device), ``dt``, ``itimestep`` and optional ``diags``."""
        import torch
        lib = load_library()
        cfg = cfgs if cfgs is not None else self.cfgs
        arr = (TempoDomain * len(domains))()
        for d, dom in zip(arr, domains):
            f = dom["fields"]
            if f["p"].dtype != torch.float32:
                raise TempoError(-1, "the batch step works on float32 device arrays")
            nj, nk, ni = f["p"].shape
            d.dt = float(dom["dt"])
            d.itimestep = int(dom["itimestep"])
            d.state = _state_of(f)
            for n in DIAG2 + DIAG3:
                a = (dom.get("diags") or {}).get(n)
                if a is not None:
                    setattr(d.diags, n, a.data_ptr())
            for n, v in zip(("ims", "ime", "jms", "jme", "kms", "kme", "its", "ite", "jts", "jte",
                             "kts", "kte"), [1, ni, 1, nj, 1, nk] * 2):
                setattr(d, n, v)
        dev = domains[0]["fields"]["p"].device
        s = stream if stream is not None else torch.cuda.current_stream(dev)
        _check(lib.tempo_run_batch_dev_f32_c(self._h, ctypes.byref(cfg), len(domains), arr,
                                             ctypes.c_void_p(s.cuda_stream)))

    def autotune_device(self, fields: dict, dt: float, itimestep: int, diags: Optional[dict] = None,
                        bounds=None, stream=None, cfgs: Optional[TempoCfgs] = None,
                        reps: int = 2):
        """Picks the fastest per-level kernel variant, point order and sedimentation
        variant of the mixed form for this workload (tempo_autotune_dev_f32_c) on
        private copies of the float32 CUDA tensors; returns (chosen per-level
        candidate, per-candidate time in ms): candidates 0-15 are variant v % 8 in
        order v // 8, candidates 16-21 the sedimentation variants."""
        import torch
        lib = load_library()
        cfg = cfgs if cfgs is not None else self.cfgs
        p = fields["p"]
        if p.dtype != torch.float32:
            raise TempoError(-1, "autotune works on float32 device arrays")
        nj, nk, ni = p.shape
        b = list(bounds) if bounds is not None else [1, ni, 1, nj, 1, nk] * 3
        ptrs = [(fields[n].data_ptr() if fields.get(n) is not None else None) for n in FIELDS]
        land = fields.get("land_input")
        d = TempoDiags()
        for n in DIAG2 + DIAG3:
            a = (diags or {}).get(n)
            if a is not None:
                setattr(d, n, a.data_ptr())
        s = stream if stream is not None else torch.cuda.current_stream(p.device)
        times = (ctypes.c_float * 28)()
        chosen = ctypes.c_int(-1)
        _check(lib.tempo_autotune_dev_f32_c(
            self._h, ctypes.byref(cfg), float(dt), int(itimestep), *ptrs,
            land.data_ptr() if land is not None else None, *b[6:], ctypes.byref(d),
            ctypes.c_void_p(s.cuda_stream), int(reps), times, 28, ctypes.byref(chosen)))
        return chosen.value, [float(x) for x in times]

    # ---- derivatives ----------------------------------------------------------------
    def _dev_common(self, fields, bounds, stream):
        import torch
        p = fields["p"]
        nj, nk, ni = p.shape
        b = list(bounds) if bounds is not None else [1, ni, 1, nj, 1, nk] * 3
        s = stream if stream is not None else torch.cuda.current_stream(p.device)
        return b[6:], ctypes.c_void_p(s.cuda_stream), int(p.dtype == torch.float64)

    def tl_device(self, fields: dict, dfields: dict, dt: float, itimestep: int,
                  diags: Optional[dict] = None, tdiags: Optional[dict] = None, bounds=None,
                  stream=None, cfgs: Optional[TempoCfgs] = None):
        """Tangent-linear step (tempo_tl_dev_c) on CUDA tensors: ``fields`` advance one
        step, ``dfields`` (tangents of DIFF_FIELDS) become the output tangents and
        ``tdiags`` the tangents of the diagnostics.  float64 tensors: FP64 step;
        float32: all-FP32 step."""
        cfg = cfgs if cfgs is not None else self.cfgs
        bb, sptr, fp64 = self._dev_common(fields, bounds, stream)
        x, dx = _state_of(fields), _state_of({k: v for k, v in dfields.items() if k in DIFF_FIELDS})
        d, td = TempoDiags(), TempoDiags()
        for n in DIAG2 + DIAG3:
            if diags and diags.get(n) is not None:
                setattr(d, n, diags[n].data_ptr())
            if tdiags and tdiags.get(n) is not None:
                setattr(td, n, tdiags[n].data_ptr())
        _check(load_library().tempo_tl_dev_c(self._h, ctypes.byref(cfg), float(dt), int(itimestep),
                                              fp64, ctypes.byref(x), ctypes.byref(dx), ctypes.byref(d),
                                              ctypes.byref(td), *bb, sptr))

    def adjoint_device(self, fields: dict, lam: dict, dt: float, itimestep: int,
                       lam_diags: Optional[dict] = None, bounds=None, stream=None,
                       cfgs: Optional[TempoCfgs] = None):
        """Adjoint step (tempo_adjoint_dev_c): ``fields`` is the state before the step
        (unchanged); ``lam`` holds adjoints of the step's outputs on entry and of its
        inputs on return; ``lam_diags`` the adjoints of the precipitation and refl10cm."""
        cfg = cfgs if cfgs is not None else self.cfgs
        bb, sptr, fp64 = self._dev_common(fields, bounds, stream)
        x, lm = _state_of(fields), _state_of({k: v for k, v in lam.items() if k in DIFF_FIELDS})
        ld = TempoDiags()
        for n in DIAG2 + DIAG3:
            if lam_diags and lam_diags.get(n) is not None:
                setattr(ld, n, lam_diags[n].data_ptr())
        _check(load_library().tempo_adjoint_dev_c(self._h, ctypes.byref(cfg), float(dt), int(itimestep),
                                                   fp64, ctypes.byref(x), ctypes.byref(lm),
                                                   ctypes.byref(ld), *bb, sptr))

    def set_graphs(self, on: bool = True):
        """Capture each distinct step into a CUDA graph and replay it (tempo_set_graphs)."""
        _check(load_library().tempo_set_graphs(self._h, int(bool(on))))

    def set_ml_cloud_number(self, weights: dict):
        """The cloud-number network of the ML path (tempo_set_ml_cloud_number_c); keys
        nc_ml_trans_mean, nc_ml_trans_var, nc_ml_w00, nc_ml_b00, nc_ml_w01, nc_ml_b01
        (the reference's names, src/module_mp_tempo_ml.F90:33-98)."""
        arrs = [np.ascontiguousarray(np.asarray(weights[k], dtype=np.float64))
                for k in ("nc_ml_trans_mean", "nc_ml_trans_var", "nc_ml_w00", "nc_ml_b00",
                          "nc_ml_w01", "nc_ml_b01")]
        _check(load_library().tempo_set_ml_cloud_number_c(self._h, *[_np_ptr(a, ctypes.c_double) for a in arrs]))

    def set_points_variant(self, v: int):
        _check(load_library().tempo_set_points_variant(self._h, int(v)))

    def set_points_order(self, order: int):
        """0: phase A's points level-major (default); 1: grouped by regime."""
        _check(load_library().tempo_set_points_order(self._h, int(order)))

    def set_sedim_variant(self, v: int):
        """Sedimentation kernel variant 0..11: v % 3 + 1 levels loaded together per
        substep sweep; (v // 3) % 2 splits a column's species over two threads; v < 6
        runs a species' substeps level by level where they fit, v >= 6 substep by
        substep."""
        _check(load_library().tempo_set_sedim_variant(self._h, int(v)))

    def set_host_slabs(self, n: int):
        """Row slabs of later host-array runs (0: from the tile's size)."""
        _check(load_library().tempo_set_host_slabs(self._h, int(n)))

    def tuning(self) -> dict:
        """The context's kernel choices (tempo_tuning_c)."""
        out = (ctypes.c_int * 3)()
        _check(load_library().tempo_tuning_c(self._h, out))
        return dict(points_variant=out[0], points_order=out[1], sedim_variant=out[2])

    def aerosol_surface_emissions(self, dt: float, nwfa, nwfa2d, kts: int = 1, stream=None):
        """tempo_aerosol_surface_emissions (driver:516-529) on CUDA tensors."""
        import torch
        nj, nk, ni = nwfa.shape
        s = stream if stream is not None else torch.cuda.current_stream(nwfa.device)
        _check(load_library().tempo_aerosol_surface_emissions_dev_c(
            self._h, float(dt), nwfa.data_ptr(), nwfa2d.data_ptr(), 1, ni, 1, nj, 1, nk, kts,
            ctypes.c_void_p(s.cuda_stream)))

    # ---- tables ------------------------------------------------------------------------
    def get_table(self, name: str) -> np.ndarray:
        lib = load_library()
        n = ctypes.c_long()
        _check(lib.tempo_get_table_c(self._h, name.encode(), None, 0, ctypes.byref(n)))
        out = np.empty(n.value, dtype=np.float64)
        _check(lib.tempo_get_table_c(self._h, name.encode(), _np_ptr(out, ctypes.c_double),
                                     n.value, None))
        return out

    def write_table(self, family: str, path: os.PathLike):
        _check(load_library().tempo_write_table_c(self._h, family.encode(), str(path).encode()))

    def build_tables(self) -> float:
        ms = ctypes.c_float()
        _check(load_library().tempo_build_tables_c(self._h, ctypes.byref(ms)))
        return ms.value

    KERNELS = ("prep", "order", "points", "sedim", "final")

    def set_kernel_timing(self, on: bool = True):
        """Record CUDA events around the kernels of each later run."""
        _check(load_library().tempo_set_kernel_timing(self._h, int(bool(on))))

    def kernel_times(self) -> dict:
        """Durations (ms) of the kernels of the last run (the regime-order pair as one
        entry); waits for it."""
        ms = (ctypes.c_float * 5)()
        _check(load_library().tempo_kernel_times_c(self._h, ms))
        return dict(zip(self.KERNELS, (float(x) for x in ms)))

    def stats(self) -> dict:
        out = (ctypes.c_long * 8)()
        _check(load_library().tempo_last_stats_c(self._h, out))
        return dict(columns=out[0], early_exit=out[1], substeps_rain=out[2],
                    substeps_graupel=out[3], substeps_snow=out[4], substeps_ice=out[5],
                    substeps_cloud=out[6], launches=out[7])


def tempo_init(aerosolaware_flag=None, hailaware_flag=None, semi_sedi_flag=None,
               cloud_condensation_flag=None, refl10cm_from_melting_flag=None,
               ml_for_bl_nc_flag=None, ml_for_nc_flag=None, force_init_flag=None,
               tempo_cfgs: Optional[TempoCfgs] = None, table_dir=None, build_tables=None,
               device: int = 0):
    """tempo_init (driver:42-182): returns (tempo_cfgs, context)."""
    cfgs = tempo_cfgs if tempo_cfgs is not None else default_cfgs()
    ctx = TempoContext(table_dir=table_dir, build_tables=build_tables, device=device, cfgs=cfgs,
                       aerosolaware_flag=aerosolaware_flag, hailaware_flag=hailaware_flag,
                       semi_sedi_flag=semi_sedi_flag,
                       cloud_condensation_flag=cloud_condensation_flag,
                       refl10cm_from_melting_flag=refl10cm_from_melting_flag,
                       ml_for_bl_nc_flag=ml_for_bl_nc_flag, ml_for_nc_flag=ml_for_nc_flag,
                       force_init_flag=force_init_flag)
    return ctx.cfgs, ctx


def tempo_run(ctx: TempoContext, tempo_cfgs: TempoCfgs, dt: float, itimestep: int,
              tempo_diags: Optional[dict] = None, bounds=None, **arrays):
    """tempo_run (driver:187-513) on host NumPy arrays named as in the reference
    (t, th, pii, p, w, dz, qv, qc, qr, qi, qs, qg, ni, nr, nc, nwfa, nifa, ng, qb,
    land_input, ...).  Updates the arrays in place and fills ``tempo_diags``."""
    ctx.run(arrays, dt, itimestep, diags=tempo_diags, bounds=bounds, cfgs=tempo_cfgs)
