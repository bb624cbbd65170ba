"""Helpers of the decision-trace tests: the test-only library variant that records every
table index and branch decision of a step (built with TEMPO_TRACE), and the comparison
of its records with the oracle's (same layout: TraceSlot in
tempo_gb300/csrc/tempo_types.h, TRP/TRC in oracle/oracle_main.c)."""
from __future__ import annotations

import contextlib
import ctypes

import numpy as np

TRACE_POINT, TRACE_COLUMN = 16, 10
SLOTS = {0: "check_initial", 1: "check_rates", 2: "check_condensation", 3: "check_evaporation",
         4: "check_final", 5: "warm_rain", 6: "rain_snow", 7: "rain_graupel",
         8: "rain_freezing", 9: "cloud_freezing", 10: "ice_processes", 11: "riming",
         12: "droplet_evaporation", 13: "limiter", 14: "index_range", 15: "unused15"}
COLUMN_SLOTS = ("substeps_rain", "substeps_graupel", "substeps_snow", "substeps_ice",
                "ktop_rain", "ktop_graupel", "ktop_snow", "ktop_ice", "ktop_cloud", "unused")


@contextlib.contextmanager
def trace_library(tg):
    """The trace variant as the binding's library for the duration of the block.  Only
    contexts created inside the block may be used inside it."""
    path = tg.build.build(trace=True)
    saved = tg._lib
    tg._lib = None
    try:
        lib = tg.load_library(path)
        lib.tempo_set_trace_c.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        yield lib
    finally:
        tg._lib = saved


def split(trace: np.ndarray, ncol: int, nz: int):
    """(points (ncol, nz, TRACE_POINT), columns (ncol, TRACE_COLUMN))."""
    pts = trace[: ncol * nz * TRACE_POINT].reshape(ncol, nz, TRACE_POINT)
    cols = trace[ncol * nz * TRACE_POINT:].reshape(ncol, TRACE_COLUMN)
    return pts, cols


def mismatches(a: np.ndarray, b: np.ndarray, ncol: int, nz: int, columns=None) -> dict:
    """Per slot: number of points (columns) whose records differ, over `columns`
    (bool (ncol,), default all)."""
    pa, ca = split(a, ncol, nz)
    pb, cb = split(b, ncol, nz)
    sel = np.ones(ncol, bool) if columns is None else columns
    out = {}
    for s, name in SLOTS.items():
        out[name] = int((pa[sel, :, s] != pb[sel, :, s]).sum())
    for j, name in enumerate(COLUMN_SLOTS):
        out[name] = int((ca[sel, j] != cb[sel, j]).sum())
    return out
