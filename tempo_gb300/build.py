"""Builds libtempo_gb300.so in-tree for sm_103a (nvcc + g++, no cmake).

Translation units compile in parallel; the FP64 step and the table builders are
compiled without FMA contraction (-fmad=false) so their arithmetic matches the
reference's unfused FP64 order.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libtempo_gb300.so"
# test-only variant that records every table index and branch decision of a step
# (TEMPO_TRACE; tests/test_decision_trace.py); never loaded by the product
TRACE_BUILD = PKG / "_build_trace"
TRACE_LIB = PKG / "libtempo_gb300_trace.so"
INCLUDE = REPO / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I", str(INCLUDE),
               "-I", str(CSRC), *ARCH]
# (source, extra flags, object name)
UNITS = [
    ("tempo_step_f64.cu", ["-fmad=false"], "tempo_step_f64"),
    ("tempo_step_f32.cu", [], "tempo_step_f32"),
    ("tempo_points_f32.cu", ["-DTEMPO_VARIANT_SET=0"], "tempo_points_f32_lo"),
    ("tempo_points_f32.cu", ["-DTEMPO_VARIANT_SET=1"], "tempo_points_f32_hi"),
    ("tempo_tables.cu", ["-fmad=false"], "tempo_tables"),
    ("tempo_deriv_f64.cu", ["-fmad=false"], "tempo_deriv_f64"),
    ("tempo_deriv_f32.cu", [], "tempo_deriv_f32"),
    ("tempo_noalloc.cu", [], "tempo_noalloc"),
    ("tempo_melt.cu", ["-fmad=false"], "tempo_melt"),
    ("tempo_validate.cu", [], "tempo_validate"),
    ("tempo_batch.cu", [], "tempo_batch"),
]
HOST_UNITS = ["tempo_capi.cpp", "tempo_host_init.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_include() -> str:
    nv = Path(_nvcc()).resolve()
    return str(nv.parent.parent / "include")


def _sources():
    return sorted(CSRC.glob("*")) + sorted(INCLUDE.glob("*.h")) + [Path(__file__)]


def up_to_date(lib: Path = LIB) -> bool:
    if not lib.exists():
        return False
    t = lib.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _sources())


def build(force: bool = False, verbose: bool = False, trace: bool = False) -> Path:
    """Compiles the library (trace=True: the test-only decision-trace variant)."""
    lib, bdir = (TRACE_LIB, TRACE_BUILD) if trace else (LIB, BUILD)
    if not force and up_to_date(lib):
        return lib
    bdir.mkdir(exist_ok=True)
    nvcc = _nvcc()
    defs = ["-DTEMPO_TRACE"] if trace else []
    jobs = []
    for src, extra, name in UNITS:
        obj = bdir / (name + ".o")
        jobs.append([nvcc, *NVCC_COMMON, *defs, *extra, "-c", str(CSRC / src), "-o", str(obj)])
    for src in HOST_UNITS:
        obj = bdir / (Path(src).stem + ".o")
        jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", *defs,
                     "-I", str(INCLUDE), "-I", str(CSRC), "-I", _cuda_include(),
                     "-c", str(CSRC / src), "-o", str(obj)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(run, jobs))
    objs = [str(bdir / (name + ".o")) for _, _, name in UNITS] + \
           [str(bdir / (Path(s).stem + ".o")) for s in HOST_UNITS]
    tmp = lib.with_suffix(f".so.tmp{os.getpid()}")
    run([nvcc, *ARCH, "-shared", "-o", str(tmp), *objs, "-lcudart_static"])
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
