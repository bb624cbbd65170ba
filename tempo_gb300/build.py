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


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _sources())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    for src, extra, name in UNITS:
        obj = BUILD / (name + ".o")
        jobs.append([nvcc, *NVCC_COMMON, *extra, "-c", str(CSRC / src), "-o", str(obj)])
    for src in HOST_UNITS:
        obj = BUILD / (Path(src).stem + ".o")
        jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
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
    objs = [str(BUILD / (name + ".o")) for _, _, name in UNITS] + \
           [str(BUILD / (Path(s).stem + ".o")) for s in HOST_UNITS]
    tmp = LIB.with_suffix(f".so.tmp{os.getpid()}")
    run([nvcc, *ARCH, "-shared", "-o", str(tmp), *objs, "-lcudart_static"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
