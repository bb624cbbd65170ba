"""Double-float building blocks of the mixed form's island (CPU).

tests/dfloat_check.cpp runs the header's operations on the host against long double on
seeded random operands.  Bounds in units of u^2 (u = 2^-24, u^2 = 3.6e-15): the
published bounds of the division algorithms (Joldes, Muller, Popescu 2017: DWDivDW2
15 u^2 + 56 u^3, DWDivFP3 3 u^2) and of the addition of a float (DWPlusFP, 2 u^2); for
the double-word addition (SloppyDWPlusDW) a few u^2 of the operands' magnitude
|a| + |b|, also on sums of nearly equal values of opposite sign (the saturation
differences), and a few u^2 relative on same-sign sums; a few u^2 for the product; for
the saturation polynomials Horner's error scale (u^2 times the sum of the terms'
magnitudes), with the relative error above -20 degC (no cancellation there)."""
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent
CSRC = HERE.parent / "tempo_gb300" / "csrc"

BOUNDS = {"div": 15.01, "div_float": 3.0, "mul": 4.0, "add": 3.0, "add_same_sign": 3.0,
          "add_float": 2.0}
POLY_SCALED = 8.0
POLY_REL_WARM = 32.0


def _cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return str(Path(nvcc).resolve().parent.parent / "include")


@pytest.fixture(scope="module")
def results(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    exe = tmp_path_factory.mktemp("dfloat") / "dfloat_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", str(CSRC),
                    "-I", _cuda_include(), str(HERE / "dfloat_check.cpp"), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    res = {}
    for line in out.splitlines():
        name, n, *vals = line.split()
        res[name] = (int(n), [float(v) for v in vals])
    return res


@pytest.mark.parametrize("op", sorted(BOUNDS))
def test_operation_within_bound(results, op):
    n, (err,) = results[op]
    assert n > 0 and err <= BOUNDS[op], (op, err)


@pytest.mark.parametrize("poly", ["poly_liquid", "poly_ice"])
def test_saturation_polynomial(results, poly):
    n, (scaled, rel_warm) = results[poly]
    assert scaled <= POLY_SCALED, (poly, scaled)
    assert rel_warm <= POLY_REL_WARM, (poly, rel_warm)
