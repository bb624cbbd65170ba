"""Powers with the size distributions' compile-time exponents in the mixed form (CPU).

tests/power_check.cpp runs tempo_gb300/csrc/tempo_powers.h's FP32 products, square
root and division on the host -- IEEE-rounded as on the device -- against long double
pow on seeded random arguments over the ranges the step feeds them (the slopes the size
checks allow, where no power leaves the normal FP32 range).  The error grows with the
number of roundings: up to about 5 units of 2^-24 for x^7 or x^-7, against 0.5 for a
correctly rounded FP32 pow."""
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent
CSRC = HERE.parent / "tempo_gb300" / "csrc"
BOUND = 6.0  # units of 2^-24 (three roundings of about 2 units each, at most)


def _cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return str(Path(nvcc).resolve().parent.parent / "include")


@pytest.fixture(scope="module")
def results(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    exe = tmp_path_factory.mktemp("powers") / "power_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", str(CSRC),
                    "-I", _cuda_include(), str(HERE / "power_check.cpp"), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {line.split()[0]: [float(v) for v in line.split()[1:]] for line in out.splitlines()}


def test_every_used_exponent_is_checked(results):
    assert len(results) == 15, sorted(results)


@pytest.mark.parametrize("name", ["cre0", "cre1", "cre2", "cre3", "cre5n", "cre6n", "cre7n",
                                  "cre8n", "cre9", "cre10n", "cre11", "cge0", "cge1", "cge3",
                                  "cge9"])
def test_power_within_bound(results, name):
    e, n, err = results[name]
    assert n > 0 and err <= BOUND, (name, e, err)
