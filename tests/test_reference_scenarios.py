"""The reference's own integration scenarios (test/tests.F90, run by
test/run_tempo_tests.F90) on its real-data fixture, the 59-level MPAS column:
graupel sedimentation and snow sedimentation at dt = 1 ... 600 s over 1200 s, and the
aerosol-aware / non-aerosol-aware cloud-number runs at dt = 20 s.

The reference writes these scenarios' outputs to text files and asserts nothing, so
the golden arrays (tests/golden/scenarios_oracle.npz, made by make_golden.py) are the
oracle's outputs: the CPU test holds the oracle to them, the GPU test holds the CUDA
FP64 path to them through the C ABI (``tempo_run_c``), every step of every scenario.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
import make_golden as mg  # noqa: E402

# Relative tolerance with absolute floors per field (the reference's existence
# thresholds, params:135-136, in per-kg units): FP64 end to end, libm ulp differences
# accumulated over up to 1200 steps.
TOL = 1e-11
FLOORS = {"qg": 1e-12, "qb": 1e-12, "qs": 1e-12, "qc": 1e-12, "qv": 1e-12, "ng": 1e-6,
          "nc": 1e-6, "t": 1.0, "graupel_med_vol_diam": 1e-9,
          "cloud_number_mixing_ratio": 1e-6, "precip_sum": 1e-12}


def _field_of(key):
    tail = key.split("__")[-1]
    for p in ("step1_", "final_"):
        if tail.startswith(p):
            return tail[len(p):]
    return tail


def _compare(got: dict, want):
    worst = (0.0, None)
    for k, v in got.items():
        w = want[k]
        assert v.shape == w.shape, k
        e = np.abs(v - w) / np.maximum(np.abs(w), FLOORS[_field_of(k)])
        m = float(e.max()) if e.size else 0.0
        if m > worst[0]:
            worst = (m, k)
    return worst


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN / "scenarios_oracle.npz")


@pytest.fixture(scope="module")
def column():
    z = np.load(GOLDEN / "mpas_59lev_column.npz")
    return {k: z[k] for k in z.files}


def test_column_fixture_shape(column):
    assert set(column) == set(mg.COLUMN_FIELDS)
    assert all(v.shape == (59,) for v in column.values())
    assert np.array_equal(column["klev"], np.arange(1, 60))


@pytest.mark.parametrize("name", list(mg.SCENARIOS))
def test_oracle_reproduces_golden(oracle_mod, column, golden, name):
    step = mg.oracle_step_fn()
    for dt in mg.SCENARIOS[name][0]:
        got = mg.run_scenario(step, column, name, dt)
        worst, key = _compare(got, golden)
        assert worst <= TOL, (key, worst)


def _gpu_step_fn(ctx):
    import tempo_gb300 as tg
    from parity_util import make_diags

    def step(f, dt, itimestep, over):
        d = make_diags(f["p"].shape)
        ctx.run(f, dt, itimestep, diags=d, cfgs=tg.default_cfgs(**over))
        return d
    return step


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(mg.SCENARIOS))
def test_gpu_fp64_matches_golden(ctx_hail, column, golden, name):
    step = _gpu_step_fn(ctx_hail)
    for dt in mg.SCENARIOS[name][0]:
        got = mg.run_scenario(step, column, name, dt)
        worst, key = _compare(got, golden)
        assert worst <= TOL, (key, worst)
