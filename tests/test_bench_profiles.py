"""The benchmark's roofline inputs that come from the committed ncu summaries (CPU).

bench.py scales the DRAM traffic and the FP32 operation count of a profiled
65 536-column step to its own column count; these tests read the same figures the
benchmark reads, and check that every summary under profiles/ states the command that
made it, with ncu's clocks left alone."""
import re
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO))


@pytest.fixture(scope="module")
def bench():
    import bench as b
    return b


def test_traffic_scales_with_columns(bench):
    t65 = bench.traffic_from_profiles(65536)
    assert t65 is not None and t65 > 0
    assert bench.traffic_from_profiles(1 << 20) == pytest.approx(16 * t65)
    # measured DRAM bytes exceed the algorithmic bytes (8 092 B per column-step)
    assert t65 > 8092 * 65536


def test_fp32_ops_scale_with_columns(bench):
    f65 = bench.fp32_ops_from_profiles(65536)
    assert f65 is not None and f65 > 0
    assert bench.fp32_ops_from_profiles(1 << 20) == pytest.approx(16 * f65)


@pytest.mark.parametrize("path", sorted((REPO / "profiles").glob("*.md")), ids=lambda p: p.name)
def test_summary_states_its_command(path):
    txt = re.sub(r"\\\n\s*", " ", path.read_text())  # join continued command lines
    assert "ncu " in txt, path.name
    for line in re.findall(r"^ncu .*$", txt, flags=re.M):
        assert "--clock-control none" in line, (path.name, line)
    assert "python" in txt, path.name
