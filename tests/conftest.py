"""Shared fixtures.  `gpu`-marked tests need a GB300 and the built CUDA library;
everything else runs on the CPU (the oracle is test infrastructure)."""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))

TABLES = REPO / "tables"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the CUDA library")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def oracle_tables(oracle_mod, tmp_path_factory):
    """Oracle initialised hail-aware with its own table build, and the three tables
    written in the reference's big-endian file format (plus the CCN file)."""
    o = oracle_mod
    o.init(True, TABLES / "ccn_activate.bin")
    o.build_big_tables()
    d = tmp_path_factory.mktemp("tables")
    lib = o.load()
    assert lib.oracle_write_freezewater(str(d / "freeze_water_data_tempo_v3").encode()) == 0
    assert lib.oracle_write_qr_acr_qs(str(d / "qr_acr_qs_data_tempo_v3").encode()) == 0
    assert lib.oracle_write_qr_acr_qg(str(d / "qr_acr_qg_data_tempo_v3").encode()) == 0
    (d / "ccn_activate.bin").write_bytes((TABLES / "ccn_activate.bin").read_bytes())
    return d


@pytest.fixture(scope="session")
def tg():
    """The CUDA library's Python binding (built in-tree if stale)."""
    import tempo_gb300
    tempo_gb300.build.build()
    return tempo_gb300


@pytest.fixture(scope="session")
def ctx_hail(tg, oracle_tables):
    """Hail-aware context on the oracle's tables (read from the reference file format)."""
    return tg.TempoContext(table_dir=oracle_tables, build_tables=False,
                           cfgs=tg.default_cfgs(hailaware_flag=1))


@pytest.fixture(scope="session")
def ctx_nohail(tg, oracle_tables):
    return tg.TempoContext(table_dir=oracle_tables, build_tables=False,
                           cfgs=tg.default_cfgs(hailaware_flag=0))
