"""Table files on the host, without a GPU: tempo_check_table_c mirrors the reference's
check_before_table_read (src/module_mp_tempo_driver.F90:652-700) -- the file exists
and has the table's size -- and also decodes the contents, so that a truncated file,
a file written in the other byte order, or one with a NaN, negative or out-of-range
value is refused with TEMPO_ERR_TABLE before any device work."""
import struct
from pathlib import Path

import numpy as np
import pytest

TABLES = Path(__file__).resolve().parents[1] / "tables"
CCN_COUNT = 7 * 9 * 7 * 5 * 4
QS_COUNT = 37 * 9 * 37 * 37          # per array of qr_acr_qs (ntb_s, ntb_t, ntb_r1, ntb_r)
QS_BYTES = 12 * QS_COUNT * 8


def _code(tg, name, path):
    with pytest.raises(tg.TempoError) as e:
        tg.check_table(name, path)
    return e.value.code, str(e.value)


def test_shipped_ccn_table_passes(tg):
    tg.check_table("ccn_activate", TABLES / "ccn_activate.bin")


def test_missing_file(tg, tmp_path):
    code, msg = _code(tg, "qr_acr_qs", tmp_path / "nothere")
    assert code == -3 and "not found" in msg


def test_unknown_table_name(tg, tmp_path):
    code, _ = _code(tg, "qr_acr_xx", TABLES / "ccn_activate.bin")
    assert code == -1


def test_truncated_ccn(tg, tmp_path):
    p = tmp_path / "ccn_activate.bin"
    p.write_bytes((TABLES / "ccn_activate.bin").read_bytes()[:-100])
    code, msg = _code(tg, "ccn_activate", p)
    assert code == -3 and "size" in msg


def test_ccn_record_markers_in_the_other_byte_order(tg, tmp_path):
    b = bytearray((TABLES / "ccn_activate.bin").read_bytes())
    n = struct.unpack(">i", bytes(b[:4]))[0]
    assert n == CCN_COUNT * 4
    b[:4] = struct.pack("<i", n)
    b[-4:] = struct.pack("<i", n)
    p = tmp_path / "ccn_activate.bin"
    p.write_bytes(bytes(b))
    code, msg = _code(tg, "ccn_activate", p)
    assert code == -3 and "marker" in msg


def test_ccn_value_out_of_range(tg, tmp_path):
    b = bytearray((TABLES / "ccn_activate.bin").read_bytes())
    b[4 + 4 * 17: 4 + 4 * 18] = struct.pack(">f", 1.5)
    p = tmp_path / "ccn_activate.bin"
    p.write_bytes(bytes(b))
    code, msg = _code(tg, "ccn_activate", p)
    assert code == -3 and "out of [0, 1]" in msg


def _qs_values(seed=0):
    """Values distributed like a collection table: zeros and positive rates spanning
    many decades."""
    rng = np.random.default_rng(seed)
    v = 10.0 ** rng.uniform(-25, 5, 12 * QS_COUNT)
    v[rng.uniform(size=v.size) < 0.3] = 0.0
    return v


def test_stream_table_big_endian_passes(tg, tmp_path):
    p = tmp_path / "qr_acr_qs_data_tempo_v3"
    p.write_bytes(_qs_values().astype(">f8").tobytes())
    assert p.stat().st_size == QS_BYTES
    tg.check_table("qr_acr_qs", p)


def test_stream_table_in_the_other_byte_order(tg, tmp_path):
    p = tmp_path / "qr_acr_qs_data_tempo_v3"
    p.write_bytes(_qs_values().astype("<f8").tobytes())
    code, msg = _code(tg, "qr_acr_qs", p)
    assert code == -3 and "byte order" in msg


def test_stream_table_truncated(tg, tmp_path):
    p = tmp_path / "qr_acr_qs_data_tempo_v3"
    p.write_bytes(_qs_values().astype(">f8").tobytes()[:-8 * 1000])
    code, msg = _code(tg, "qr_acr_qs", p)
    assert code == -3 and "size" in msg


@pytest.mark.parametrize("bad", [np.nan, np.inf, -1.0e-3])
def test_stream_table_bad_value(tg, tmp_path, bad):
    v = _qs_values()
    v[5 * QS_COUNT + 1234] = bad
    p = tmp_path / "qr_acr_qs_data_tempo_v3"
    p.write_bytes(v.astype(">f8").tobytes())
    code, msg = _code(tg, "qr_acr_qs", p)
    assert code == -3 and str(5 * QS_COUNT + 1234) in msg


def test_init_refuses_a_bad_table_before_device_work(tg, tmp_path):
    """tempo_init_c checks every table file's size before it touches a device: on a
    machine without a GPU a truncated table still reads TEMPO_ERR_TABLE, not
    TEMPO_ERR_CUDA."""
    (tmp_path / "ccn_activate.bin").write_bytes((TABLES / "ccn_activate.bin").read_bytes())
    for name in ("freeze_water_data_tempo_v3", "qr_acr_qs_data_tempo_v3", "qr_acr_qg_data_tempo_v3"):
        (tmp_path / name).write_bytes(b"\0" * 64)
    with pytest.raises(tg.TempoError) as e:
        tg.TempoContext(table_dir=tmp_path, build_tables=False)
    assert e.value.code == -3 and "size" in str(e.value)
