"""The drop-in boundary's argument lists against the reference's, on the CPU.

tests/golden/reference_signatures.json holds the reference's dummy argument lists of
tempo_init and tempo_run (src/module_mp_tempo_driver.F90:42-54, 187-198), of
tempo_aerosol_surface_emissions (:516) and the components of ty_tempo_driver_diags
(:18-34) and ty_tempo_cfgs (src/module_mp_tempo_cfgs.F90:14-35), extracted by
tests/golden/make_signatures.py.  The C header and the Fortran ISO_C_BINDING module
must keep them name for name and in order.  With TEMPO_REFERENCE pointing at a
reference checkout the fixture itself is re-extracted and compared."""
import json
import os
import re
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
HEADER = REPO / "include" / "tempo_gb300.h"
SHIM = REPO / "fortran" / "module_mp_tempo_gb300.F90"
SIG = json.loads((REPO / "tests" / "golden" / "reference_signatures.json").read_text())

sys.path.insert(0, str(REPO / "tests" / "golden"))
import make_signatures as ms  # noqa: E402


def c_params(fn: str) -> list:
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    m = re.search(r"\b" + fn + r"\s*\((.*?)\);", text, re.S)
    assert m, fn
    return [re.split(r"[\s*]+", p.strip())[-1] for p in m.group(1).split(",")]


def c_struct_fields(name: str) -> list:
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    m = re.search(r"typedef struct \{([^{}]*)\}\s*" + name + ";", text)
    assert m, name
    out = []
    for decl in m.group(1).split(";"):
        for part in decl.split(","):
            nm = re.sub(r"\[.*?\]", "", part).strip().split()[-1:] if part.strip() else []
            if nm:
                out.append(nm[0].lstrip("*"))
    return out


def test_tempo_run_c_keeps_the_reference_list():
    assert c_params("tempo_run_c") == ["ctx"] + SIG["tempo_run"]


def test_tempo_run_f32_c_keeps_the_reference_list():
    assert c_params("tempo_run_f32_c") == ["ctx"] + SIG["tempo_run"]


def test_tempo_init_c_keeps_the_reference_list():
    assert c_params("tempo_init_c")[:9] == SIG["tempo_init"]
    assert c_params("tempo_init_c")[9:] == ["table_dir", "build_tables", "device", "ctx"]


def test_device_entry_points_keep_the_state_order():
    """The device-array entry points drop only the inert inputs (qc_bl .. thten_swrad
    and ids..kde) and add the stream."""
    inert = set(SIG["tempo_run"][SIG["tempo_run"].index("qc_bl"):SIG["tempo_run"].index("land_input")])
    inert |= {"ids", "ide", "jds", "jde", "kds", "kde"}
    want = ["ctx"] + [a for a in SIG["tempo_run"] if a not in inert] + ["stream"]
    for fn in ("tempo_run_dev_c", "tempo_run_dev_f32_c", "tempo_run_dev_f32_noalloc_c"):
        assert c_params(fn) == want, fn


def test_c_structs_keep_the_reference_components():
    assert c_struct_fields("tempo_cfgs_t") == SIG["ty_tempo_cfgs"]
    assert c_struct_fields("tempo_diags_t") == SIG["ty_tempo_driver_diags"]


def test_fortran_module_keeps_the_reference_lists():
    text = SHIM.read_text()
    assert ms.subroutine_args(text, "tempo_init") == SIG["tempo_init"]
    assert ms.subroutine_args(text, "tempo_run") == SIG["tempo_run"]
    assert ms.subroutine_args(text, "tempo_aerosol_surface_emissions") == \
        SIG["tempo_aerosol_surface_emissions"]
    assert ms.type_components(text, "ty_tempo_driver_diags") == SIG["ty_tempo_driver_diags"]


def test_fortran_bind_c_types_match_the_header():
    text = SHIM.read_text()
    assert ms.type_components(text, "tempo_cfgs_c") == SIG["ty_tempo_cfgs"]
    assert ms.type_components(text, "tempo_diags_c") == SIG["ty_tempo_driver_diags"]


def test_fortran_interfaces_match_the_header():
    """Every bind(c) interface of the module names a function the header declares, with
    the header's parameter names in the header's order."""
    src = ms._join_continuations(SHIM.read_text())
    fns = re.findall(r"function\s+(\w+)\s*\(([^)]*)\)\s*bind\(c,\s*name='(\w+)'\)", src, re.I)
    assert {f[2] for f in fns} >= {"tempo_init_c", "tempo_run_c", "tempo_run_f32_c",
                                    "tempo_ctx_destroy", "tempo_last_error", "tempo_set_precision"}
    for name, args, cname in fns:
        assert name == cname
        fargs = [a.strip() for a in args.split(",") if a.strip()]
        assert fargs == (c_params(cname) if fargs else []), cname


def test_fortran_module_passes_every_optional_array():
    """tempo_run forwards each optional array of the reference through opt3/opt2i (NULL
    when absent) and each required one through c_loc, in the C ABI's order."""
    src = ms._join_continuations(SHIM.read_text())
    call = re.search(r"rc\s*=\s*tempo_run_c\((.*?)\)\s*else", src, re.S | re.I).group(1)
    items = [re.sub(r"\s+", "", x) for x in re.split(r",(?![^()]*\))", call)]
    names = []
    for it in items[4:-19]:
        m = re.fullmatch(r"(?:opt3|opt2i|c_loc)\((\w+)\)", it)
        assert m, it
        names.append(m.group(1))
    assert names == SIG["tempo_run"][3:SIG["tempo_run"].index("ids")]


@pytest.mark.skipif(not os.environ.get("TEMPO_REFERENCE"), reason="TEMPO_REFERENCE not set")
def test_fixture_matches_the_reference_checkout():
    assert ms.extract(Path(os.environ["TEMPO_REFERENCE"])) == SIG
