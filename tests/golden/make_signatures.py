"""Extracts the reference's driver interface into reference_signatures.json: the dummy
argument lists of tempo_init and tempo_run (src/module_mp_tempo_driver.F90:42-54 and
187-198), the components of ty_tempo_driver_diags (driver:18-34) and of ty_tempo_cfgs
(src/module_mp_tempo_cfgs.F90:14-35), in declaration order.

Usage: python tests/golden/make_signatures.py <TEMPO reference checkout>
(or set TEMPO_REFERENCE).  tests/test_boundary.py compares include/tempo_gb300.h and
fortran/module_mp_tempo_gb300.F90 with the committed fixture."""
from __future__ import annotations

import json
import os
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def _join_continuations(text: str) -> str:
    text = re.sub(r"!.*", "", text)                 # comments
    return re.sub(r"&\s*\n\s*&?", " ", text)         # continuation lines


def subroutine_args(text: str, name: str) -> list[str]:
    src = _join_continuations(text)
    m = re.search(r"^\s*subroutine\s+" + name + r"\s*\(([^)]*)\)", src, re.M | re.I)
    if not m:
        raise ValueError(f"subroutine {name} not found")
    return [a.strip().lower() for a in m.group(1).split(",") if a.strip()]


def type_components(text: str, name: str) -> list[str]:
    src = _join_continuations(text)
    m = re.search(r"^\s*type\s*(?:,[^:]*)?::\s*" + name + r"\s*$(.*?)^\s*(?:contains|end\s*type)",
                  src, re.M | re.I | re.S)
    if not m:
        raise ValueError(f"type {name} not found")
    out = []
    for line in m.group(1).splitlines():
        if "::" not in line:
            continue
        decl = re.sub(r"\([^)]*\)", "", line.split("::", 1)[1])   # array bounds
        for part in decl.split(","):
            nm = part.split("=")[0].strip().lower()
            if re.fullmatch(r"[a-z_]\w*", nm):
                out.append(nm)
    return out


def extract(ref: Path) -> dict:
    drv = (ref / "src" / "module_mp_tempo_driver.F90").read_text()
    cfg = (ref / "src" / "module_mp_tempo_cfgs.F90").read_text()
    return {
        "tempo_init": subroutine_args(drv, "tempo_init"),
        "tempo_run": subroutine_args(drv, "tempo_run"),
        "tempo_aerosol_surface_emissions": subroutine_args(drv, "tempo_aerosol_surface_emissions"),
        "ty_tempo_driver_diags": type_components(drv, "ty_tempo_driver_diags"),
        "ty_tempo_cfgs": type_components(cfg, "ty_tempo_cfgs"),
    }


def main(argv):
    root = argv[1] if len(argv) > 1 else os.environ.get("TEMPO_REFERENCE")
    if not root:
        raise SystemExit(f"usage: {argv[0]} <TEMPO reference checkout> (or set TEMPO_REFERENCE)")
    sig = extract(Path(root))
    (HERE / "reference_signatures.json").write_text(json.dumps(sig, indent=1) + "\n")
    print({k: len(v) for k, v in sig.items()})


if __name__ == "__main__":
    main(sys.argv)
