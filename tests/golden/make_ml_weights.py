"""Writes tests/golden/ml_cloud_number.npz: the cloud-number network of the reference
(src/module_mp_tempo_ml.F90:33-98: input scaler means and variances, two dense layers)
parsed from the reference's source file, for the tests of the ML cloud-number path.

    python tests/golden/make_ml_weights.py [path to src/module_mp_tempo_ml.F90]
"""
import re
import sys
from pathlib import Path

import numpy as np

NAMES = ("nc_ml_trans_mean", "nc_ml_trans_var", "nc_ml_w00", "nc_ml_w01", "nc_ml_b00", "nc_ml_b01")
SIZES = {"nc_ml_trans_mean": 7, "nc_ml_trans_var": 7, "nc_ml_w00": 168, "nc_ml_w01": 24,
         "nc_ml_b00": 24, "nc_ml_b01": 1}


def parse(text: str) -> dict:
    out = {}
    for name in NAMES:
        m = re.search(name + r"\s*=\s*\[(.*?)\]", text, re.S)
        assert m, name
        body = m.group(1).replace("&", " ").replace("\n", " ")
        vals = [float(v.strip().replace("_wp", "").replace("d", "e"))
                for v in body.split(",") if v.strip()]
        assert len(vals) == SIZES[name], (name, len(vals))
        out[name] = np.array(vals, dtype=np.float64)
    return out


def main():
    import os
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TEMPO_REFERENCE")
    if not root:
        raise SystemExit(f"usage: {sys.argv[0]} <TEMPO reference checkout> (or set TEMPO_REFERENCE)")
    src = Path(root) / "src" / "module_mp_tempo_ml.F90"
    data = parse(src.read_text())
    out = Path(__file__).resolve().parent / "ml_cloud_number.npz"
    np.savez(out, **data)
    print("wrote", out, {k: v.shape for k, v in data.items()})


if __name__ == "__main__":
    main()
