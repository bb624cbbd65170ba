"""Regenerates the golden fixtures of this directory.

    python tests/golden/make_golden.py [path/to/reference/checkout]

1. ``mpas_59lev_column.npz``: the reference's only real-data fixture,
   test/data/mpas_59lev_test.txt (one 59-level MPAS column, 18 fields), parsed
   verbatim into float64 arrays so that tests can run without the reference checkout.
2. ``scenarios_oracle.npz``: the oracle's outputs for the reference's own integration
   scenarios on that column (test/tests.F90, driven by test/run_tempo_tests.F90):
   graupel and snow sedimentation at dt = 1, 10, 20, 60, 120, 300, 600 s over 1200 s,
   and the aerosol-aware / non-aerosol-aware cloud-number runs at dt = 20 s.  The
   reference's scenarios write their outputs to text files without assertions, so
   these arrays are regression fixtures of the oracle, not reference outputs.

Only this script reads the reference checkout; the tests read the .npz files.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(HERE.parent))

COLUMN_FIELDS = ("klev", "qv", "qc", "qr", "qi", "qs", "qg", "ni", "nr", "nc", "nwfa", "nifa",
                 "theta", "ng", "volg", "pressure", "w", "dz")
SEDI_DTS = (1.0, 10.0, 20.0, 60.0, 120.0, 300.0, 600.0)   # run_tempo_tests.F90:11-12
INTEGRATION_TIME = 1200                                  # tests.F90:46


def read_column(path: Path) -> dict:
    rows = [line.split() for line in path.read_text().splitlines()[1:] if line.strip()]
    a = np.array([[float(v) for v in r] for r in rows], dtype=np.float64)
    assert a.shape == (59, 18), a.shape
    return {n: a[:, i].copy() for i, n in enumerate(COLUMN_FIELDS)}


def _col(v):
    return np.array(v, dtype=np.float64).reshape(1, -1, 1)  # a copy: the step updates in place


def scenario_fields(col: dict, name: str) -> dict:
    """Initial 3-D fields (nj=1, nk=59, ni=1) of one scenario, as tests.F90 sets them."""
    z = np.zeros_like(col["qv"])
    t = col["theta"] * (col["pressure"] / 100000.0) ** 0.286
    f = dict(t=t, p=col["pressure"], dz=col["dz"], qv=col["qv"])
    if name == "graupel_sedimentation":        # tests.F90:70-83
        f.update(w=z, qc=z, qr=z, nr=z, qi=z, qs=z, ni=z, qg=col["qg"], ng=col["ng"],
                 qb=col["volg"] * 1000.0)
    elif name == "snow_sedimentation":         # tests.F90:170-180
        f.update(w=z, qc=z, qr=z, nr=z, qi=z, qs=col["qs"], ni=z, qg=z, ng=z, qb=z)
    elif name == "cloud_number_aerosolaware":  # tests.F90:251-264
        f.update(w=col["w"], qc=col["qc"], nc=col["nc"], qr=col["qr"], nr=col["nr"],
                 qi=col["qi"], qs=col["qs"], ni=col["ni"], qg=z)
    elif name == "cloud_number_non_aerosolaware":  # tests.F90:339-352
        f.update(w=col["w"], qc=col["qc"], qr=col["qr"], nr=col["nr"], qi=col["qi"],
                 qs=col["qs"], ni=col["ni"], qg=z)
    else:
        raise KeyError(name)
    return {k: _col(v) for k, v in f.items()}


def scenario_cfg(name: str) -> dict:
    over = dict(turn_off_micro_flag=1)
    if name == "graupel_sedimentation":
        over["graupel_med_vol_diam_flag"] = 1
    if name == "cloud_number_non_aerosolaware":
        over["cloud_number_mixing_ratio_flag"] = 1
    return over


# scenario -> (dts, tracked precip diagnostic, final fields kept, diagnostics kept)
SCENARIOS = {
    "graupel_sedimentation": (SEDI_DTS, "graupel_liquid_equiv_precip", ("qg", "ng", "qb"),
                              ("graupel_med_vol_diam",)),
    "snow_sedimentation": (SEDI_DTS, "snow_liquid_equiv_precip", ("qs",), ()),
    "cloud_number_aerosolaware": ((20.0,), None, ("qc", "nc", "qv", "t"), ()),
    "cloud_number_non_aerosolaware": ((20.0,), None, ("qc", "qv", "t"),
                                      ("cloud_number_mixing_ratio",)),
}


def run_scenario(step_fn, col: dict, name: str, dt: float) -> dict:
    """Runs one scenario through ``step_fn(fields, dt, itimestep, cfg_over) -> diags`` and
    returns the arrays kept for comparison (keys prefixed with the scenario and dt)."""
    dts, precip, keep, keep_d = SCENARIOS[name]
    f = scenario_fields(col, name)
    over = scenario_cfg(name)
    nsteps = int(INTEGRATION_TIME / dt)
    psum = 0.0
    series = []
    out = {}
    for step in range(1, nsteps + 1):
        d = step_fn(f, dt, step, over)
        if precip:
            psum = psum + float(d[precip][0, 0])
            series.append(psum)
        if step == 1:
            for k in keep:
                out[f"step1_{k}"] = f[k][0, :, 0].copy()
    for k in keep:
        out[f"final_{k}"] = f[k][0, :, 0].copy()
    for k in keep_d:
        out[f"final_{k}"] = d[k][0, :, 0].copy()
    if precip:
        out["precip_sum"] = np.array(series)
    tag = f"{name}__dt{int(dt)}"
    return {f"{tag}__{k}": v for k, v in out.items()}


def oracle_step_fn():
    import oracle
    from parity_util import make_diags
    oracle.build()
    oracle.init(True, REPO / "tables" / "ccn_activate.bin")

    def step(f, dt, itimestep, over):
        d = make_diags(f["p"].shape)
        rc = oracle.run(oracle.default_cfgs(**over), dt, itimestep, f, d, nthreads=1)
        assert rc == 0, rc
        return d
    return step


def reference_root(argv) -> Path:
    """The reference checkout: the first argument, else $TEMPO_REFERENCE."""
    import os
    root = argv[1] if len(argv) > 1 else os.environ.get("TEMPO_REFERENCE")
    if not root:
        raise SystemExit(f"usage: {argv[0]} <TEMPO reference checkout> (or set TEMPO_REFERENCE)")
    return Path(root)


def main(argv):
    ref = reference_root(argv)
    col = read_column(ref / "test" / "data" / "mpas_59lev_test.txt")
    np.savez_compressed(HERE / "mpas_59lev_column.npz", **col)
    step = oracle_step_fn()
    out = {}
    for name, (dts, *_rest) in SCENARIOS.items():
        for dt in dts:
            out.update(run_scenario(step, col, name, dt))
    np.savez_compressed(HERE / "scenarios_oracle.npz", **out)
    print(f"wrote {len(out)} arrays")


if __name__ == "__main__":
    main(sys.argv)
