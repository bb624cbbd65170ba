"""Benchmark of the TEMPO column step on GB300.

Workload (default): 1024 x 1024 = 1,048,576 columns x 65 levels on the stretched
20-km grid, 40 % clear columns, dt = 30 s (the batched FP32 forward configuration),
synthetic seeded profiles generated on the device.  One "step" = one column step over
all columns; the state is carried from step to step like a model integration.

Prints ONE JSON line.  `value` is device-resident throughput (column-steps/s) of the
mixed-precision (FP32 bulk, FP64 islands) path; `e2e` is the same metric through the
host C ABI (tempo_run_f32_c: host arrays, host<->device copies inside the timed
region).  `--impl reference` times the CPU restatement of the reference (the Fortran
reference has no compiler here) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

METRIC = "column-steps/s @65 lev: FP32 vs FP64 GPU vs CPU at stated err; adjoint/fwd ratio"
# algorithmic HBM bytes per column-step, hail off: read 15 3-D fields, write 12
# prognostic + 4 diagnostic 3-D fields, plus 8 2-D diagnostics
N_IN3, N_OUT3, N_OUT2 = 15, 16, 8


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ni", type=int, default=1024)
    ap.add_argument("--nj", type=int, default=1024)
    ap.add_argument("--nz", type=int, default=65)
    ap.add_argument("--dt", type=float, default=30.0)
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=8)
    ap.add_argument("--tuning", default=None,
                    help="points variant, point order, sedimentation variant (e.g. 5,1,5): "
                         "set instead of autotuning (for profiling a fixed configuration)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-multi", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-precision", action="store_true")
    ap.add_argument("--ref-columns", type=int, default=131072,
                    help="columns per step of the reference arm's bounded sample")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons)}


def peaks():
    try:
        return json.loads((REPO / "MEASURED_PEAKS.json").read_text())
    except Exception:
        return {}


def traffic_from_profiles(ncol: int):
    """DRAM bytes of one step at ncol columns: the ncu figure of the 65 536-column step
    in profiles/step_dram_traffic_65k.md, scaled by columns (every term of the traffic
    grows with the number of columns)."""
    import re
    try:
        txt = (REPO / "profiles" / "step_dram_traffic_65k.md").read_text()
        m = re.search(r"dram_bytes_per_step_(\d+)_columns = (\d+)", txt)
        return float(m.group(2)) * ncol / float(m.group(1)) if m else None
    except OSError:
        return None


def fp32_ops_from_profiles(ncol: int):
    """FP32 floating-point operations of one step at ncol columns (add, multiply and 2 per
    fused multiply-add, thread instructions counted by ncu on a 65 536-column step in
    profiles/step_fp32_ops_65k.md), scaled by columns."""
    import re
    try:
        txt = (REPO / "profiles" / "step_fp32_ops_65k.md").read_text()
        m = re.search(r"fp32_flops_per_step_(\d+)_columns = (\d+)", txt)
        return float(m.group(2)) * ncol / float(m.group(1)) if m else None
    except OSError:
        return None


def cpu_baseline(seconds: float, nz: int, dt: float, sample_cols: int = 16384):
    """The FP64 CPU restatement (oracle port) on all host cores, bounded sample."""
    import oracle
    from tempo_gb300 import workloads as W
    oracle.build()
    oracle.init(False, REPO / "tables" / "ccn_activate.bin")
    oracle.build_big_tables()
    wl = W.stretched_grid(seed=11, ni=sample_cols, nj=1, nz=nz, steps=1, dt=dt)
    cfg = oracle.default_cfgs(hailaware_flag=0)
    f = {k: v.copy() for k, v in wl.fields.items()}
    nj, nk, ni = f["p"].shape
    d = {"rain_precip": np.zeros((nj, ni)), "refl10cm": np.zeros((nj, nk, ni)),
         "re_cloud": np.zeros((nj, nk, ni)), "re_ice": np.zeros((nj, nk, ni)),
         "re_snow": np.zeros((nj, nk, ni))}
    oracle.run(cfg, dt, 1, f, d)  # warm
    n, t0 = 0, time.perf_counter()
    while True:
        oracle.run(cfg, dt, 2 + n, f, d)
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    cores = os.cpu_count()
    return {"value": sample_cols * n / el, "unit": "column-steps/s", "cores": cores,
            "kind": "port",
            "sample": f"{n} steps x {sample_cols} columns x {nz} levels of the same generator, "
                      f"FP64 CPU restatement, {cores} OpenMP threads, {el:.1f} s"}


# per-field floors below which differences are measured against the floor (the
# reference's existence thresholds r1 = 1e-12, r2 = 1e-6, in per-kg units)
FLOORS = {"t": 1.0, "qv": 1e-12, "qc": 1e-12, "qr": 1e-12, "qi": 1e-12, "qs": 1e-12,
          "qg": 1e-12, "ni": 1e-6, "nr": 1e-6, "nc": 1e-6, "nwfa": 1.0, "nifa": 1.0,
          "rain_precip": 1e-12, "snow_liquid_equiv_precip": 1e-12,
          "graupel_liquid_equiv_precip": 1e-12, "ice_liquid_equiv_precip": 1e-12,
          "re_cloud": 1e-9, "re_ice": 1e-9, "re_snow": 1e-9}


def mixed_vs_fp64(f32, d32, f64, d64, x0):
    """Per-field max and RMS relative error of one mixed step against one FP64 step
    from the same state x0; relative to the larger of the FP64 result, the field's
    value before the step (an update that cancels) and the floor; reflectivity as max
    and RMS absolute dBZ difference."""
    import torch
    out = {}
    for src32, src64 in ((f32, f64), (d32, d64)):
        for k, fl in FLOORS.items():
            if k in src32 and k in src64:
                a = src32[k].double()
                b = src64[k]
                den = b.abs().clamp_min(fl)
                if k in x0:
                    den = torch.maximum(den, x0[k].double().abs())
                e = (a - b).abs() / den
                out[k] = {"max": float(e.max()), "rms": float(torch.sqrt((e * e).mean())),
                          "frac_gt_1e-5": float((e > 1e-5).double().mean())}
    if "refl10cm" in d32:
        e = (d32["refl10cm"].double() - d64["refl10cm"]).abs()
        out["refl10cm_dbz"] = {"max_abs": float(e.max()),
                               "rms_abs": float(torch.sqrt((e * e).mean()))}
    return out


def adjoint_timing(ctx, tg, W, torch, device, reps=3):
    """Forward, tangent-linear and adjoint step on the adjoint workload: 65536 columns x
    65 levels (256 x 256), dt = 60 s, cost J = sum of surface precipitation + 1e-3 x
    sum of linear reflectivity x dz.  ms per call from CUDA events on the current
    stream; FP64 (forward = the FP64 step) and FP32 (forward = the mixed-precision
    production step; the tangent-linear and adjoint steps differentiate the all-FP32
    step)."""
    from tempo_gb300.autograd import cost_precip_reflectivity
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    diff = ("t", "qv", "qc", "nc", "qr", "nr", "qi", "ni", "qs", "qg")

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    base = W.stretched_grid_torch(seed=7, ni=256, nj=256, nz=65, device=device, dtype=torch.float64)
    out = {"workload": "65536 columns x 65 levels, dt=60s, J = sum precip + 1e-3 sum Ze dz",
           "reps": reps}
    for name, dtype in (("fp64", torch.float64), ("fp32", torch.float32)):
        f = {k: v.to(dtype) for k, v in base.items()}
        nj, nk, ni = f["p"].shape
        dg = {n: torch.zeros((nj, ni), dtype=dtype, device=device) for n in tg.DIAG2[:4]}
        dg["refl10cm"] = torch.zeros((nj, nk, ni), dtype=dtype, device=device)
        x = {k: v.clone() for k, v in f.items()}
        ctx.tl_device(x, {}, 60.0, 1, diags=dg)
        leaf = {k: v.clone().requires_grad_(True) for k, v in dg.items()}
        J = cost_precip_reflectivity(leaf, f["dz"])
        gl = torch.autograd.grad(J, list(leaf.values()))
        lamd = {k: g.detach().contiguous() for k, g in zip(leaf, gl)}
        ctx.set_precision(tg.PREC_FP64 if dtype == torch.float64 else tg.PREC_MIXED)
        xf = {k: v.clone() for k, v in f.items()}
        fwd_ms = timed(lambda: ctx.run_device(xf, 60.0, 2, diags=dg))
        xt = {k: v.clone() for k, v in f.items()}
        dx = {k: 1e-3 * f[k] for k in diff}
        tl_ms = timed(lambda: ctx.tl_device(xt, dx, 60.0, 2, diags=dg))
        lam0 = {k: torch.zeros_like(f[k]) for k in diff}
        lam = {k: v.clone() for k, v in lam0.items()}

        def adj():
            for k in diff:
                lam[k].copy_(lam0[k])
            ctx.adjoint_device(f, lam, 60.0, 1, lam_diags=lamd)
        ad_ms = timed(adj)
        out[name] = {"forward_ms": fwd_ms, "tl_ms": tl_ms, "adjoint_ms": ad_ms,
                     "adjoint_over_forward": ad_ms / fwd_ms,
                     "grad_norm": float(sum((lam[k].double() ** 2).sum() for k in diff) ** 0.5)}
        del f, x, xf, xt, dx, lam, lam0, dg, leaf
        torch.cuda.empty_cache()
    ctx.set_precision(tg.PREC_MIXED)
    return out


def multi_domain(ctx, tg, W, torch, device, steps=3):
    """The uneven multi-domain batch: 24 domains with log-uniform column counts
    (1e3 .. 5e5), 50 to 128 levels and dt of 10 to 60 s (seeded descriptors), the large
    tables rebuilt on the GPU first.  One batch step is ONE launch sequence over every
    domain (tempo_run_batch_dev_f32_c: prep, regime order, the persistent points kernel
    drawing (domain, point) items from one work queue, sedimentation and final kernels
    over all domains); the same domains stepped one call each are timed beside it.  ms
    from CUDA events; value = all domains' columns x steps / time; the level-point rate
    and the rate in 65-level column equivalents compare it with the single-domain run."""
    doms = W.domain_set(seed=0)
    table_ms = ctx.build_tables()
    data = []
    for d, (ncol, nz, dt, seed) in enumerate(doms):
        f = W.stretched_grid_torch(seed=100 + d, ni=ncol, nj=1, nz=nz, device=device, dtype=torch.float32)
        dg = {n: torch.zeros((1, ncol), device=device) for n in tg.DIAG2}
        dg.update({n: torch.zeros((1, nz, ncol), device=device)
                   for n in ("refl10cm", "re_cloud", "re_ice", "re_snow")})
        data.append((f, dg, dt))
    ncols = sum(d[0] for d in doms)
    npoints = sum(d[0] * d[1] for d in doms)
    ctx.set_graphs(False)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def batch(it):
        ctx.run_batch_device([dict(fields=f, diags=dg, dt=dt, itimestep=it) for f, dg, dt in data])

    def sequential(it):
        for f, dg, dt in data:
            ctx.run_device(f, dt, it, diags=dg)

    def timed(fn, it0):
        fn(it0)
        torch.cuda.synchronize()
        e0.record(stream)
        for it in range(it0 + 1, it0 + 1 + steps):
            fn(it)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    ms = timed(batch, 1)
    ms_seq = timed(sequential, 2 + steps)
    # kernel durations of one batch step and of one step per domain (CUDA events of the
    # library on the launching stream)
    ctx.set_kernel_timing(True)
    batch(3 + 2 * steps)
    kb = ctx.kernel_times()
    ks = {k: 0.0 for k in kb}
    for f, dg, dt in data:
        ctx.run_device(f, dt, 4 + 2 * steps, diags=dg)
        for k, v in ctx.kernel_times().items():
            ks[k] += v
    ctx.set_kernel_timing(False)
    del data
    torch.cuda.empty_cache()
    return {"workload": "24 domains, columns log-uniform in [1e3, 5e5], nz in {50, 65, 90, 128}, "
                        "dt in {10, 20, 30, 60} s, mixed precision, tables rebuilt first, one "
                        "launch sequence per batch step",
            "domains": [{"columns": n, "levels": z, "dt": t} for n, z, t, _ in doms],
            "columns": ncols, "column_levels": npoints, "table_build_ms": table_ms, "steps": steps,
            "ms_per_batch_step": ms, "value": ncols / (ms / 1e3), "unit": "column-steps/s",
            "level_point_steps_per_s": npoints / (ms / 1e3),
            "columns65_steps_per_s": npoints / 65.0 / (ms / 1e3),
            "sequential_ms_per_step": ms_seq,
            "sequential_value": ncols / (ms_seq / 1e3),
            "batch_kernel_ms": kb, "sequential_kernel_ms_sum": ks}


def precision_study(tg, W, torch, device, ncol_side=512):
    """The precision study on hail-aware deep convection: 262 144 hail-aware deep-convective columns x 65
    levels (qg lognormal, median 2 g/kg clipped at 8, ng log-uniform 1e2..1e5, graupel
    density 300..900 kg m-3, supercooled cloud water; the seeded generator on the
    device), on a hail-aware context: one step of the mixed form (FP32 bulk, FP64-grade
    islands) and one of the FP64 GPU path from the same state, against the FP64 CPU
    oracle run from the same state with the same tables.  Columns whose oracle step
    passed a rounding tie of an index (the graupel density class at its clamp, a substep
    count) are counted and left out: there the reference's own result depends on the
    last bit of a libm value.  Per field: max and RMS relative error (relative to the
    larger of the oracle's value and the field's existence floor), the fraction of
    points beyond 1e-5, the normwise error max|d| / max|ref| and the relative RMS
    ||d|| / ||ref||; column water budget (total water plus surface precipitation,
    after minus before) against the oracle's, relative to the column's water; 10-cm
    reflectivity difference in dBZ."""
    import tempfile
    import oracle
    dt = 30.0
    ctx = tg.TempoContext(build_tables=True, cfgs=tg.default_cfgs(hailaware_flag=1))
    gen = W.stretched_grid_torch(seed=3, ni=ncol_side, nj=ncol_side, nz=65, device=device,
                          dtype=torch.float32, hail=True, deep=True)
    fields = {k: v.cpu().numpy() for k, v in gen.items()}
    del gen
    ncols = ncol_side * ncol_side
    over = dict(hailaware_flag=1, rain_med_vol_diam_flag=1, graupel_med_vol_diam_flag=1)
    cfg = tg.default_cfgs(**over)
    x0 = {k: v.astype(np.float64) for k, v in fields.items()}
    nj, nk, ni = fields["p"].shape
    dnames = tg.DIAG2 + ("refl10cm", "re_cloud", "re_ice", "re_snow", "rain_med_vol_diam",
                         "graupel_med_vol_diam")

    def gpu(dtype, prec):
        f = {k: torch.tensor(v, device=device, dtype=dtype) for k, v in fields.items()}
        d = {n: torch.zeros((nj, ni) if n in tg.DIAG2 else (nj, nk, ni), device=device, dtype=dtype)
             for n in dnames}
        ctx.set_precision(prec)
        ctx.run_device(f, dt, 1, diags=d, cfgs=cfg)
        torch.cuda.synchronize()
        return ({k: v.double().cpu().numpy() for k, v in f.items()},
                {k: v.double().cpu().numpy() for k, v in d.items()})

    fm, dm = gpu(torch.float32, tg.PREC_MIXED)
    f64, d64 = gpu(torch.float64, tg.PREC_FP64)
    # the oracle on every column, with the context's tables
    with tempfile.TemporaryDirectory() as td:
        for fam, fn in (("qr_acr_qg", "qr_acr_qg_data_tempo_v3"), ("qr_acr_qs", "qr_acr_qs_data_tempo_v3"),
                        ("freezewater", "freeze_water_data_tempo_v3")):
            ctx.write_table(fam, Path(td) / fn)
        oracle.build()
        oracle.init(True, REPO / "tables" / "ccn_activate.bin")
        lib = oracle.load()
        for fn, rd in (("freeze_water_data_tempo_v3", lib.oracle_read_freezewater),
                       ("qr_acr_qs_data_tempo_v3", lib.oracle_read_qr_acr_qs),
                       ("qr_acr_qg_data_tempo_v3", lib.oracle_read_qr_acr_qg)):
            if rd(f"{td}/{fn}".encode()) != 0:
                raise IOError(f"oracle could not read {fn}")
    ctx.close()
    fo = {k: v.copy() for k, v in x0.items()}
    do = {n: np.zeros((nj, ni) if n in tg.DIAG2 else (nj, nk, ni)) for n in dnames}
    ties = np.zeros((nj, ni), np.int32)
    t0 = time.perf_counter()
    oracle.run(oracle.default_cfgs(**over), dt, 1, fo, do, ties=ties)
    oracle_s = time.perf_counter() - t0
    clean = (ties & 1) == 0

    floors = dict(FLOORS, ng=1e-6, qb=1e-12, rain_med_vol_diam=1e-9, graupel_med_vol_diam=1e-9,
                  max_hail_diameter_sfc=1e-6, max_hail_diameter_column=1e-6)

    def errs(A, B):
        out = {}
        for k, fl in floors.items():
            if k not in A or k not in B:
                continue
            m = clean[:, None, :] if A[k].ndim == 3 else clean
            a, b = A[k][np.broadcast_to(m, A[k].shape)], B[k][np.broadcast_to(m, B[k].shape)]
            d = np.abs(a - b)
            e = d / np.maximum(np.abs(b), fl)
            # the same with the floor at 1e-7 of the field's largest value (the FP32
            # resolution of the field's scale)
            es = d / np.maximum(np.abs(b), 1e-7 * max(np.abs(b).max(), 1e-300))
            out[k] = {"max": float(e.max()), "rms": float(np.sqrt((e * e).mean())),
                      "frac_gt_1e-5": float((e > 1e-5).mean()),
                      "max_scaled_floor": float(es.max()),
                      "frac_scaled_floor_gt_1e-5": float((es > 1e-5).mean()),
                      "normwise": float(d.max() / max(np.abs(b).max(), 1e-300)),
                      "rel_rms": float(np.sqrt((d * d).sum() / max((b * b).sum(), 1e-300)))}
        a, b = A["refl10cm"], B["refl10cm"]
        e = np.abs(a - b)[np.broadcast_to(clean[:, None, :], a.shape)]
        out["refl10cm_dbz"] = {"max_abs": float(e.max()), "rms_abs": float(np.sqrt((e * e).mean()))}
        return out

    roverrv = 287.04 / 461.5
    rho = roverrv * x0["p"] / (287.04 * x0["t"] * (np.maximum(1e-10, x0["qv"]) + roverrv))

    def budget(F, D):
        q = sum(F[n] for n in ("qv", "qc", "qr", "qi", "qs", "qg"))
        return (q * rho * x0["dz"]).sum(axis=1) + sum(D[n] for n in tg.DIAG2[:4])

    w0 = budget(x0, {n: 0.0 for n in tg.DIAG2[:4]})
    ro = budget(fo, do) - w0
    cons = {name: float(np.max((np.abs(budget(F, D) - w0 - ro) / w0)[clean]))
            for name, F, D in (("mixed", fm, dm), ("fp64_gpu", f64, d64))}
    return {"workload": f"{ncols} hail-aware deep-convective columns x {nk} levels, dt={dt}s "
                        "(seeded generator on the device)",
            "oracle_columns": ncols, "oracle_tie_columns": int((~clean).sum()),
            "oracle_seconds": oracle_s,
            "mixed_vs_oracle": errs({**fm, **dm}, {**fo, **do}),
            "fp64_gpu_vs_oracle": errs({**f64, **d64}, {**fo, **do}),
            "column_water_budget_vs_oracle_max_rel": cons}


def run_reference(args, rank, world):
    """The reference arm: the FP64 CPU restatement on all host cores (the Fortran
    reference has no compiler on either machine), W untimed and K timed steps, each
    step one bounded sample of the workload's columns.  Rank 0 only."""
    if rank != 0:
        return
    import oracle
    from tempo_gb300 import workloads as W
    oracle.build()
    oracle.init(False, REPO / "tables" / "ccn_activate.bin")
    oracle.build_big_tables()
    ncol = args.ref_columns
    wl = W.stretched_grid(seed=11, ni=ncol, nj=1, nz=args.nz, steps=1, dt=args.dt)
    cfg = oracle.default_cfgs(hailaware_flag=0)
    f = {k: v.copy() for k, v in wl.fields.items()}
    nj, nk, ni = f["p"].shape
    d = {"rain_precip": np.zeros((nj, ni)), "refl10cm": np.zeros((nj, nk, ni)),
         "re_cloud": np.zeros((nj, nk, ni)), "re_ice": np.zeros((nj, nk, ni)),
         "re_snow": np.zeros((nj, nk, ni))}
    it = 1
    for _ in range(args.warmup):
        oracle.run(cfg, args.dt, it, f, d)
        it += 1
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.run(cfg, args.dt, it, f, d)
        it += 1
    el = time.perf_counter() - t0
    value = ncol * args.steps / el
    cores = os.cpu_count()
    sample = (f"each step {ncol} of the {args.ni * args.nj} columns x {args.nz} levels of the "
              f"same generator, FP64 CPU restatement, {cores} OpenMP threads, "
              f"{args.steps} steps in {el:.1f} s")
    line = {"metric": METRIC, "impl": "reference", "value": value, "unit": "column-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded stretched-grid column generator)",
            "config": {"workload": f"{args.ni * args.nj} columns x {args.nz} levels, stretched 20 km grid, "
                                   f"dt={args.dt}s; each timed step is a bounded sample of "
                                   f"{ncol} of its columns (ms_per_step is the sample's)",
                       "parallelism": "cpu-openmp"},
            "cpu_baseline": {"value": value, "unit": "column-steps/s", "cores": cores,
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "column-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    import torch.distributed as dist
    import tempo_gb300 as tg
    from tempo_gb300 import workloads as W

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    tg.build.build()
    ctx = tg.TempoContext(build_tables=True, device=local, cfgs=tg.default_cfgs(hailaware_flag=0))
    ctx.set_precision(tg.PREC_MIXED)
    ni, nj, nz = args.ni, args.nj, args.nz
    ncol = ni * nj
    f32 = W.stretched_grid_torch(seed=rank, ni=ni, nj=nj, nz=nz, device=f"cuda:{local}",
                          dtype=torch.float32)
    diag = {n: torch.zeros((nj, ni), device=f"cuda:{local}", dtype=torch.float32) for n in tg.DIAG2}
    diag.update({n: torch.zeros((nj, nz, ni), device=f"cuda:{local}", dtype=torch.float32)
                 for n in ("refl10cm", "re_cloud", "re_ice", "re_snow")})
    stream = torch.cuda.current_stream()
    # warm-up: the first steps move the generated state towards the ones the timed steps
    # see (condensation, evaporation and sedimentation change where the work is); the
    # autotuner then scores every per-level kernel variant in both point orders
    # (level-major, regime) over the next steps on a private copy of that state, and the
    # last warm-up step captures the CUDA graph of the chosen candidate (the timed steps
    # replay it, with per-kernel timing events in the graph): W warm-up steps in all
    ctx.set_points_variant(4)
    it = 1
    for _ in range(max(args.warmup - 1, 1)):
        ctx.run_device(f32, args.dt, it, diags=diag)
        it += 1
    if args.tuning:
        pv, po, sv = (int(x) for x in args.tuning.split(","))
        ctx.set_points_variant(pv)
        ctx.set_points_order(po)
        ctx.set_sedim_variant(sv)
        variant_ms = []
    else:
        variant, variant_ms = ctx.autotune_device(f32, args.dt, it, diags=diag, reps=6)
    tuning = ctx.tuning()
    ctx.set_kernel_timing(True)
    ctx.set_graphs(True)
    ctx.run_device(f32, args.dt, it, diags=diag)
    ctx.kernel_times()
    it += 1
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # per-kernel durations: CUDA events recorded by the library around its four
    # kernels on the launching stream, read after each step
    kms = {k: 0.0 for k in ctx.KERNELS}
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            ctx.run_device(f32, args.dt, it, diags=diag)
            it += 1
            for k, v in ctx.kernel_times().items():
                kms[k] += v
        e1.record(stream)
        torch.cuda.synchronize()
    ctx.set_kernel_timing(False)
    ctx.set_graphs(False)
    ms = e0.elapsed_time(e1)
    kms = {k: v / args.steps for k, v in kms.items()}
    step_kernel_ms = sum(kms.values())
    stats = ctx.stats()
    if world > 1:
        t = torch.tensor([ms], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    value = world * ncol * args.steps / (ms / 1e3)

    # FP64 drop-in on the same columns (a few steps; FP64 is 1/64 rate on GB300).  Its
    # first step, from the same state as one mixed step, gives the mixed form's error.
    ctx.set_precision(tg.PREC_FP64)
    f64 = {k: v.double() for k, v in f32.items()}
    d64 = {k: v.double() for k, v in diag.items()}
    x0 = {k: v.clone() for k, v in f32.items() if k in FLOORS}
    ctx.run_device(f64, args.dt, it, diags=d64)
    ctx.set_precision(tg.PREC_MIXED)
    ctx.run_device(f32, args.dt, it, diags=diag)
    torch.cuda.synchronize()
    mixed_error = mixed_vs_fp64(f32, diag, f64, d64, x0)
    del x0
    ctx.set_precision(tg.PREC_FP64)
    e0.record(stream)
    for s in range(args.fp64_steps):
        ctx.run_device(f64, args.dt, 2 + s, diags=d64)
    e1.record(stream)
    torch.cuda.synchronize()
    ms64 = e0.elapsed_time(e1) / args.fp64_steps
    del f64, d64
    torch.cuda.empty_cache()

    # end-to-end through the host C ABI (pinned host arrays, copies in the timed region)
    ctx.set_precision(tg.PREC_MIXED)
    host = {k: v.cpu().pin_memory().numpy() for k, v in f32.items()}
    hdiag = {k: torch.zeros(v.shape, dtype=torch.float32).pin_memory().numpy() for k, v in diag.items()}
    h2d = sum(a.nbytes for a in host.values())
    d2h = sum(a.nbytes for k, a in host.items() if k not in ("p", "w", "dz")) + \
        sum(a.nbytes for a in hdiag.values())
    ctx.run(host, args.dt, 1, diags=hdiag)
    # each call returns after its last copy back, so the host clock brackets one step
    e2e_step_ms = []
    t0 = time.perf_counter()
    for s in range(args.e2e_steps):
        ts = time.perf_counter()
        ctx.run(host, args.dt, 2 + s, diags=hdiag)
        e2e_step_ms.append(round((time.perf_counter() - ts) * 1e3, 2))
    e2e_s = (time.perf_counter() - t0) / args.e2e_steps
    e2e_value = world * ncol / e2e_s

    adjoint = None
    if not args.no_adjoint:
        del host, hdiag
        try:
            adjoint = adjoint_timing(ctx, tg, W, torch, f"cuda:{local}")
        except Exception as e:  # reported beside the headline, never required
            adjoint = {"error": str(e)}

    prec = None
    if not args.no_precision:
        try:
            prec = precision_study(tg, W, torch, f"cuda:{local}")
        except Exception as e:  # reported beside the headline, never required
            prec = {"error": str(e)}
        torch.cuda.empty_cache()

    multi = None
    if not args.no_multi:
        try:
            ctx.set_precision(tg.PREC_MIXED)
            multi = multi_domain(ctx, tg, W, torch, f"cuda:{local}")
        except Exception as e:  # reported beside the headline, never required
            multi = {"error": str(e)}

    pk = peaks()
    hbm = pk.get("hbm_gbs")
    peak_src = "measured" if hbm else "fallback"
    hbm = hbm or 6800.0
    alg_bytes = ncol * (4 * nz * (N_IN3 + N_OUT3) + 4 * N_OUT2)
    achieved = alg_bytes / (step_kernel_ms / 1e3) / 1e9
    # FP32 pipe roofline beside the HBM one: the step's FP32 operations over its kernel
    # time, against SMs x 128 FP32 lanes x 2 x the maximum SM clock (nominal)
    flops = fp32_ops_from_profiles(ncol)
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    fp32_peak = sms * 128 * 2 * float(pk.get("sm_max_mhz") or 2070.0) * 1e6 / 1e12
    fp32_roof = None
    if flops:
        fp32_ach = flops / (step_kernel_ms / 1e3) / 1e12
        fp32_roof = {"achieved": fp32_ach, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": fp32_ach / fp32_peak, "flops_per_step": flops,
                     "source": "ncu FP32 add/mul/fma thread instructions of one 65 536-column "
                               "step scaled by columns; peak nominal (SMs x 128 x 2 x max clock)"}
    clocks = clk.summary()
    out = {
        "metric": METRIC, "value": value, "unit": "column-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded stretched-grid column generator on device)",
        "config": {"workload": f"{ncol} columns x {nz} levels, stretched 20 km grid, "
                               f"40% clear, dt={args.dt}s, mixed precision (FP32 bulk, FP64 "
                               f"islands), aerosol-aware, hail-aware off",
                   "columns_per_gpu": ncol, "levels": nz, "dt": args.dt,
                   "l2": "inputs (8.5 GB) larger than L2", "parallelism": f"replicas x{world}"},
        "fp64_value": world * ncol / (ms64 / 1e3), "fp64_ms_per_step": ms64,
        "fp32_over_fp64": ms64 / ms_step,
        "mixed_error_vs_fp64": mixed_error,
        "autotune": {**tuning, "points_order": ("level-major", "regime")[tuning["points_order"]],
                     "points_ms_per_candidate": variant_ms[:16], "sedim_ms_per_variant": variant_ms[16:]},
        "e2e": {"value": e2e_value, "unit": "column-steps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "path": "tempo_run_f32_c (host arrays)",
                "step_ms": e2e_step_ms, "median_step_ms": statistics.median(e2e_step_ms)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic_from_profiles(ncol),
                     "traffic_source": "ncu dram bytes of one 65 536-column step scaled by columns",
                     "kernel": "column step = tempo_{prep,regime_order,points,sedim,final}_kernel",
                     "algorithmic_bytes_per_launch": alg_bytes, "peak_source": peak_src,
                     "kernel_ms": kms,
                     "kernel_share": {k: v / step_kernel_ms for k, v in kms.items()}},
        "fp32_roofline": fp32_roof,
        "adjoint": adjoint,
        "multi_domain": multi,
        "precision_study_hail": prec,
        "gpu_launches": args.steps * stats.get("launches", 1),
        "clocks": clocks,
        "step_stats": stats,
    }
    if rank == 0 and not args.no_cpu:
        try:
            out["cpu_baseline"] = cpu_baseline(args.cpu_seconds, nz, args.dt)
            cv = out["cpu_baseline"]["value"]
            # precision-matched speed-ups over the FP64 CPU restatement: the FP64 GPU
            # drop-in (same arithmetic) beside the mixed form (the headline)
            out["speedup_over_cpu"] = {"fp64_gpu": out["fp64_value"] / cv, "mixed_gpu": value / cv,
                                       "mixed_gpu_e2e": e2e_value / cv}
        except Exception as e:  # the baseline is reported, never required
            out["cpu_baseline"] = {"value": None, "error": str(e)}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
