"""Tangent-linear and adjoint of the column step through the C ABI.

* dot-product test: <TL dx, lam> = <dx, AD lam> for random input perturbations and
  random output adjoints (FP64 to 1e-11, FP32 to 1e-4);
* the tangent-linear step's values are the FP64 step's (to 1e-12);
* centred finite differences of the FP64 step (relative epsilon 1e-4) against the
  gradient of the precipitation/reflectivity cost from torch.autograd, on sampled
  (point, field) pairs whose difference quotients are stable (eps and eps/2 agree), i.e.
  away from thresholds;
* the FP32 gradient against the FP64 gradient.
Workload: the stretched-grid generator, dt = 60 s.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIFF = ("t", "qv", "qc", "nc", "qr", "nr", "qi", "ni", "qs", "qg")


def _setup(W, torch, dtype, ni=48, nj=8, seed=4):
    wl = W.stretched_grid(seed=seed, ni=ni, nj=nj, steps=1, dt=60.0)
    f = {k: torch.tensor(v, dtype=dtype, device="cuda") for k, v in wl.fields.items()}
    return wl, f


def _diags(f, torch):
    nj, nk, ni = f["p"].shape
    d = {n: torch.zeros((nj, ni), dtype=f["p"].dtype, device="cuda")
         for n in ("rain_precip", "ice_liquid_equiv_precip", "snow_liquid_equiv_precip",
                   "graupel_liquid_equiv_precip")}
    d["refl10cm"] = torch.zeros((nj, nk, ni), dtype=f["p"].dtype, device="cuda")
    return d


@pytest.mark.parametrize("dtype_name,tol", [("float64", 1e-11), ("float32", 1e-4)])
def test_dot_product(ctx_nohail, dtype_name, tol):
    torch = pytest.importorskip("torch")
    from tempo_gb300 import workloads as W
    dtype = getattr(torch, dtype_name)
    ctx = ctx_nohail
    wl, f = _setup(W, torch, dtype)
    g = torch.Generator(device="cuda").manual_seed(11)
    dx = {k: (f[k] if k != "t" else torch.ones_like(f[k])) *
          torch.randn(f[k].shape, generator=g, device="cuda", dtype=dtype) for k in DIFF}
    x = {k: v.clone() for k, v in f.items()}
    y = {k: v.clone() for k, v in f.items()}
    dy = {k: v.clone() for k, v in dx.items()}
    d, td = _diags(f, torch), _diags(f, torch)
    ctx.tl_device(y, dy, wl.dt, 1, diags=d, tdiags=td)
    lam = {k: torch.randn(f[k].shape, generator=g, device="cuda", dtype=dtype) /
           y[k].abs().max().clamp_min(1e-30) for k in DIFF}
    lamd = {k: torch.randn(v.shape, generator=g, device="cuda", dtype=dtype) for k, v in td.items()}
    lx = {k: v.clone() for k, v in lam.items()}
    ctx.adjoint_device(x, lx, wl.dt, 1, lam_diags=lamd)
    torch.cuda.synchronize()
    for k in f:  # the adjoint leaves the state it was given untouched
        assert torch.equal(x[k], f[k]), k
    lhs = sum(float((dy[k].double() * lam[k].double()).sum()) for k in DIFF) + \
        sum(float((td[k].double() * lamd[k].double()).sum()) for k in td)
    rhs = sum(float((dx[k].double() * lx[k].double()).sum()) for k in DIFF)
    assert abs(lhs - rhs) <= tol * max(abs(lhs), abs(rhs)), (lhs, rhs)


def test_tl_values_equal_fp64_step(ctx_nohail):
    torch = pytest.importorskip("torch")
    from tempo_gb300 import workloads as W
    ctx = ctx_nohail
    wl, f = _setup(W, torch, torch.float64)
    a = {k: v.clone() for k, v in f.items()}
    b = {k: v.clone() for k, v in f.items()}
    da, db = _diags(f, torch), _diags(f, torch)
    ctx.run_device(a, wl.dt, 1, diags=da)      # the context's default: FP64
    ctx.tl_device(b, {}, wl.dt, 1, diags=db)
    torch.cuda.synchronize()
    for k in DIFF:   # FP64 parity bar: 1e-12 relative
        torch.testing.assert_close(b[k], a[k], rtol=1e-12, atol=1e-300)
    for k in da:
        torch.testing.assert_close(db[k], da[k], rtol=1e-12, atol=1e-12)


def _cost_and_grad(ctx, f, dt, torch):
    from tempo_gb300.autograd import cost_precip_reflectivity, tempo_step
    x = {k: (v.clone().requires_grad_(k in DIFF)) for k, v in f.items()}
    new, diags = tempo_step(ctx, x, dt, 1)
    J = cost_precip_reflectivity(diags, f["dz"])
    J.backward()
    return float(J.detach()), {k: x[k].grad for k in DIFF}


def test_gradient_matches_finite_differences(ctx_nohail):
    torch = pytest.importorskip("torch")
    from tempo_gb300 import workloads as W
    from tempo_gb300.autograd import cost_precip_reflectivity, tempo_step
    ctx = ctx_nohail
    wl, f = _setup(W, torch, torch.float64, ni=24, nj=4)
    J0, grad = _cost_and_grad(ctx, f, wl.dt, torch)

    def J_of(ff):
        with torch.no_grad():
            _, d = tempo_step(ctx, ff, wl.dt, 1)
            return float(cost_precip_reflectivity(d, f["dz"]))

    rng = np.random.default_rng(3)
    nz_idx = {k: torch.nonzero(f[k]).cpu().numpy() for k in DIFF}
    checked, bad = 0, []
    for _ in range(800):
        if checked >= 60:
            break
        k = DIFF[rng.integers(len(DIFF))]
        nonzero = nz_idx[k]
        if len(nonzero) == 0:
            continue
        j, l, i = (int(v) for v in nonzero[rng.integers(len(nonzero))])
        x0 = float(f[k][j, l, i])
        h = 1e-4 * abs(x0)
        Jh = {}
        for m in (1.0, -1.0, 0.5, -0.5):
            ff = {kk: v.clone() for kk, v in f.items()}
            ff[k][j, l, i] += m * h
            Jh[m] = J_of(ff)
        c1 = (Jh[1.0] - Jh[-1.0]) / (2 * h)
        c2 = (Jh[0.5] - Jh[-0.5]) / h
        dp, dm = (Jh[1.0] - J0) / h, (J0 - Jh[-1.0]) / h
        floor = 1e-9 * abs(J0) / abs(x0)
        # differentiable here: the one-sided quotients agree (no kink or clip at x0)
        # and the centred ones converge (no threshold crossed within the perturbation)
        if abs(dp - dm) > 1e-2 * abs(c1) + floor or abs(c1 - c2) > 1e-4 * abs(c2) + floor:
            continue
        g = float(grad[k][j, l, i])
        checked += 1
        if abs(g - c2) > 1e-4 * abs(c2) + floor:
            bad.append((k, j, l, i, x0, g, c2, dp, dm))
    assert checked >= 40, checked
    assert len(bad) <= 0.05 * checked, (len(bad), checked, bad[:5])


def test_fp32_gradient_close_to_fp64(ctx_nohail):
    torch = pytest.importorskip("torch")
    from tempo_gb300 import workloads as W
    ctx = ctx_nohail
    wl, f64 = _setup(W, torch, torch.float64)
    f32 = {k: v.float() for k, v in f64.items()}
    f64 = {k: v.double() for k, v in f32.items()}  # identical inputs
    _, g64 = _cost_and_grad(ctx, f64, wl.dt, torch)
    _, g32 = _cost_and_grad(ctx, f32, wl.dt, torch)
    for k in DIFF:
        a, b = g32[k].double(), g64[k]
        scale = b.abs().max().clamp_min(1e-300)
        e = (a - b).abs() / scale
        assert float((e > 1e-3).double().mean()) <= 1e-2, (k, float(e.max()))
