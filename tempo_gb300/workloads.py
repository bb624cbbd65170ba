"""Seeded synthetic column workloads for the TEMPO column step.

The reference measures on no public dataset; these generators stand in for real
model columns with the shapes, sizes and value distributions of the five benchmark
configurations:

* ``uniform_grid``: 256 columns x 60 levels, uniform dz = 250 m, dt = 20 s,
  aerosol-aware, no hail prognostics (ng/qb not passed).
* ``stretched_grid``: 1024 x 1024 columns x 65 levels on a stretched grid (dz 50 m at the
  surface to 500 m at 20 km), 40 % clear columns, random cloud base/depth,
  w ~ N(0, 3) with 5 % convective columns, dt = 30 s.
* ``hail_convection``: 262144 deep-convective columns x 65 levels with hail-aware
  2-moment graupel (ng, qb passed), dt = 30 s.
* ``stretched_grid_dt60``: 65536 columns from the stretched-grid generator, dt = 60 s.
* ``domain_set``: 24 domains, column counts log-uniform in 1e3..5e5, nz in
  {50, 65, 90, 128}, dt in {10, 20, 30, 60}.

Fields are returned as float64 arrays shaped ``(nj, nk, ni)`` -- the Fortran
``(i, k, j)`` memory order of ``tempo_run`` with i fastest -- and k = 0 is the
surface, as in the reference.  Mixing ratios are kg/kg, numbers 1/kg, qb is
L/kg (the unit ``tempo_run`` expects, module_mp_tempo_main.F90:1168).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

G = 9.8
RD = 287.04
T0 = 273.15


def calc_rslf(p: np.ndarray, t: np.ndarray) -> np.ndarray:
    """Liquid saturation mixing ratio, the polynomial of module_mp_tempo_utils.F90:285-309."""
    c = [.611583699E03, .444606896E02, .143177157e01, .264224321e-1, .299291081e-3,
         .203154182e-5, .702620698e-8, .379534310e-11, -.321582393e-13]
    x = np.maximum(-80.0, t - 273.16)
    esl = c[8]
    for ci in c[7::-1]:
        esl = ci + x * esl
    esl = np.minimum(esl, p * 0.15)
    return 0.622 * esl / (p - esl)


def stretched_dz(nz: int, top: float = 20000.0, dz0: float = 50.0, dz1: float = 500.0) -> np.ndarray:
    """dz_k = dz0 + (dz1-dz0) * (k/(nz-1))**p with p solved so that sum(dz) = top."""
    s = np.arange(nz) / (nz - 1)

    def total(p):
        return float(np.sum(dz0 + (dz1 - dz0) * s ** p))

    lo, hi = 0.05, 20.0
    target = top
    if total(lo) < target:  # cannot reach: use the largest spacing
        return dz0 + (dz1 - dz0) * s ** lo
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if total(mid) > target:
            lo = mid
        else:
            hi = mid
    return dz0 + (dz1 - dz0) * s ** (0.5 * (lo + hi))


@dataclass
class Workload:
    name: str
    dt: float
    fields: dict            # name -> (nj, nk, ni) float64
    hail: bool              # ng/qb passed (hail-aware graupel prognostics)
    steps: int = 1
    meta: dict = field(default_factory=dict)

    @property
    def shape(self):
        return self.fields["p"].shape

    @property
    def ncol(self) -> int:
        nj, _, ni = self.shape
        return nj * ni

    @property
    def nz(self) -> int:
        return self.shape[1]

    def copy(self) -> "Workload":
        return Workload(self.name, self.dt, {k: v.copy() for k, v in self.fields.items()},
                        self.hail, self.steps, dict(self.meta))


def _lognormal(rng, median, sigma, size):
    return median * np.exp(sigma * rng.standard_normal(size))


def _profiles(rng, ncol: int, dz: np.ndarray, *, cloud_base=None, cloud_depth=None,
              clear=None, w=None, hail=False, deep=False):
    """Build one set of column profiles (ncol, nz) from the shared generator."""
    nz = dz.size
    zc = np.cumsum(dz) - 0.5 * dz                        # level-centre heights (m)
    z = np.broadcast_to(zc, (ncol, nz))
    t = np.where(z <= 12000.0, 300.0 - 6.5e-3 * z, 300.0 - 6.5e-3 * 12000.0)
    p = np.empty((ncol, nz))
    p[:, 0] = 100000.0 * np.exp(-G * zc[0] / (RD * t[:, 0]))
    for k in range(1, nz):
        dzh = zc[k] - zc[k - 1]
        tbar = 0.5 * (t[:, k] + t[:, k - 1])
        p[:, k] = p[:, k - 1] * np.exp(-G * dzh / (RD * tbar))
    rh = np.where(z < 10000.0, rng.uniform(0.7, 1.05, (ncol, nz)), 0.3)
    rho = p / (RD * t)
    qc = np.zeros((ncol, nz)); nc = np.zeros((ncol, nz))
    qr = np.zeros((ncol, nz)); nr = np.zeros((ncol, nz))
    qi = np.zeros((ncol, nz)); ni = np.zeros((ncol, nz))
    qs = np.zeros((ncol, nz)); qg = np.zeros((ncol, nz)); ng = np.zeros((ncol, nz))
    qb = np.zeros((ncol, nz))
    if cloud_base is None:
        zb = np.full((ncol, 1), 1000.0)
        zt = np.full((ncol, 1), 4000.0)
        zr = np.full((ncol, 1), 3000.0)
        zi_top = np.full((ncol, 1), 12000.0)
    else:
        zb = cloud_base[:, None]
        zt = (cloud_base + cloud_depth)[:, None]
        zr = np.minimum(zb + 0.5 * (zt - zb), 4150.0)    # rain below mid-cloud, under 0 degC
        zi_top = zt
    in_cloud = (z >= zb) & (z <= zt)
    warm = t > T0
    liq = in_cloud & (t > T0 - 20.0) if cloud_base is not None else in_cloud
    qc = np.where(liq, _lognormal(rng, 0.3e-3, 0.5, (ncol, nz)), 0.0)
    if deep:                                              # supercooled water 0..-20 degC
        sc = in_cloud & (t <= T0) & (t > T0 - 20.0)
        qc = np.where(sc, np.minimum(_lognormal(rng, 0.8e-3, 0.6, (ncol, nz)), 2.0e-3), qc)
    nc = np.where(qc > 0, 1.0e8, 0.0)
    rain = z < zr
    qr = np.where(rain, _lognormal(rng, 0.5e-3, 0.5, (ncol, nz)), 0.0)
    n0 = 8.0e6
    lam = (math.pi * 1000.0 * n0 / (rho * np.maximum(qr, 1e-30))) ** 0.25
    nr = np.where(qr > 0, n0 / (lam * rho), 0.0)
    ice = (~warm) & (z <= zi_top) & ((z >= zb) if cloud_base is not None else True)
    qi = np.where(ice, _lognormal(rng, 0.02e-3, 0.5, (ncol, nz)), 0.0)
    ni = np.where(qi > 0, 1.0e5, 0.0)
    qs = np.where(ice, _lognormal(rng, 0.3e-3, 0.5, (ncol, nz)), 0.0)
    if hail:
        qg = np.where(ice | (in_cloud & warm), np.minimum(_lognormal(rng, 2.0e-3, 0.6, (ncol, nz)), 8.0e-3), 0.0)
        ng = np.where(qg > 0, 10.0 ** rng.uniform(2.0, 5.0, (ncol, nz)), 0.0)
        rhog = rng.uniform(300.0, 900.0, (ncol, nz))
        qb = np.where(qg > 0, 1000.0 * qg / rhog, 0.0)
    else:
        qg = np.where(ice, _lognormal(rng, 0.1e-3, 0.5, (ncol, nz)), 0.0)
        ng = np.where(qg > 0, 1.0e3, 0.0)
        qb = np.where(qg > 0, qg / 500.0 * 1000.0, 0.0)
    if clear is not None:
        m = clear[:, None]
        for a in (qc, nc, qr, nr, qi, ni, qs, qg, ng, qb):
            a[np.broadcast_to(m, a.shape)] = 0.0
    cloudy = in_cloud if clear is None else in_cloud & ~clear[:, None]
    rh = np.where(cloudy, np.maximum(rh, rng.uniform(0.98, 1.02, (ncol, nz))), rh)
    qv = rh * calc_rslf(p, t)
    if w is None:
        w = rng.standard_normal((ncol, nz))
    out = dict(t=t, p=p, w=w, dz=np.broadcast_to(dz, (ncol, nz)).copy(), qv=qv, qc=qc, qr=qr,
               qi=qi, qs=qs, qg=qg, ni=ni, nr=nr, nc=nc,
               nwfa=np.full((ncol, nz), 1.0e9), nifa=np.full((ncol, nz), 1.0e6),
               ng=ng, qb=qb)
    return out


def _to3d(cols: dict, ni: int, nj: int, hail: bool) -> dict:
    out = {}
    for k, v in cols.items():
        if not hail and k in ("ng", "qb"):
            continue
        a = np.ascontiguousarray(v, dtype=np.float64)          # (ncol, nz)
        nz = a.shape[1]
        out[k] = np.ascontiguousarray(a.reshape(nj, ni, nz).transpose(0, 2, 1))
    return out


def uniform_grid(seed: int = 0, ncol: int = 256, nz: int = 60) -> Workload:
    rng = np.random.default_rng(np.random.PCG64(1000 + seed))
    dz = np.full(nz, 250.0)
    cols = _profiles(rng, ncol, dz)
    return Workload("uniform_grid", 20.0, _to3d(cols, ncol, 1, hail=False), hail=False,
                    meta=dict(ncol=ncol, nz=nz, seed=seed))


def _stretched_cols(rng, ncol, nz, hail=False, deep=False):
    dz = stretched_dz(nz)
    clear = rng.uniform(size=ncol) < (0.0 if deep else 0.4)
    base = rng.uniform(300.0, 3000.0, ncol)
    depth = rng.uniform(0.5e3, 12e3, ncol) if not deep else rng.uniform(8e3, 14e3, ncol)
    w = 3.0 * rng.standard_normal((ncol, nz))
    conv = rng.uniform(size=ncol) < 0.05
    w[conv] = rng.uniform(5.0, 20.0, (int(conv.sum()), 1))
    return _profiles(rng, ncol, dz, cloud_base=base, cloud_depth=depth, clear=clear, w=w,
                     hail=hail, deep=deep)


def stretched_grid(seed: int = 0, ni: int = 1024, nj: int = 1024, nz: int = 65,
            steps: int = 10, dt: float = 30.0) -> Workload:
    rng = np.random.default_rng(np.random.PCG64(2000 + seed))
    cols = _stretched_cols(rng, ni * nj, nz)
    return Workload("stretched_grid", dt, _to3d(cols, ni, nj, hail=False), hail=False, steps=steps,
                    meta=dict(ncol=ni * nj, nz=nz, seed=seed))


def hail_convection(seed: int = 0, ni: int = 512, nj: int = 512, nz: int = 65, dt: float = 30.0) -> Workload:
    rng = np.random.default_rng(np.random.PCG64(3000 + seed))
    cols = _stretched_cols(rng, ni * nj, nz, hail=True, deep=True)
    return Workload("hail_convection", dt, _to3d(cols, ni, nj, hail=True), hail=True,
                    meta=dict(ncol=ni * nj, nz=nz, seed=seed))


def stretched_grid_dt60(seed: int = 0, ni: int = 256, nj: int = 256, nz: int = 65) -> Workload:
    wl = stretched_grid(seed=seed + 7, ni=ni, nj=nj, nz=nz, steps=1, dt=60.0)
    wl.name = "stretched_grid_dt60"
    return wl


def domain_set(seed: int = 0, ndom: int = 24, scale: float = 1.0):
    """Domain descriptors (ncol, nz, dt, seed) of the uneven multi-domain batch."""
    rng = np.random.default_rng(np.random.PCG64(5000 + seed))
    out = []
    for d in range(ndom):
        ncol = int(round(10 ** rng.uniform(3.0, math.log10(5e5)) * scale))
        nz = int(rng.choice([50, 65, 90, 128]))
        dt = float(rng.choice([10.0, 20.0, 30.0, 60.0]))
        out.append((max(ncol, 1), nz, dt, int(rng.integers(0, 2**31 - 1))))
    return out


def domain_set_member(ncol: int, nz: int, dt: float, seed: int) -> Workload:
    rng = np.random.default_rng(np.random.PCG64(seed))
    cols = _stretched_cols(rng, ncol, nz)
    return Workload("domain_set", dt, _to3d(cols, ncol, 1, hail=False), hail=False,
                    meta=dict(ncol=ncol, nz=nz, seed=seed))


def column_water(fields: dict) -> np.ndarray:
    """Column-integrated total water (kg m-2) per column from (nj, nk, ni) fields."""
    t, p, dz = fields["t"], fields["p"], fields["dz"]
    qv = np.maximum(1e-10, fields["qv"])
    roverrv = RD / 461.5
    rho = roverrv * p / (RD * t * (qv + roverrv))
    q = qv + fields["qc"] + fields["qr"] + fields["qi"] + fields["qs"] + fields["qg"]
    return np.sum(q * rho * dz, axis=1)


def stretched_grid_torch(seed: int = 0, ni: int = 1024, nj: int = 1024, nz: int = 65,
                  device: str = "cuda", dtype=None, hail: bool = False, deep: bool = False,
                  clear_frac: float = 0.4):
    """The stretched-grid generator evaluated with torch on the GPU (for the 10^6-column
    benchmark, where the NumPy version would spend minutes on the host).  Same recipe
    and distributions as :func:`_profiles` via :func:`_stretched_cols`, drawn from a
    torch generator seeded with 2000 + seed, so the values differ from the NumPy
    stream.  Returns a dict of (nj, nz, ni) tensors."""
    import torch

    dtype = dtype or torch.float32
    g = torch.Generator(device=device)
    g.manual_seed(2000 + seed)
    ncol = ni * nj
    f64 = torch.float64
    dz = torch.as_tensor(stretched_dz(nz), dtype=f64, device=device)

    def U(lo, hi, shape):
        return lo + (hi - lo) * torch.rand(shape, generator=g, device=device, dtype=f64)

    def N(shape):
        return torch.randn(shape, generator=g, device=device, dtype=f64)

    def LN(median, sigma, shape):
        return median * torch.exp(sigma * N(shape))

    zc = torch.cumsum(dz, 0) - 0.5 * dz
    z = zc.expand(ncol, nz)
    t = torch.where(z <= 12000.0, 300.0 - 6.5e-3 * z, torch.full_like(z, 300.0 - 6.5e-3 * 12000.0))
    p = torch.empty((ncol, nz), dtype=f64, device=device)
    p[:, 0] = 100000.0 * torch.exp(-G * zc[0] / (RD * t[:, 0]))
    for k in range(1, nz):
        tbar = 0.5 * (t[:, k] + t[:, k - 1])
        p[:, k] = p[:, k - 1] * torch.exp(-G * (zc[k] - zc[k - 1]) / (RD * tbar))
    rh = torch.where(z < 10000.0, U(0.7, 1.05, (ncol, nz)), torch.full_like(z, 0.3))
    rho = p / (RD * t)
    clear = U(0, 1, (ncol,)) < (0.0 if deep else clear_frac)
    base = U(300.0, 3000.0, (ncol,))
    depth = U(8e3, 14e3, (ncol,)) if deep else U(0.5e3, 12e3, (ncol,))
    w = 3.0 * N((ncol, nz))
    conv = U(0, 1, (ncol,)) < 0.05
    w = torch.where(conv[:, None], U(5.0, 20.0, (ncol, 1)).expand(ncol, nz), w)
    zb, zt = base[:, None], (base + depth)[:, None]
    zr = torch.clamp(zb + 0.5 * (zt - zb), max=4150.0)
    in_cloud = (z >= zb) & (z <= zt)
    warm = t > T0
    liq = in_cloud & (t > T0 - 20.0)
    zero = torch.zeros((ncol, nz), dtype=f64, device=device)
    qc = torch.where(liq, LN(0.3e-3, 0.5, (ncol, nz)), zero)
    if deep:
        sc = in_cloud & (t <= T0) & (t > T0 - 20.0)
        qc = torch.where(sc, torch.clamp(LN(0.8e-3, 0.6, (ncol, nz)), max=2.0e-3), qc)
    nc = torch.where(qc > 0, torch.full_like(qc, 1.0e8), zero)
    qr = torch.where(z < zr, LN(0.5e-3, 0.5, (ncol, nz)), zero)
    lam = (math.pi * 1000.0 * 8.0e6 / (rho * torch.clamp(qr, min=1e-30))) ** 0.25
    nr = torch.where(qr > 0, 8.0e6 / (lam * rho), zero)
    ice = (~warm) & (z <= zt) & (z >= zb)
    qi = torch.where(ice, LN(0.02e-3, 0.5, (ncol, nz)), zero)
    ni_ = torch.where(qi > 0, torch.full_like(qi, 1.0e5), zero)
    qs = torch.where(ice, LN(0.3e-3, 0.5, (ncol, nz)), zero)
    if hail:
        qg = torch.where(ice | (in_cloud & warm), torch.clamp(LN(2.0e-3, 0.6, (ncol, nz)), max=8.0e-3), zero)
        ng = torch.where(qg > 0, 10.0 ** U(2.0, 5.0, (ncol, nz)), zero)
        qb = torch.where(qg > 0, 1000.0 * qg / U(300.0, 900.0, (ncol, nz)), zero)
    else:
        qg = torch.where(ice, LN(0.1e-3, 0.5, (ncol, nz)), zero)
        ng = qb = None
    m = clear[:, None]
    hydro = [qc, nc, qr, nr, qi, ni_, qs, qg] + ([ng, qb] if hail else [])
    hydro = [torch.where(m, zero, a) for a in hydro]
    cloudy = in_cloud & ~m
    rh = torch.where(cloudy, torch.maximum(rh, U(0.98, 1.02, (ncol, nz))), rh)
    x = torch.clamp(t - 273.16, min=-80.0)
    c = [.611583699E03, .444606896E02, .143177157e01, .264224321e-1, .299291081e-3,
         .203154182e-5, .702620698e-8, .379534310e-11, -.321582393e-13]
    esl = torch.full_like(x, c[8])
    for ci in c[7::-1]:
        esl = ci + x * esl
    esl = torch.minimum(esl, p * 0.15)
    qv = rh * 0.622 * esl / (p - esl)
    names = ["qc", "nc", "qr", "nr", "qi", "ni", "qs", "qg"] + (["ng", "qb"] if hail else [])
    cols = dict(zip(names, hydro))
    cols.update(t=t, p=p, w=w, dz=dz.expand(ncol, nz), qv=qv,
                nwfa=torch.full((ncol, nz), 1.0e9, dtype=f64, device=device),
                nifa=torch.full((ncol, nz), 1.0e6, dtype=f64, device=device))
    out = {}
    for k, v in cols.items():
        out[k] = v.reshape(nj, ni, nz).permute(0, 2, 1).contiguous().to(dtype)
        del v
    return out
