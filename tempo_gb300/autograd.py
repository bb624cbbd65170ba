"""The column step as a differentiable torch operation.

``tempo_step(ctx, fields, dt, itimestep)`` runs one step of the TEMPO column
microphysics on CUDA tensors and returns the new state and the diagnostics that a cost
function usually needs (surface precipitation of rain, ice, snow and graupel, and the
10-cm reflectivity).  Its backward pass is the library's hand-written adjoint
(``tempo_adjoint_dev_c``): branches, clips and table bins are those of the forward
trajectory, sedimentation is reversed substep by substep from checkpoints.

float64 tensors give the FP64 step and its exact adjoint; float32 tensors the
all-FP32 step and its adjoint.  Differentiated inputs: t (or th), qv, qc, nc, qr, nr,
qi, ni, qs, qg and, hail-aware, ng and qb.  Pressure, vertical velocity, layer depths,
Exner function, aerosols and land flags are constants of the step.
"""
from __future__ import annotations

from typing import Optional

import torch

from . import DIFF_FIELDS, TempoCfgs, TempoContext

STATE = ("t", "th", "qv", "qc", "nc", "qr", "nr", "qi", "ni", "qs", "qg", "ng", "qb", "nwfa", "nifa")
CONST = ("pii", "p", "w", "dz", "land_input")
PRECIP = ("rain_precip", "ice_liquid_equiv_precip", "snow_liquid_equiv_precip",
          "graupel_liquid_equiv_precip")
OUT_DIAGS = PRECIP + ("refl10cm",)


class _TempoStepFn(torch.autograd.Function):
    @staticmethod
    def forward(fctx, tctx: TempoContext, cfgs: Optional[TempoCfgs], dt: float, itimestep: int,
                names: tuple, consts: dict, *tensors):
        fields = dict(zip(names, tensors))
        fields.update(consts)
        new = {k: v.detach().clone() for k, v in fields.items() if k in STATE}
        run = dict(consts)
        run.update(new)
        p = fields["p"]
        nj, nk, ni = p.shape
        diags = {n: torch.zeros((nj, ni), dtype=p.dtype, device=p.device) for n in PRECIP}
        diags["refl10cm"] = torch.zeros((nj, nk, ni), dtype=p.dtype, device=p.device)
        # the forward value of the all-FP32 / FP64 step: the tangent-linear call with no
        # tangent advances the state exactly like the step the adjoint differentiates
        tctx.tl_device(run, {}, dt, itimestep, diags=diags, cfgs=cfgs)
        fctx.tctx, fctx.cfgs, fctx.dt, fctx.itimestep = tctx, cfgs, dt, itimestep
        fctx.names, fctx.consts = names, consts
        fctx.save_for_backward(*tensors)
        outs = tuple(new[n] for n in names) + tuple(diags[n] for n in OUT_DIAGS)
        return outs

    @staticmethod
    def backward(fctx, *grads):
        tensors = fctx.saved_tensors
        names = fctx.names
        fields = dict(zip(names, tensors))
        fields.update(fctx.consts)
        n = len(names)
        lam = {}
        for name, g, x in zip(names, grads[:n], tensors):
            if name in DIFF_FIELDS:
                lam[name] = (g if g is not None else torch.zeros_like(x)).detach().clone().contiguous()
        lam_diags = {}
        for name, g in zip(OUT_DIAGS, grads[n:]):
            if g is not None:
                lam_diags[name] = g.detach().contiguous()
        fctx.tctx.adjoint_device(fields, lam, fctx.dt, fctx.itimestep, lam_diags=lam_diags,
                                 cfgs=fctx.cfgs)
        grads_in = tuple(lam.get(name) if name in DIFF_FIELDS else None for name in names)
        return (None, None, None, None, None, None) + grads_in


def tempo_step(tctx: TempoContext, fields: dict, dt: float, itimestep: int,
               cfgs: Optional[TempoCfgs] = None):
    """One differentiable step: returns (new state dict, diagnostics dict)."""
    names = tuple(n for n in STATE if fields.get(n) is not None)
    consts = {n: fields[n] for n in CONST if fields.get(n) is not None}
    outs = _TempoStepFn.apply(tctx, cfgs, dt, itimestep, names, consts,
                              *[fields[n].contiguous() for n in names])
    new = dict(zip(names, outs[:len(names)]))
    diags = dict(zip(OUT_DIAGS, outs[len(names):]))
    return new, diags


def cost_precip_reflectivity(diags: dict, dz: torch.Tensor, weight: float = 1e-3) -> torch.Tensor:
    """J = sum of surface precipitation (rain, ice, snow, graupel) + weight * sum over
    levels of the linear 10-cm reflectivity times the layer depth (Ze in mm^6 m^-3 from
    the dBZ diagnostic, diags:94-119)."""
    j = sum(diags[n].sum() for n in PRECIP)
    ze = torch.pow(10.0, diags["refl10cm"] / 10.0)
    return j + weight * (ze * dz).sum()
