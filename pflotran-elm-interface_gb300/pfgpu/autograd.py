"""torch.autograd wrapper of the operator-split step.

RStepFunction.apply(engine, state, dt, dlogK_sec, dlogK_mnrl, dlnk, lnarea, total0)
returns the final totals (ncomp, ncells) of one RStep per cell, as a
differentiable function of
  dlogK_sec (nsec), dlogK_mnrl (nmnrl): shifts of every logK (all temperatures)
  dlnk (nmnrl):                          ln of the rate-constant multipliers
  lnarea (nmnrl, ncells):                ln of every cell's mineral area
  total0 (ncomp, ncells):                the transported totals entering the step
The backward pass calls pf_adjoint, which recomputes the forward solve from the
saved inputs (no Newton iterate is stored) and solves the implicit-function-
theorem adjoint per substep with the converged LU of the exact Jacobian.
"""
from __future__ import annotations

import torch

from .network import CellState

STATE_OUT = ("total", "pri_molal", "pri_act_coef", "sec_act_coef", "sec_molal", "mnrl_volfrac",
             "mnrl_rate", "status", "newton_its", "num_substeps")


def _prepared(engine, state, dlogK_sec, dlogK_mnrl, dlnk, lnarea, total0):
    st = state.copy()
    st.a["total"].copy_(total0.detach())
    if engine.net.nmnrl:
        st.a["mnrl_area"].copy_(torch.exp(lnarea.detach()))
    engine.shift_parameters(dlogK_sec.detach().cpu().numpy() if engine.net.nsec else None,
                            dlogK_mnrl.detach().cpu().numpy() if engine.net.nmnrl else None,
                            dlnk.detach().cpu().numpy() if engine.net.nmnrl else None)
    return st


class RStepFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, engine, state: CellState, dt, dlogK_sec, dlogK_mnrl, dlnk, lnarea, total0):
        st = _prepared(engine, state, dlogK_sec, dlogK_mnrl, dlnk, lnarea, total0)
        try:
            engine.rstep(st, dt, stats=False)
        finally:
            engine.shift_parameters()
        ctx.engine, ctx.state, ctx.dt = engine, state, dt
        ctx.save_for_backward(dlogK_sec, dlogK_mnrl, dlnk, lnarea, total0)
        ctx.mark_non_differentiable()
        return st.a["total"].clone()

    @staticmethod
    def backward(ctx, grad_total):
        dlogK_sec, dlogK_mnrl, dlnk, lnarea, total0 = ctx.saved_tensors
        eng = ctx.engine
        st = _prepared(eng, ctx.state, dlogK_sec, dlogK_mnrl, dlnk, lnarea, total0)
        try:
            g = eng.adjoint(st, ctx.dt, dL_dtotal=grad_total.contiguous())
        finally:
            eng.shift_parameters()
        return (None, None, None, g["dL_dlogK_sec"], g["dL_dlogK_mnrl"], g["dL_dlnk"], g["dL_dlnarea"],
                g["dL_dtotal0"])


def rstep_totals(engine, state, dt, dlogK_sec, dlogK_mnrl, dlnk, lnarea, total0):
    return RStepFunction.apply(engine, state, dt, dlogK_sec, dlogK_mnrl, dlnk, lnarea, total0)
