"""Adjoint of the RHS and of the RK step, over the C ABI.

* `RHSFunction` / `StepFunction`: torch.autograd.Function wrappers whose
  backward passes call the hand-written VJP kernels (amrs_rhs_vjp_box,
  amrs_rk_stage_vjp_box).  Gradients flow to the state; the viscosity
  gradient is returned through `CheckpointedAdjoint`.
* `CheckpointedAdjoint`: multi-step adjoint of `CNSLevel.advance` that keeps
  every k-th state, recomputes the RK stages of a segment on the way back and
  runs the stage VJPs in reverse (cotangents of S1 and of each stage input
  follow the stage programs of src/tim/CNS_advance.cpp:51-166).

The reference has no adjoint (its lib/autodiff submodule is empty); the
checks are central finite differences and a dot-product test against the
CPU oracle's dual-number JVP.
"""
from __future__ import annotations

import torch

from . import capi
from .problems import NGHOST


def _valid(t):
    g = NGHOST
    return t[:, g:-g, g:-g, g:-g]


class RHSFunction(torch.autograd.Function):
    """dSdt = RHS(U) for one ghost-filled box (KEEP + viscous)."""

    @staticmethod
    def forward(ctx, U, handle, dxinv, lo):
        U = U.contiguous()
        n = tuple(s - 2 * NGHOST for s in U.shape[1:])
        out = torch.empty((U.shape[0],) + n, dtype=U.dtype, device=U.device)
        handle.rhs_box(U, dxinv, out, lo)
        ctx.save_for_backward(U)
        ctx.handle, ctx.dxinv, ctx.lo = handle, dxinv, lo
        return out

    @staticmethod
    def backward(ctx, gout):
        (U,) = ctx.saved_tensors
        ubar = torch.empty_like(U)
        ctx.handle.rhs_vjp_box(U, gout.contiguous(), ubar, ctx.dxinv, ctx.lo)
        return ubar, None, None, None


class StepFunction(torch.autograd.Function):
    """U^{n+1} (valid cells) from U^n (valid cells) by one RK step of a
    single-box level with the level's boundary codes."""

    @staticmethod
    def forward(ctx, Uv, level, dt):
        g = NGHOST
        S1 = torch.zeros(level.shape, dtype=torch.float64, device=level.dev)
        S1[:, g:-g, g:-g, g:-g] = Uv
        stages, out = _forward_step(level, S1, dt)
        ctx.level, ctx.dt, ctx.stages = level, dt, stages
        return _valid(out).clone()

    @staticmethod
    def backward(ctx, wbar):
        s1bar, _ = _step_vjp(ctx.level, ctx.stages, ctx.dt, wbar.contiguous())
        return s1bar, None, None


def _forward_step(level, S1, dt):
    """One RK step from the ghosted S1; returns the ghost-filled stage inputs
    (as used by each stage) and the result (ghosted buffer)."""
    progs = capi.rk_program(level.order_rk, level.stages_rk, dt)
    stages = []
    cur = None
    for p in progs:
        src = S1 if p.src_state == 0 else cur
        inp = src.clone()
        level.fill_patch(inp)
        out = torch.empty_like(S1)
        level.h.rk_stage_box(p, inp, S1, out, level.dxinv, level.lo)
        stages.append((p, inp))
        cur = out
    return stages, cur


def _step_vjp(level, stages, dt, wbar, param_bar=None):
    """Cotangent of U^n (valid) from the cotangent of U^{n+1} (valid)."""
    ns = len(stages)
    outbar = [None] * ns
    outbar[-1] = wbar
    s1bar = torch.zeros_like(wbar)
    for s in range(ns - 1, -1, -1):
        p, inp = stages[s]
        if outbar[s] is None:
            outbar[s] = torch.zeros_like(wbar)
        if level.has_ext_dir():
            # ghosts beyond ext_dir sides came from bcnormal after the
            # library's fill: reverse bcnormal first, then the library's fill
            ug = torch.empty_like(inp)
            level.h.rk_stage_vjp_box_ghosted(p, inp, outbar[s], s1bar, ug, level.dxinv, level.lo,
                                             param_bar=param_bar)
            ug = level.bcnormal_vjp(inp, ug)
            capi.fill_halo_box_adjoint(ug, level.bc_lo, level.bc_hi, level.lo)
            inbar = _valid(ug).contiguous()
        else:
            inbar = torch.zeros_like(wbar)
            level.h.rk_stage_vjp_box(p, level.bc_lo, level.bc_hi, inp, outbar[s], s1bar, inbar, level.dxinv,
                                     level.lo, param_bar=param_bar)
        if p.src_state == 0:
            s1bar += inbar
        else:
            if outbar[s - 1] is None:
                outbar[s - 1] = torch.zeros_like(wbar)
            outbar[s - 1] += inbar
    return s1bar, param_bar


class CheckpointedAdjoint:
    """Reverse-mode sensitivity of a scalar of the final state after N steps,
    storing every k-th state (k = `every`) and recomputing in between.  The
    last segment's stage inputs are kept from the forward pass, so it is not
    recomputed; with every >= N nothing is (all stage inputs are kept: three
    ghosted states per step, e.g. 8 GB for 200 steps of a 64^3 box)."""

    def __init__(self, level, every=20):
        self.level = level
        self.every = every

    def run(self, U0v, nsteps, dt, objective_grad):
        """Returns (objective input state gradient on valid cells, param_bar
        [d/d visc_ref, d/d cond_ref], final state valid).  `objective_grad`
        maps the final valid state to its gradient."""
        lev = self.level
        g = NGHOST
        ckpt = {}
        S = torch.zeros(lev.shape, dtype=torch.float64, device=lev.dev)
        S[:, g:-g, g:-g, g:-g] = U0v
        last = ((nsteps - 1) // self.every) * self.every  # start of the last segment
        kept = []
        for n in range(nsteps):
            if n % self.every == 0:
                ckpt[n] = _valid(S).clone()
            stages, out = _forward_step(lev, S, dt)
            if n >= last:
                kept.append(stages)
            S = out
        final = _valid(S).clone()
        wbar = objective_grad(final)
        pbar = torch.zeros(2, dtype=torch.float64, device=lev.dev)
        seg_starts = sorted(ckpt)
        for a in reversed(seg_starts):
            b = min(a + self.every, nsteps)
            if a == last:
                saved = kept
            else:
                # recompute the segment, keeping each step's stage inputs
                S = torch.zeros(lev.shape, dtype=torch.float64, device=lev.dev)
                S[:, g:-g, g:-g, g:-g] = ckpt[a]
                saved = []
                for n in range(a, b):
                    stages, out = _forward_step(lev, S, dt)
                    saved.append(stages)
                    S = out
            for n in range(b - 1, a - 1, -1):
                wbar, _ = _step_vjp(lev, saved[n - a], dt, wbar, param_bar=pbar)
        return wbar, pbar, final


def kinetic_energy(Uv):
    """KE = <0.5 |m|^2 / rho> over the valid cells."""
    return (0.5 * (Uv[1] ** 2 + Uv[2] ** 2 + Uv[3] ** 2) / Uv[0]).mean()


def kinetic_energy_grad(Uv):
    n = Uv[0].numel()
    g = torch.zeros_like(Uv)
    r = Uv[0]
    g[0] = -0.5 * (Uv[1] ** 2 + Uv[2] ** 2 + Uv[3] ** 2) / (r * r) / n
    g[1] = Uv[1] / r / n
    g[2] = Uv[2] / r / n
    g[3] = Uv[3] / r / n
    return g
