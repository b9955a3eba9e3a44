"""Python mirror of the reference's CNS level over the C ABI.

`CNSLevel` keeps the call surface of `class CNS : AmrLevel` for one level
(src/CNS.h:10-166): `compute_rhs(S, dSdt)` (src/tim/CNS_advance.cpp:186-427),
`advance(time, dt)` (src/tim/CNS_advance.cpp:14-183), `est_time_step()`
(src/CNS.cpp:380-395), `compute_initial_dt` / `compute_new_dt`
(src/CNS.cpp:282-377) and `print_total`'s conserved totals
(src/CNS.cpp:532-621).  Every numerical step runs in the CUDA library; this
module only sequences calls and owns the device buffers (torch tensors).
"""
from __future__ import annotations

import numpy as np
import torch

from . import capi
from .problems import NCONS, NGHOST


class CNSLevel:
    """One single-box level: state S1 (U^n) plus two work buffers, all ghosted."""

    def __init__(self, scheme, closures, U0, dx, bc_lo=(-1, -1, -1), bc_hi=(-1, -1, -1), lo=(0, 0, 0),
                 order_rk=3, stages_rk=3, device=0, bcnormal=None):
        """`bcnormal`, if given, fills the ghost cells beyond the ext_dir
        sides (codes 1, 6) after the library's fill, as the problem's
        bcnormal does in cns_bcfill (src/set/bcs.cpp:30-100): either a
        callable `bcnormal(t)` on the ghosted state tensor written with torch
        operations (differentiated by torch autograd in the adjoint), or a
        problems.BCNormal that the library evaluates on the device beyond
        code-6 y sides (the adjoint differentiates the same formula written
        in torch).  Without it those ghost cells keep the values of U0."""
        self.scheme, self.closures = scheme, closures
        self.bcnormal = bcnormal
        self.h = capi.Handle(scheme, closures, device)
        self.dev = torch.device("cuda", device)
        self.dx = tuple(float(v) for v in dx)
        self.dxinv = tuple(1.0 / v for v in self.dx)
        self.lo = tuple(lo)
        self.bc_lo, self.bc_hi = tuple(bc_lo), tuple(bc_hi)
        self.order_rk, self.stages_rk = order_rk, stages_rk
        U0 = np.ascontiguousarray(U0, dtype=np.float64)
        self.shape = U0.shape
        self.n = tuple(s - 2 * NGHOST for s in U0.shape[1:][::-1])  # (nx, ny, nz)
        # all three buffers start as U0: ghost cells beyond ext_dir sides
        # (codes 1, 6) are the caller's and keep these values
        first = torch.from_numpy(U0).to(self.dev)
        self.bufs = [first, first.clone(), first.clone()]
        self.h.set_domain(self.lo, self.n, self.bc_lo, self.bc_hi)
        self.cur = 0
        self.time = 0.0
        self.dt_dev = torch.zeros(1, dtype=torch.float64, device=self.dev)

    # ------------------------------------------------------------ state --
    @property
    def S(self):
        return self.bufs[self.cur]

    def state_host(self):
        return self.S.cpu().numpy()

    def valid(self, t=None):
        t = self.S if t is None else t
        g = NGHOST
        return t[:, g:-g, g:-g, g:-g]

    # ------------------------------------------------------------ calls --
    def fill_patch(self, t, stream=None):
        """Ghost fill of `t` in place (single-level FillPatch): periodic
        images and physical BCs, then the ext_dir ghosts by `bcnormal`."""
        if self.bcnormal is None:
            capi.fill_halo_box(t, self.bc_lo, self.bc_hi, self.lo, stream)
        elif callable(self.bcnormal):
            capi.fill_halo_box(t, self.bc_lo, self.bc_hi, self.lo, stream)
            self.bcnormal(t)
        else:
            capi.fill_halo_box_bcnormal(t, self.bc_lo, self.bc_hi, self.closures, self.bcnormal, self.lo, stream)

    def has_ext_dir(self):
        return any(b in (1, 6) for b in self.bc_lo + self.bc_hi)

    def bcnormal_vjp(self, t, gbar):
        """Reverse of `bcnormal` on the ghost-filled `t`: the cotangents of the
        ghost cells it wrote (in the ghosted `gbar`) go to the cells it read.
        Returns the folded ghosted cotangent.  Without a bcnormal the ext_dir
        ghosts are constants and their cotangents are simply not used."""
        if self.bcnormal is None:
            return gbar
        fill = self.bcnormal if callable(self.bcnormal) else _isothermal_wall_torch(self.bcnormal, self.closures,
                                                                                   self.bc_lo, self.bc_hi, self.lo)
        with torch.enable_grad():
            x = t.detach().clone().requires_grad_(True)
            y = x.clone()
            fill(y)
            (gx,) = torch.autograd.grad(y, x, grad_outputs=gbar)
        return gx

    def compute_rhs(self, S, dSdt, stream=None):
        """CNS::compute_rhs for the box: S ghost-filled, dSdt valid-only."""
        self.h.rhs_box(S, self.dxinv, dSdt, self.lo, stream)
        return dSdt

    def advance(self, time, dt, stream=None):
        """CNS::advance: one RK step of order_rk / stages_rk; returns dt."""
        progs = capi.rk_program(self.order_rk, self.stages_rk, dt)
        s1 = self.cur
        work = [i for i in range(3) if i != s1]
        cur = s1
        which = 0
        for p in progs:
            src = s1 if p.src_state == 0 else cur
            out = work[which]
            if out == src:
                which ^= 1
                out = work[which]
            self.fill_patch(self.bufs[src], stream)
            self.h.rk_stage_box(p, self.bufs[src], self.bufs[s1], self.bufs[out], self.dxinv, self.lo, stream)
            cur = out
            which ^= 1
        self.cur = cur
        self.time = time + dt
        return dt

    def est_time_step(self, cfl, stream=None):
        """CNS::estTimeStep: cfl * min dx/(|u|+c) (host-synchronising)."""
        self.h.est_timestep(self.S, self.dx, cfl, self.dt_dev, self.lo, stream)
        return float(self.dt_dev.item())

    def compute_initial_dt(self, cfl):
        """CNS::computeInitialDt for a single level with dynamic dt."""
        return self.est_time_step(cfl)

    def compute_new_dt(self, cfl, dt_old, stop_time, change_max=1.1):
        """CNS::computeNewDt (src/CNS.cpp:319-377): growth capped at 1.1x and
        the last step clamped to stop_time."""
        dt_min = min(self.est_time_step(cfl), change_max * dt_old)
        dt0 = dt_min
        eps = 0.001 * dt0
        if stop_time >= 0.0 and self.time + dt0 > stop_time - eps:
            dt0 = stop_time - self.time
        return dt0

    def totals(self):
        """Conserved totals as CNS::printTotal reports them: sum over valid
        cells times the domain volume (src/CNS.cpp:538-541)."""
        vol = 1.0
        for d in range(3):
            vol *= self.n[d] * self.dx[d]
        v = self.valid()
        return (v.reshape(NCONS, -1).sum(dim=1) * vol).cpu().numpy()

    def print_total(self, dt):
        """What CNS::printTotal reports (src/CNS.cpp:532-611): the conserved
        totals, the min/max of each primitive and the convective CFL table
        for time step dt, from the current state; a dict keyed as
        capi.PRIM_STATS_KEYS plus 'totals'."""
        out = torch.empty(21, dtype=torch.float64, device=self.dev)
        self.h.prim_stats(self.S, self.dx, dt, out, self.lo)
        d = dict(zip(capi.PRIM_STATS_KEYS, out.cpu().numpy().tolist()))
        d["totals"] = self.totals().tolist()
        return d

    def write_plotfile(self, path, step=0, derive=None, prob_lo=(0.0, 0.0, 0.0)):
        """CNS::writePlotFile of this single-box level (src/CNS.cpp:644-874):
        the state and the derived quantities `derive` (default all of
        pressure, temperature, x/y/z_velocity) at the current time."""
        from . import plotfile
        box = (self.lo, self.n)
        return plotfile.write_plotfile(path, [box], [self.S], self.closures, self.dx, prob_lo, box, self.time, step,
                                       plotfile.DERIVED_NAMES if derive is None else derive)

    def run(self, stop_time, max_step, cfl=None, dt=None):
        """The reference's main loop (src/main.cpp:66-75) for one level."""
        steps = 0
        if cfl is not None:
            dt_cur = self.compute_initial_dt(cfl)
        else:
            dt_cur = dt
        while steps < max_step and self.time < stop_time:
            self.advance(self.time, dt_cur)
            steps += 1
            if cfl is not None:
                dt_cur = self.compute_new_dt(cfl, dt_cur, stop_time)
        return steps


def _isothermal_wall_torch(bn, cl, bc_lo, bc_hi, lo):
    """The device bcnormal of kind 1 (the channel problem's isothermal
    no-slip wall beyond code-6 y sides) as torch operations on the ghosted
    state, for differentiating it by autograd in the adjoint: the same
    formula, with the floor max(T, Tmin) passing the derivative along the
    branch taken."""
    g = NGHOST

    def fill(t):
        ny = t.shape[2] - 2 * g
        for side in (0, 1):
            if (bc_hi if side else bc_lo)[1] != 6:
                continue
            jf = g if side == 0 else g + ny - 1  # tensor row of the first interior cell
            s = t[:, :, jf, :].clone()
            rho = s[0]
            ue, ve, we = -s[1] / rho, -s[2] / rho, -s[3] / rho
            eint = (s[4] - 0.5 * (s[1] * s[1] + s[2] * s[2] + s[3] * s[3]) / rho) / rho
            p = (cl.gamma - 1.0) * rho * eint
            tint = p / (cl.Rspec * rho)
            jdom = lo[1] if side == 0 else lo[1] + ny - 1  # index of the first interior row
            for gi in range(1, g + 1):
                j = jdom - gi if side == 0 else jdom + gi
                x = bn.prob_lo[1] + (j + 0.5) * bn.dx[1]
                if side == 0:
                    dratio = (bn.prob_lo[1] - x) / ((jdom + 0.5) * bn.dx[1] - bn.prob_lo[1])
                else:
                    dratio = (x - bn.prob_hi[1]) / (bn.prob_hi[1] - (jdom + 0.5) * bn.dx[1])
                te = torch.clamp_min(bn.Tw + dratio * (bn.Tw - tint), bn.Tmin)
                re = p / (cl.Rspec * te)
                ekin = 0.5 * (ue * ue + ve * ve + we * we)
                row = jf - gi if side == 0 else jf + gi
                t[0, :, row, :] = re
                t[1, :, row, :] = re * ue
                t[2, :, row, :] = re * ve
                t[3, :, row, :] = re * we
                t[4, :, row, :] = re * (p / (re * (cl.gamma - 1.0)) + ekin)

    return fill
