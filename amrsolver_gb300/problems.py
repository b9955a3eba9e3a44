"""Closures, scheme switches and seeded synthetic initial states.

The parameter names follow the reference's problem plugin and run-time keys:
`Closures` mirrors `closures_derived_t<Visc, Cond, calorifically_perfect_gas_t>`
(src/cls/Closures.h:72-182) and `Scheme` mirrors the `cns.*` keys read by
`CNS::read_params` (src/CNS.cpp:85-136).

Every generator returns host float64 arrays in the Array4 layout used across
this package: (ncomp, nz+2g, ny+2g, nx+2g), component-major with i fastest
and the ghost cells included.  The same bytes feed the GPU path and the CPU
oracle, so transcendental functions appear only here.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

NCONS = 5
NPRIM = 6
NGHOST = 3
URHO, UMX, UMY, UMZ, UET = range(5)


@dataclasses.dataclass
class Closures:
    """Ideal gas + transport closures (src/cls/Closures.h:72-182).

    visc_law / cond_law: 0 = constant (visc_const_t / cond_const_t),
    1 = Sutherland (visc_suth_t / cond_suth_t).
    """
    gamma: float = 1.40
    cv: float = 0.0
    cp: float = 0.0
    Rspec: float = 0.0
    visc_law: int = 1
    cond_law: int = 1
    visc_ref: float = 1.458e-6
    Tvisc_ref: float = 110.4
    cond_ref: float = 2.495e-3
    Tcond_ref: float = 194.0
    Cshock: float = 1.0
    Cdamp: float = 0.01

    @staticmethod
    def ideal_gas(gamma=1.40, mw=28.96e-3, Ru=8.31451, **kw):
        """calorifically_perfect_gas_t initialisers (src/cls/Closures.h:75-81)."""
        cv = Ru / (mw * (gamma - 1.0))
        cp = gamma * Ru / (mw * (gamma - 1.0))
        Rspec = Ru / mw
        return Closures(gamma=gamma, cv=cv, cp=cp, Rspec=Rspec, **kw)

    @staticmethod
    def air_sutherland():
        """The Sods example's closures: Sutherland viscosity and conductivity."""
        return Closures.ideal_gas(visc_law=1, cond_law=1, visc_ref=1.458e-6, Tvisc_ref=110.4,
                                  cond_ref=2.495e-3, Tcond_ref=194.0)

    @staticmethod
    def nondimensional(mu, prandtl=0.71, gamma=1.40):
        """R = 1 gas (T = p/rho) with constant viscosity mu and k = cp*mu/Pr."""
        c = Closures.ideal_gas(gamma=gamma, mw=1.0, Ru=1.0, visc_law=0, cond_law=0)
        c.visc_ref = float(mu)
        c.cond_ref = float(c.cp * mu / prandtl)
        return c


@dataclasses.dataclass
class Scheme:
    """cns.* switches: flux_euler 0 = MUSCL/Riemann, 1 = KEEP, 2 = WENO5-JS LLF
    (any value other than 1 and 2 takes the Riemann path, as in the
    reference).

    riemann_weno (not a reference switch): on the Riemann path, 0 (default)
    the reference's MUSCL states, 1 WENO5-Riemann (an extension:
    WENO5-reconstructed primitive states fed to the two-shock solver).

    weno_fast (not a reference switch): 0 (default) evaluates WENO5 in the
    reference's operation order (bit-identical results); 1 forms the weights
    over a common denominator (faster, rounding differences only).

    rhs_source: cns.rhs_source; the source is the problem's user_source,
    here a constant body force per unit mass `body_force` (the channel
    problem's, exm/Channel/prob.h:189-193, is (fx, 0, 0)).
    """
    rhs_euler: int = 1
    rhs_visc: int = 1
    flux_euler: int = 1
    order_keep: int = 4
    art_diss: int = 0
    weno_fast: int = 0
    riemann_weno: int = 0
    rhs_source: int = 0
    body_force: tuple = (0.0, 0.0, 0.0)


@dataclasses.dataclass
class BCNormal:
    """A problem bcnormal the library evaluates on the device beyond code-6
    y sides (amrs_bcnormal).  kind 1: the channel problem's isothermal
    no-slip wall (exm/Channel/prob.h:158-186) with wall temperature Tw and
    the floor Tmin (50 there); prob_lo / prob_hi / dx: the geometry, as
    cns_bcfill computes the ghost/first-cell distance ratio from them."""
    Tw: float
    prob_lo: tuple
    prob_hi: tuple
    dx: tuple
    Tmin: float = 0.0
    kind: int = 1

    @staticmethod
    def channel_wall(Tw, n, dx, prob_lo=(0.0, 0.0, 0.0), Tmin=0.0):
        """Geometry from the cell counts n and sizes dx (prob_hi = prob_lo + n dx)."""
        hi = tuple(float(prob_lo[d]) + n[d] * float(dx[d]) for d in range(3))
        return BCNormal(float(Tw), tuple(float(v) for v in prob_lo), hi, tuple(float(v) for v in dx), float(Tmin))


@dataclasses.dataclass
class BoxSpec:
    lo: tuple
    hi: tuple

    @property
    def shape(self):
        return tuple(self.hi[d] - self.lo[d] + 1 for d in range(3))

    @property
    def cells(self):
        s = self.shape
        return s[0] * s[1] * s[2]


def ghosted_shape(n, g=NGHOST, ncomp=NCONS):
    nx, ny, nz = n
    return (ncomp, nz + 2 * g, ny + 2 * g, nx + 2 * g)


def valid(U, g=NGHOST):
    """View of the valid cells of a ghosted field."""
    return U[:, g:-g, g:-g, g:-g] if g > 0 else U


def prims_to_cons(rho, u, v, w, p, gamma):
    U = np.empty((NCONS,) + rho.shape)
    U[URHO] = rho
    U[UMX] = rho * u
    U[UMY] = rho * v
    U[UMZ] = rho * w
    U[UET] = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v + w * w)
    return U


def cell_centres(n, dx, lo=(0, 0, 0), origin=(0.0, 0.0, 0.0), g=NGHOST):
    """Ghost-inclusive cell-centre coordinates (z, y, x order meshgrid)."""
    ax = [origin[d] + (np.arange(lo[d] - g, lo[d] + n[d] + g) + 0.5) * dx[d] for d in range(3)]
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    return X, Y, Z


# ----------------------------------------------------------------- configs --
def tgv(n=128, mach=0.1, gamma=1.4, g=NGHOST, amp=1.0):
    """Taylor-Green vortex on the periodic box [0,2pi]^3, rho = 1.

    u = V0 sin x cos y cos z, v = -V0 cos x sin y cos z, w = 0,
    p = 1/(gamma M^2) + V0^2 (cos 2x + cos 2y)(cos 2z + 2)/16, V0 = amp.
    Ghost cells hold the periodic continuation.
    """
    nn = (n, n, n)
    h = 2.0 * math.pi / n
    X, Y, Z = cell_centres(nn, (h, h, h), g=g)
    rho = np.ones_like(X)
    u = amp * np.sin(X) * np.cos(Y) * np.cos(Z)
    v = -amp * np.cos(X) * np.sin(Y) * np.cos(Z)
    w = np.zeros_like(X)
    p = 1.0 / (gamma * mach * mach) + amp * amp * (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2.0) / 16.0
    return prims_to_cons(rho, u, v, w, p, gamma), (h, h, h)


def sod(nx=256, ny=8, nz=8, gamma=1.4, g=NGHOST):
    """Sod tube on x in [0,1] (cube cells): (rho,p) = (1,1) left, (0.125,0.1) right."""
    h = 1.0 / nx
    X, Y, Z = cell_centres((nx, ny, nz), (h, h, h), g=g)
    left = X < 0.5
    rho = np.where(left, 1.0, 0.125)
    p = np.where(left, 1.0, 0.1)
    z = np.zeros_like(X)
    return prims_to_cons(rho, z, z, z, p, gamma), (h, h, h)


BATCH_EDGES = (8, 16, 24, 32, 48, 64)


def batched_boxes(nboxes=512, seed=1234, h=1.0 / 64, gamma=1.4, g=NGHOST, edges=BATCH_EDGES):
    """Synthetic AMR level: disjoint boxes with seeded edge lengths per dimension.

    rho = 1 + 0.2 exp(-|x-c|^2/0.01) (random centre c inside each box),
    velocity components ~ U(-0.1, 0.1) per cell (ghosts drawn from the same
    field), p = 1/gamma.  Boxes sit side by side along x in index space.
    Returns (list of BoxSpec, list of ghosted arrays, dx).
    """
    rng = np.random.default_rng(seed)
    specs, fields = [], []
    xoff = 0
    for _ in range(nboxes):
        n = tuple(int(e) for e in rng.choice(edges, size=3))
        lo = (xoff, 0, 0)
        hi = (xoff + n[0] - 1, n[1] - 1, n[2] - 1)
        xoff += n[0] + 2 * g + 8
        X, Y, Z = cell_centres(n, (h, h, h), lo=lo, g=g)
        c = [(lo[d] + rng.random() * n[d]) * h for d in range(3)]
        r2 = (X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2
        rho = 1.0 + 0.2 * np.exp(-r2 / 0.01)
        u = rng.uniform(-0.1, 0.1, X.shape)
        v = rng.uniform(-0.1, 0.1, X.shape)
        w = rng.uniform(-0.1, 0.1, X.shape)
        p = np.full_like(X, 1.0 / gamma)
        specs.append(BoxSpec(lo, hi))
        fields.append(prims_to_cons(rho, u, v, w, p, gamma))
    return specs, fields, (h, h, h)


def ensemble_members(nmembers=64, n=48, seed=4321):
    """Parameters of the TGV ensemble: M ~ U(0.05,0.3), Re ~ U(200,3200)."""
    rng = np.random.default_rng(seed)
    mach = rng.uniform(0.05, 0.3, nmembers)
    re = rng.uniform(200.0, 3200.0, nmembers)
    return [(float(m), float(r)) for m, r in zip(mach, re)]


def random_turbulence(n=256, mach_t=0.6, k0=4.0, seed=99, gamma=1.4, g=NGHOST):
    """Solenoidal random-phase velocity with E(k) ~ k^4 exp(-2 (k/k0)^2).

    rho = 1, p = 1/gamma (so c = 1), velocity scaled so that
    sqrt(<u^2+v^2+w^2>)/c = mach_t.  Generated by FFT on the host.
    """
    rng = np.random.default_rng(seed)
    k1 = np.fft.fftfreq(n, d=1.0 / n)
    KZ, KY, KX = np.meshgrid(k1, k1, k1, indexing="ij")
    k2 = KX * KX + KY * KY + KZ * KZ
    kk = np.sqrt(k2)
    k2s = np.where(k2 == 0, 1.0, k2)
    spec = kk ** 4 * np.exp(-2.0 * (kk / k0) ** 2)
    amp = np.sqrt(spec / np.where(kk == 0, 1.0, 4 * math.pi * kk * kk))
    amp[kk == 0] = 0.0
    comps = []
    for _ in range(3):
        ph = rng.uniform(0, 2 * math.pi, kk.shape)
        comps.append(amp * np.exp(1j * ph))
    cx, cy, cz = comps
    # project out the compressive part: c - k (k.c)/|k|^2
    dot = (KX * cx + KY * cy + KZ * cz) / k2s
    cx, cy, cz = cx - KX * dot, cy - KY * dot, cz - KZ * dot
    u = np.real(np.fft.ifftn(cx))
    v = np.real(np.fft.ifftn(cy))
    w = np.real(np.fft.ifftn(cz))
    urms = math.sqrt(float(np.mean(u * u + v * v + w * w)))
    s = mach_t / urms
    u, v, w = u * s, v * s, w * s
    h = 2.0 * math.pi / n
    rho = np.ones((n, n, n))
    p = np.full((n, n, n), 1.0 / gamma)
    Uv = prims_to_cons(rho, u, v, w, p, gamma)
    U = np.empty((NCONS, n + 2 * g, n + 2 * g, n + 2 * g))
    U[:, g:-g, g:-g, g:-g] = Uv
    # periodic ghosts
    U[:] = np.pad(Uv, ((0, 0), (g, g), (g, g), (g, g)), mode="wrap")
    return U, (h, h, h)


def periodic_pad(Uvalid, g=NGHOST):
    return np.pad(Uvalid, ((0, 0), (g, g), (g, g), (g, g)), mode="wrap")


def random_state(n, seed=0, gamma=1.4, amp=0.1, g=NGHOST):
    """Smooth-ish random positive state for unit tests (ghosts random too)."""
    rng = np.random.default_rng(seed)
    shape = (n[2] + 2 * g, n[1] + 2 * g, n[0] + 2 * g)
    rho = 1.0 + amp * rng.uniform(-1, 1, shape)
    u = amp * rng.uniform(-1, 1, shape)
    v = amp * rng.uniform(-1, 1, shape)
    w = amp * rng.uniform(-1, 1, shape)
    p = 1.0 / gamma + amp * rng.uniform(-1, 1, shape) * 0.5
    return prims_to_cons(rho, u, v, w, p, gamma)
