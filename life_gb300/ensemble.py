"""Seeded synthetic workloads built from LIFE case descriptions.

:func:`ensemble_cases` draws the batched-ensemble workload: independent
channel cases of uneven lattice size, each holding either rigid cylinders or
a set of clamped flexible filaments, with per-case Reynolds number and
collision model. :func:`canopy_case` draws one serving request: a canopy of
flexible stalks clamped on the bottom wall of a boundary-layer channel (the
arrangement of the reference's Honami example geometry).

Every case is an ordinary ``(CaseParams, bodies)`` pair in lattice units
(Dx = Dt = 1); nothing here touches the GPU.
"""
from __future__ import annotations

import math
from typing import List, Sequence, Tuple

import numpy as np

from .case import BOUNDARY_LAYER, CONVECTIVE, VELOCITY, WALL, CaseParams, Circle, Filament

CS2 = 1.0 / 3.0
TAU_MIN = 0.53  # BGK stays stable over the benchmarked steps above this
# Filament thickness in lattice units. The beam's axial stiffness is
# EA = 12 EI / H^2 for a given bending stiffness EI, so a thin section keeps
# soft filaments practically inextensible (with H = 1 the softest ones
# stretch by tens of percent under drag and the coupling diverges).
THICKNESS = 0.1


def _lattice(Nx: int, Ny: int, tau: float, precision: int, **kw) -> CaseParams:
    nu = (tau - 0.5) * CS2
    base = dict(Nx=Nx, Ny=Ny, height_p=float(Ny - 1), rho_p=1.0, nu_p=nu, omega=1.0 / tau,
                precision=precision)
    base.update(kw)
    return CaseParams(**base)


def _tau_for(u: float, length: float, re: float) -> Tuple[float, float]:
    """Relaxation time for Re = u L / nu, held at TAU_MIN or above; returns
    (tau, the Reynolds number it gives)."""
    tau = 0.5 + 3.0 * u * length / re
    if tau < TAU_MIN:
        tau = TAU_MIN
    return tau, u * length / ((tau - 0.5) * CS2)


def filament_modulus(stiffness: float, u: float, length: float, height: float = THICKNESS) -> float:
    """Young's modulus for a non-dimensional bending stiffness
    EI / (rho_f U^2 L^3) with I = H^3 / 12 and rho_f = 1."""
    return stiffness * u * u * length ** 3 * 12.0 / height ** 3


def ensemble_cases(n: int = 64, seed: int = 20260101, precision: int = 0, u_in: float = 0.04,
                   mass_ratio: float = 10.0, stiffness=(1e-2, 1e-1),
                   thickness: float = THICKNESS) -> List[Tuple[CaseParams, list]]:
    """The batched-ensemble workload: n channel cases, inlet u_in on the left
    (ramped in over 400 steps), convective outlet, no-slip top and bottom.

    Per case: width uniform in 256..2048 and height in 128..512 (multiples of
    32); with probability 1/2 it holds 0-4 rigid cylinders (D uniform 16..48),
    else 1-8 flexible filaments clamped at their leading end (L uniform
    20..60, one element per lattice unit, bending stiffness EI/(rho U^2 L^3)
    log-uniform over `stiffness`, mass ratio `mass_ratio`, thickness
    THICKNESS), in rows at least one filament length apart and columns 2.5
    lengths apart (out of each other's near wake); Re uniform
    50..300 on the largest body (tau held at 0.53 or above); BGK or central
    moments with probability 1/2. Bodies that would not fit the lattice are
    dropped. The filaments start straight and the ramped inflow bends them.
    With unit elements and U = 0.04, filaments softer than about 1e-2 flap
    with tip speeds beyond the lattice's low-Mach range and their coupling
    diverges within 10000 steps (the subiteration cap), as do filaments in
    rows closer than their length; hence the defaults.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(n):
        W = int(rng.integers(8, 65)) * 32
        H = int(rng.integers(4, 17)) * 32
        cylinders = bool(rng.random() < 0.5)
        re = float(rng.uniform(50.0, 300.0))
        cm = bool(rng.random() < 0.5)
        bodies: list = []
        if cylinders:
            m = int(rng.integers(0, 5))
            ds = [float(rng.uniform(16.0, 48.0)) for _ in range(m)]
            ds = [min(d, H / 3.0) for d in ds]
            x = 0.0
            for k, d in enumerate(ds):
                x = (max(1.5 * d, W / 8.0) if k == 0 else x + 2.5 * max(ds))
                if x + 2.0 * d > 0.75 * W:
                    break
                y = H / 2.0 + (H / 6.0 if k % 2 else 0.0) * (1 if k % 4 == 1 else -1)
                bodies.append(Circle(x=round(x, 3), y=round(y, 3), radius=round(d / 2.0, 3), ID=k))
            lref = max([2.0 * b.radius for b in bodies], default=32.0)
        else:
            m = int(rng.integers(1, 9))
            lengths = [int(rng.integers(20, 61)) for _ in range(m)]
            lo, hi = math.log10(stiffness[0]), math.log10(stiffness[1])
            stiff = [float(10.0 ** rng.uniform(lo, hi)) for _ in range(m)]
            lmax = max(lengths)
            x0 = max(W / 8.0, 20.0)
            ncols = max(1, int((0.7 * W - x0) // (2.5 * lmax)))
            nrows = max(1, min(math.ceil(m / ncols), int(H // lmax) - 1))
            m = min(m, ncols * nrows)
            for k in range(m):
                col, row = k % ncols, k // ncols
                x = x0 + col * 2.5 * lmax
                y = H * (row + 1) / (nrows + 1)
                L = lengths[k]
                bodies.append(Filament(x=round(x, 3), y=round(y, 3), length=float(L), height=thickness,
                                       angle_deg=0.0, flexible=True, n_elements=L, clamped=True,
                                       rho=mass_ratio * L / thickness,
                                       E=filament_modulus(stiff[k], u_in, L, thickness), ID=k))
            lref = float(max(b.length for b in bodies))
        tau, _ = _tau_for(u_in, lref, re)
        kw = dict(wall_left=VELOCITY, wall_right=CONVECTIVE, wall_bottom=WALL, wall_top=WALL,
                  uxInlet_p=u_in, inlet_ramp=400.0, central_moments=cm, ref_L=lref, subTol=1e-8)
        out.append((_lattice(W, H, tau, precision, **kw), bodies))
    return out


def canopy_case(rng: np.random.Generator, precision: int = 1, mass_ratio: float = 10.0,
                stiffness=(1e-2, 1e-1), thickness: float = THICKNESS) -> Tuple[CaseParams, list, int]:
    """One serving request: a canopy of 8-32 stalks clamped on the bottom wall
    (angle 90 degrees), evenly spaced, length 20-40 lattice units with 20
    corotational elements each, bending stiffness log-uniform over
    `stiffness` (mass ratio and thickness as in ensemble_cases, for the same
    reason), in a 512-4096 x 256-1024 lattice (multiples of 32) with a
    boundary-layer inlet of 0.02-0.06 and a free-slip top. Returns (params,
    bodies, steps) with steps uniform in 2000..20000."""
    W = int(rng.integers(16, 129)) * 32
    H = int(rng.integers(8, 33)) * 32
    m = int(rng.integers(8, 33))
    u = float(rng.uniform(0.02, 0.06))
    steps = int(rng.integers(2000, 20001))
    lengths = [float(rng.uniform(20.0, 40.0)) for _ in range(m)]
    lo, hi = math.log10(stiffness[0]), math.log10(stiffness[1])
    stiff = [float(10.0 ** rng.uniform(lo, hi)) for _ in range(m)]
    lmax = max(lengths)
    x0, x1 = max(W / 8.0, 40.0), 0.75 * W
    gap = (x1 - x0) / max(m - 1, 1)
    if gap < 4.0:
        m = max(1, int((x1 - x0) // 4.0) + 1)
        gap = (x1 - x0) / max(m - 1, 1)
    bodies = [Filament(x=round(x0 + k * gap, 3), y=0.0, length=lengths[k], height=thickness, angle_deg=90.0,
                       flexible=True, n_elements=20, clamped=True, rho=mass_ratio * lengths[k] / thickness,
                       E=filament_modulus(stiff[k], u, lengths[k], thickness), ID=k) for k in range(m)]
    tau, _ = _tau_for(u, lmax, 100.0)
    from .case import FREESLIP
    p = _lattice(W, H, tau, precision, wall_left=VELOCITY, wall_right=CONVECTIVE, wall_bottom=WALL,
                 wall_top=FREESLIP, profile=BOUNDARY_LAYER, uxInlet_p=u, inlet_ramp=400.0, ref_L=lmax,
                 subTol=1e-8)
    return p, bodies, steps


def sites(cases: Sequence) -> int:
    return sum(p.Nx * p.Ny for p, _ in cases)
