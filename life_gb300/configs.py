"""The named workloads of this path, as LIFE cases (``params.h`` values plus
``geometry.config`` bodies), all in lattice units (``height_p = Ny - 1`` so
``Dx = 1``; ``nu_p`` is the lattice viscosity of ``omega``, so ``Dt = 1``).

* :func:`cavity` -- the plain-method lid-driven cavity: D2Q9 BGK, regularised
  velocity lid u = 0.1, the other three walls regularised no-slip, Re = 1000
  on a 256 x 256 lattice (nu = 0.0256, tau = 0.5768), equilibrium start at
  rho = 1, u = 0. The same setup scaled to 4096 x 4096 is the roofline
  workload.
* :func:`cylinder` -- the rigid cylinder channel: 1000 x 400, central
  moments, D = 40 at (200, 200) (125 markers, ``floor(2 pi R / Dx)``,
  reference ``src/IBMBody.cpp:55``), uniform inlet 0.04, convective outlet,
  regularised no-slip top and bottom, Re = 100 on D (tau = 0.548).
* :func:`filament` -- the flexible filament channel: 1200 x 400 BGK, inlet
  0.05, convective outlet, one filament of L = 80 clamped at (300, 200), 80
  corotational elements and 81 markers, thickness 1, EI/(rho U^2 L^3) = 0.2
  (E = 3072), mass ratio 0.5 (rho_s = 40), Re = 100 on L (tau = 0.62),
  sub-iteration tolerance 1e-8, seeded initial tip deflection (default
  0.03 L).
"""
from __future__ import annotations

from typing import List, Tuple

from .case import CONVECTIVE, PREC_F64, VELOCITY, WALL, CaseParams, Circle, Filament


def lattice_nu(omega: float) -> float:
    """Lattice viscosity of a relaxation rate, with the reference's formula
    (``src/Grid.cpp:1250-1253``: nu = (tau - 1/2) c_s^2)."""
    cs = 1.0 / (3.0 ** 0.5)
    return (1.0 / omega - 0.5) * (cs * cs)


def cavity(n: int = 256, precision: int = PREC_F64, cm: bool = False, steps: int = 20000,
           tinfo: int = None) -> CaseParams:
    omega = 1.0 / 0.5768
    return CaseParams(Nx=n, Ny=n, height_p=float(n - 1), rho_p=1.0, nu_p=lattice_nu(omega), omega=omega,
                      wall_left=WALL, wall_right=WALL, wall_bottom=WALL, wall_top=VELOCITY,
                      uxInlet_p=0.1, central_moments=cm, precision=precision, ref_L=float(n - 1),
                      nSteps=steps, tinfo=tinfo or steps, tVTK=steps, tRestart=steps)


def cylinder(precision: int = PREC_F64, steps: int = 50000, tinfo: int = 100) -> Tuple[CaseParams, List]:
    omega = 1.0 / 0.548
    p = CaseParams(Nx=1000, Ny=400, height_p=399.0, rho_p=1.0, nu_p=lattice_nu(omega), omega=omega,
                   wall_left=VELOCITY, wall_right=CONVECTIVE, wall_bottom=WALL, wall_top=WALL,
                   uxInlet_p=0.04, central_moments=True, precision=precision, ref_L=40.0,
                   nSteps=steps, tinfo=tinfo, tVTK=steps, tRestart=steps)
    return p, [Circle(x=200.0, y=200.0, radius=20.0)]


def filament(precision: int = PREC_F64, steps: int = 2000, tinfo: int = 10,
             deflect: float = 0.03) -> Tuple[CaseParams, List]:
    omega = 1.0 / 0.62
    p = CaseParams(Nx=1200, Ny=400, height_p=399.0, rho_p=1.0, nu_p=lattice_nu(omega), omega=omega,
                   wall_left=VELOCITY, wall_right=CONVECTIVE, wall_bottom=WALL, wall_top=WALL,
                   uxInlet_p=0.05, precision=precision, ref_L=80.0, initial_deflect=deflect, subTol=1e-8,
                   nSteps=steps, tinfo=tinfo, tVTK=steps, tRestart=steps)
    return p, [Filament(x=300.0, y=200.0, length=80.0, height=1.0, angle_deg=0.0, flexible=True,
                        n_elements=80, clamped=True, rho=40.0, E=3072.0)]
