"""Small LIFE cases used as parity fixtures.

Each case is a ``params.h`` (as :class:`life_gb300.case.CaseParams`) plus a
geometry list. They are sized so that the reference, the oracle and the GPU
path each finish them in well under a second, while together covering every
collision operator, boundary type, inlet profile, forcing option and body type
the reference supports.

All cases use lattice units: ``height_p = Ny - 1`` (so ``Dx = 1``) and
``nu_p`` equal to the lattice viscosity computed from ``omega`` with the
reference's own formula, which makes ``Dt`` exactly 1.
"""
from __future__ import annotations

import os
import sys
from typing import Dict, List, Tuple

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))

from life_gb300.case import (BOUNDARY_LAYER, CONVECTIVE, FLUID, FREESLIP, PARABOLIC, PRESSURE,
                             SHEAR, VELOCITY, WALL, CaseParams, Circle, Filament)


def lattice_nu(omega: float) -> float:
    cs = 1.0 / (3.0 ** 0.5)
    return (1.0 / omega - 0.5) * (cs * cs)


def lattice_case(Nx: int, Ny: int, omega: float, nsteps: int, **kw) -> CaseParams:
    nu = lattice_nu(omega)
    base = dict(Nx=Nx, Ny=Ny, height_p=float(Ny - 1), rho_p=1.0, nu_p=nu, omega=omega,
                nSteps=nsteps, tinfo=nsteps, tVTK=nsteps, tRestart=nsteps, ref_L=1.0)
    base.update(kw)
    p = CaseParams(**base)
    assert p.Dx == 1.0 and p.Dt == 1.0, (p.Dx, p.Dt)
    return p


def golden_cases() -> Dict[str, Tuple[CaseParams, List]]:
    C: Dict[str, Tuple[CaseParams, List]] = {}

    C["cavity_bgk"] = (lattice_case(40, 40, 1.0 / 0.6, 400, wall_left=WALL, wall_right=WALL,
                                    wall_bottom=WALL, wall_top=VELOCITY, uxInlet_p=0.1), [])
    C["cavity_cm"] = (lattice_case(36, 44, 1.0 / 0.55, 400, wall_left=WALL, wall_right=WALL,
                                   wall_bottom=WALL, wall_top=VELOCITY, uxInlet_p=0.1,
                                   central_moments=True), [])
    C["channel_pressure_ramp"] = (lattice_case(60, 25, 1.0 / 0.62, 300, wall_left=VELOCITY,
                                               wall_right=PRESSURE, profile=PARABOLIC,
                                               uxInlet_p=0.05, inlet_ramp=100.0), [])
    C["channel_convective_freeslip_cm"] = (lattice_case(
        64, 30, 1.0 / 0.58, 300, wall_left=VELOCITY, wall_right=CONVECTIVE, wall_bottom=WALL,
        wall_top=FREESLIP, profile=BOUNDARY_LAYER, uxInlet_p=0.04, central_moments=True), [])
    C["periodic_womersley"] = (lattice_case(24, 33, 1.0 / 0.7, 300, wall_left=FLUID,
                                            wall_right=FLUID, wall_bottom=WALL, wall_top=WALL,
                                            womersley=3.0, dpdx=2e-5, ref_U=0.01), [])
    C["velocity_walls_shear"] = (lattice_case(
        50, 31, 1.0 / 0.65, 300, wall_left=VELOCITY, wall_right=CONVECTIVE,
        wall_bottom=VELOCITY, wall_top=VELOCITY, profile=SHEAR, uxInlet_p=0.06,
        uyInlet_p=0.002, inlet_ramp=50.0, gravityY=-3e-6), [])
    C["freeslip_pressure_gravity_cm"] = (lattice_case(
        40, 28, 1.0 / 0.6, 300, wall_left=PRESSURE, wall_right=PRESSURE, wall_bottom=FREESLIP,
        wall_top=WALL, gravityX=2e-5, ux0_p=0.01, central_moments=True, ref_U=0.01), [])
    # WOMERSLEY with gravity: the force of every site depends on its density
    # after the previous step (src/Grid.cpp:52-62)
    C["womersley_gravity_cm"] = (lattice_case(26, 31, 1.0 / 0.68, 300, wall_left=FLUID,
                                              wall_right=FLUID, wall_bottom=WALL, wall_top=WALL,
                                              womersley=2.5, dpdx=2e-5, dpdy=-1e-6, gravityX=8e-6,
                                              gravityY=-3e-6, central_moments=True, ref_U=0.01), [])
    # pressure walls on y with non-periodic x walls: the corners keep the
    # previous step's normal velocity (src/Grid.cpp:354-369)
    C["pressure_top_corners"] = (lattice_case(40, 30, 1.0 / 0.6, 300, wall_left=VELOCITY,
                                              wall_right=WALL, wall_bottom=WALL, wall_top=PRESSURE,
                                              uxInlet_p=0.03, inlet_ramp=50.0), [])
    C["pressure_ywalls_convective_cm"] = (lattice_case(
        48, 28, 1.0 / 0.62, 300, wall_left=VELOCITY, wall_right=CONVECTIVE, wall_bottom=PRESSURE,
        wall_top=PRESSURE, uxInlet_p=0.04, ux0_p=0.04, uy0_p=0.002, central_moments=True), [])
    C["periodic_y_uniform_init"] = (lattice_case(
        30, 26, 1.0 / 0.75, 250, wall_left=VELOCITY, wall_right=PRESSURE, wall_bottom=FLUID,
        wall_top=FLUID, uxInlet_p=0.03, ux0_p=0.03, uy0_p=0.001), [])

    C["cylinder_rigid_cm"] = (lattice_case(80, 41, 1.0 / 0.56, 300, wall_left=VELOCITY,
                                           wall_right=CONVECTIVE, uxInlet_p=0.05,
                                           inlet_ramp=50.0, central_moments=True, ref_L=12.0),
                              [Circle(x=20.0, y=20.3, radius=6.0, ID=0)])
    C["cylinders_uni_bgk"] = (lattice_case(90, 41, 1.0 / 0.6, 250, wall_left=VELOCITY,
                                           wall_right=PRESSURE, profile=PARABOLIC,
                                           uxInlet_p=0.04, inlet_ramp=40.0, uni_epsilon=True,
                                           ref_L=8.0),
                              [Circle(x=20.0, y=14.0, radius=4.0, ID=3, number=2, dx=25.0,
                                      dy=10.0)])
    C["filament_flex_deflect"] = (lattice_case(
        80, 41, 1.0 / 0.62, 200, wall_left=VELOCITY, wall_right=CONVECTIVE, uxInlet_p=0.05,
        inlet_ramp=30.0, initial_deflect=0.05, ref_L=20.0),
        [Filament(x=20.0, y=20.0, length=20.0, height=1.0, angle_deg=0.0, flexible=True,
                  n_elements=20, clamped=True, rho=10.0, E=48.0, ID=0)])
    C["turek_like_uni"] = (lattice_case(
        100, 41, 1.0 / 0.6, 150, wall_left=VELOCITY, wall_right=PRESSURE, profile=PARABOLIC,
        uxInlet_p=0.04, inlet_ramp=40.0, uni_epsilon=True, ref_L=10.0),
        [Circle(x=20.0, y=20.0, radius=5.0, ID=0),
         Filament(x=24.6, y=20.0, length=17.5, height=1.0, angle_deg=0.0, flexible=True,
                  n_elements=None, clamped=True, rho=10.0, E=400.0, ID=1)])
    C["honami_like_cm"] = (lattice_case(
        70, 31, 1.0 / 0.6, 200, wall_left=VELOCITY, wall_right=PRESSURE, wall_bottom=WALL,
        wall_top=FREESLIP, profile=BOUNDARY_LAYER, uxInlet_p=0.04, inlet_ramp=60.0,
        central_moments=True, ref_L=10.0),
        [Filament(x=20.0, y=0.0, length=10.0, height=0.6, angle_deg=90.0, flexible=True,
                  n_elements=10, clamped=True, rho=5.0, E=300.0, ID=0, number=4, dx=9.0)])
    C["filament_supported_and_rigid"] = (lattice_case(
        90, 41, 1.0 / 0.65, 150, wall_left=VELOCITY, wall_right=CONVECTIVE, uxInlet_p=0.04,
        inlet_ramp=30.0, ref_L=15.0, subTol=1e-9),
        [Filament(x=20.0, y=25.0, length=15.0, height=1.0, angle_deg=-10.0, flexible=True,
                  n_elements=12, clamped=False, rho=8.0, E=200.0, ID=5),
         Filament(x=55.0, y=14.0, length=10.0, height=1.0, angle_deg=30.0, flexible=False,
                  n_elements=None, clamped=True, rho=1.0, E=1.0, ID=9)])
    return C
