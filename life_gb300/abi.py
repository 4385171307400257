"""ctypes mirror of the structs in ``include/life_gb300.h``.

These are the plain-C records that cross the C-ABI: :class:`LifeCaseParams`
(every ``params.h`` value), :class:`LifeBodyDesc` (one ``geometry.config``
line), :class:`LifeCaseInfo` and :class:`LifeStatus`.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

from .case import CaseParams, Circle, Filament

LIFE_OK = 0
ERRORS = {
    1: "LIFE_ERR_INVALID", 2: "LIFE_ERR_CUDA", 3: "LIFE_ERR_NAN", 4: "LIFE_ERR_SUBITER",
    5: "LIFE_ERR_SUPPORT", 6: "LIFE_ERR_GEOMETRY", 7: "LIFE_ERR_DEFLECT", 8: "LIFE_ERR_NOMEM",
    9: "LIFE_ERR_TIMEOUT", 10: "LIFE_ERR_BUSY",
}


class LifeCaseParams(C.Structure):
    _fields_ = [
        ("Nx", C.c_int32), ("Ny", C.c_int32),
        ("height_p", C.c_double), ("rho_p", C.c_double), ("nu_p", C.c_double), ("omega", C.c_double),
        ("ux0_p", C.c_double), ("uy0_p", C.c_double),
        ("gravityX", C.c_double), ("gravityY", C.c_double), ("dpdx", C.c_double), ("dpdy", C.c_double),
        ("wall_left", C.c_int32), ("wall_right", C.c_int32), ("wall_bottom", C.c_int32),
        ("wall_top", C.c_int32), ("profile", C.c_int32),
        ("uxInlet_p", C.c_double), ("uyInlet_p", C.c_double),
        ("alpha", C.c_double), ("delta", C.c_double), ("relaxMax", C.c_double), ("subTol", C.c_double),
        ("central_moments", C.c_int32),
        ("has_inlet_ramp", C.c_int32), ("inlet_ramp", C.c_double),
        ("has_womersley", C.c_int32), ("womersley", C.c_double),
        ("uni_epsilon", C.c_int32), ("ordered", C.c_int32),
        ("has_initial_deflect", C.c_int32), ("initial_deflect", C.c_double),
        ("nSteps", C.c_int32), ("tinfo", C.c_int32), ("tVTK", C.c_int32), ("tRestart", C.c_int32),
        ("ref_nu", C.c_double), ("ref_rho", C.c_double), ("ref_P", C.c_double), ("ref_L", C.c_double),
        ("ref_U", C.c_double),
        ("precision", C.c_int32), ("reserved", C.c_int32 * 7),
    ]


class LifeBodyDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("number", C.c_int32), ("id", C.c_int32), ("flexible", C.c_int32),
        ("n_elements", C.c_int32), ("clamped", C.c_int32),
        ("x", C.c_double), ("y", C.c_double), ("dx", C.c_double), ("dy", C.c_double),
        ("radius", C.c_double), ("length", C.c_double), ("height", C.c_double),
        ("angle_deg", C.c_double), ("rho", C.c_double), ("E", C.c_double),
    ]


class LifeCaseInfo(C.Structure):
    _fields_ = [
        ("Nx", C.c_int32), ("Ny", C.c_int32), ("n_bodies", C.c_int32), ("n_markers", C.c_int32),
        ("n_flex", C.c_int32), ("sim_dofs", C.c_int32), ("precision", C.c_int32), ("t", C.c_int32),
        ("Dx", C.c_double), ("Dt", C.c_double), ("Dm", C.c_double), ("Drho", C.c_double),
        ("tau", C.c_double), ("nu", C.c_double), ("c_s", C.c_double), ("device_bytes", C.c_size_t),
    ]


class LifeBatchInfo(C.Structure):
    _fields_ = [
        ("n_cases", C.c_int32), ("precision", C.c_int32), ("sites", C.c_int64),
        ("tile_w", C.c_int32), ("tile_h", C.c_int32), ("tiles", C.c_int32), ("grid", C.c_int32),
        ("kernel_nodes", C.c_int32), ("device_bytes", C.c_size_t),
    ]


class LifeServerConfig(C.Structure):
    _fields_ = [("hbm_budget", C.c_size_t), ("max_active", C.c_int32), ("steps_per_round", C.c_int32)]


class LifeRequestInfo(C.Structure):
    _fields_ = [
        ("state", C.c_int32), ("error", C.c_int32), ("steps_done", C.c_int32), ("steps", C.c_int32),
        ("submit_s", C.c_double), ("start_s", C.c_double), ("done_s", C.c_double),
        ("device_bytes", C.c_size_t), ("sites", C.c_int64),
    ]


class LifeServerStats(C.Structure):
    _fields_ = [
        ("submitted", C.c_int64), ("admitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64),
        ("active", C.c_int32), ("queued", C.c_int32), ("bytes_in_use", C.c_size_t), ("bytes_peak", C.c_size_t),
        ("rounds", C.c_int64), ("regroups", C.c_int64), ("site_steps", C.c_double), ("busy_s", C.c_double),
        ("clock_s", C.c_double),
    ]


class LifeStatus(C.Structure):
    _fields_ = [
        ("code", C.c_int32), ("t", C.c_int32), ("last_subits", C.c_int32),
        ("last_nr_its", C.c_int32), ("last_subres", C.c_double), ("relax", C.c_double),
    ]


def params_struct(p: CaseParams) -> LifeCaseParams:
    s = LifeCaseParams()
    for name in ("Nx", "Ny", "wall_left", "wall_right", "wall_bottom", "wall_top", "nSteps",
                 "tinfo", "tVTK", "tRestart"):
        setattr(s, name, int(getattr(p, name)))
    for name in ("height_p", "rho_p", "nu_p", "omega", "ux0_p", "uy0_p", "gravityX", "gravityY",
                 "dpdx", "dpdy", "uxInlet_p", "uyInlet_p", "alpha", "delta", "relaxMax", "subTol",
                 "ref_nu", "ref_rho", "ref_P", "ref_L", "ref_U"):
        setattr(s, name, float(getattr(p, name)))
    s.profile = -1 if p.profile is None else int(p.profile)
    s.central_moments = int(bool(p.central_moments))
    s.has_inlet_ramp = int(p.inlet_ramp is not None)
    s.inlet_ramp = float(p.inlet_ramp or 0.0)
    s.has_womersley = int(p.womersley is not None)
    s.womersley = float(p.womersley or 0.0)
    s.uni_epsilon = int(bool(p.uni_epsilon))
    s.ordered = int(bool(p.ordered))
    s.has_initial_deflect = int(p.initial_deflect is not None)
    s.initial_deflect = float(p.initial_deflect or 0.0)
    s.precision = int(p.precision)
    return s


def body_structs(bodies: Sequence) -> "C.Array":
    arr = (LifeBodyDesc * max(1, len(bodies)))()
    for k, b in enumerate(bodies):
        d = arr[k]
        d.number, d.id = int(b.number), int(b.ID)
        d.x, d.y, d.dx, d.dy = float(b.x), float(b.y), float(b.dx), float(b.dy)
        if isinstance(b, Circle):
            d.kind = 0  # CIRCLE_KIND
            d.radius = float(b.radius)
        elif isinstance(b, Filament):
            d.kind = 1
            d.flexible = int(bool(b.flexible))
            d.n_elements = 0 if b.n_elements is None else int(b.n_elements)
            d.clamped = int(bool(b.clamped))
            d.length, d.height, d.angle_deg = float(b.length), float(b.height), float(b.angle_deg)
            d.rho, d.E = float(b.rho), float(b.E)
        else:
            raise TypeError(f"not a body: {b!r}")
    return arr
