"""The reference's text observables, written from the device recorder's rows.

``ObjectsClass::writeTotalForces`` and ``ObjectsClass::writeTips`` (reference
``src/Objects.cpp:491-594``) append one line every ``tinfo`` steps to
``Results/TotalForces.out``, ``Results/TipPositions.out`` and
``Results/TipVelocities.out``, with the stream precision ``PRECISION`` (10
significant digits, C++ default float format, i.e. ``%.10g``). The rows come
from :meth:`life_gb300.lib.Case.records` (``life_case_record`` /
``life_case_records``); these functions only format them, so a run on the GPU
writes the same files the reference writes.
"""
from __future__ import annotations

from typing import Dict, Sequence

import numpy as np

from .case import CaseParams


def _g(x: float, precision: int = 10) -> str:
    return format(float(x), f".{precision}g")


def nd_force(p: CaseParams) -> float:
    """0.5 * ref_rho * SQ(ref_U) * ref_L, in the reference's order
    (``src/Objects.cpp:531``)."""
    return 0.5 * p.ref_rho * (p.ref_U * p.ref_U) * p.ref_L


def total_forces_lines(p: CaseParams, Dt: float, rec: Dict[str, np.ndarray]) -> Sequence[str]:
    """Lines of ``TotalForces.out`` for the recorded rows (no header)."""
    nd = nd_force(p)
    out = []
    for t, (fx, fy) in zip(rec["t"], rec["force"]):
        out.append("\t".join([str(int(t)), _g(Dt * int(t)), _g(fx), _g(fy), _g(fx / nd), _g(fy / nd)]))
    return out


def tip_lines(Dt: float, rec: Dict[str, np.ndarray], key: str = "tip_pos") -> Sequence[str]:
    """Lines of ``TipPositions.out`` (key ``tip_pos``) or ``TipVelocities.out``
    (key ``tip_vel``) for the recorded rows (no header)."""
    out = []
    for t, tips in zip(rec["t"], rec[key]):
        cols = [str(int(t)), _g(Dt * int(t))]
        for x, y in tips:
            cols += [_g(x), _g(y)]
        out.append("\t".join(cols))
    return out


TOTAL_FORCES_HEADER = "Timestep\tTime (s)\tFx (N)\tFy (N)\tCx\tCy"
TIPS_HEADER = "Timestep\tTime (s)\tTipX\tTipY"


def total_forces_text(p: CaseParams, Dt: float, rec: Dict[str, np.ndarray]) -> str:
    """Whole ``TotalForces.out`` as the reference writes it (header, then one
    line per row, each line after a newline, no trailing newline)."""
    return TOTAL_FORCES_HEADER + "".join("\n" + ln for ln in total_forces_lines(p, Dt, rec))


def tips_text(Dt: float, rec: Dict[str, np.ndarray], key: str = "tip_pos") -> str:
    return TIPS_HEADER + "".join("\n" + ln for ln in tip_lines(Dt, rec, key))


def parse_table(text: str) -> np.ndarray:
    """Numbers of a reference observables file (header skipped)."""
    rows = [ln.split("\t") for ln in text.strip("\n").splitlines()[1:] if ln.strip()]
    return np.array([[float(x) for x in r] for r in rows])
