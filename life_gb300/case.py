"""Case description in LIFE's own format.

A LIFE case is a compile-time ``params.h`` (reference ``inc/params.h:26-110``)
plus a run-time ``input/geometry.config`` (reference ``input/geometry.config``,
parsed by ``ObjectsClass::geometryReadIn``, reference ``src/Objects.cpp:324-488``).

:class:`CaseParams` holds the values of every ``params.h`` constant and switch
that the solver reads. It renders back to a ``params.h`` that the reference
compiles (``to_params_h``), so the same numbers drive both codes: every double
is written with ``repr`` (shortest round-trip form), which a C++ compiler
parses back to the identical IEEE value. :class:`Circle` and :class:`Filament`
are the two ``geometry.config`` keywords; ``geometry_config_text`` renders them.

``load_params_h`` goes the other way: it compiles an existing ``params.h``
together with ``include/life_params_pack.h`` and reads back the exact values, so
a reference case directory can be run unchanged.
"""
from __future__ import annotations

import dataclasses
import math
import os
import struct
import subprocess
import tempfile
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Union

# eLatType (reference inc/defs.h:51). eFluid on a wall means periodic.
FLUID, WALL, VELOCITY, FREESLIP, PRESSURE, CONVECTIVE = range(6)
LAT_NAMES = ["eFluid", "eWall", "eVelocity", "eFreeSlip", "ePressure", "eConvective"]
# eProfileType (reference inc/defs.h:52); None = uniform inlet (PROFILE undefined).
PARABOLIC, SHEAR, BOUNDARY_LAYER = range(3)
PROFILE_NAMES = ["eParabolic", "eShear", "eBoundaryLayer"]

# geometry.config keywords (LifeBodyDesc.kind, LIFE_BODY_CIRCLE / _FILAMENT).
CIRCLE_KIND, FILAMENT_KIND = 0, 1

# Storage/arithmetic forms of the lattice populations on the GPU.
PREC_F64, PREC_F32, PREC_F16 = 0, 1, 2
PREC_NAMES = {"f64": PREC_F64, "f32": PREC_F32, "f16": PREC_F16}


@dataclass
class CaseParams:
    """Values of the reference's ``params.h`` (names kept as in the reference)."""

    Nx: int
    Ny: int
    height_p: float
    rho_p: float
    nu_p: float
    omega: float
    ux0_p: float = 0.0
    uy0_p: float = 0.0
    gravityX: float = 0.0
    gravityY: float = 0.0
    dpdx: float = 0.0
    dpdy: float = 0.0
    wall_left: int = VELOCITY
    wall_right: int = PRESSURE
    wall_bottom: int = WALL
    wall_top: int = WALL
    profile: Optional[int] = None
    uxInlet_p: float = 0.0
    uyInlet_p: float = 0.0
    alpha: float = 0.25
    delta: float = 0.5
    relaxMax: float = 1.0
    subTol: float = 1e-8
    central_moments: bool = False
    inlet_ramp: Optional[float] = None
    womersley: Optional[float] = None
    uni_epsilon: bool = False
    ordered: bool = True
    initial_deflect: Optional[float] = None
    # output switches of params.h (VTK files; the FEM file too with vtk_fem)
    vtk: bool = False
    vtk_fem: bool = False
    nSteps: int = 100
    tinfo: int = 100
    tVTK: int = 100
    tRestart: int = 100
    ref_nu: Optional[float] = None
    ref_rho: Optional[float] = None
    ref_P: float = 0.0
    ref_L: float = 1.0
    ref_U: Optional[float] = None
    # GPU-side choice, not a params.h value: population storage form.
    precision: int = PREC_F64

    def __post_init__(self) -> None:
        if self.ref_nu is None:
            self.ref_nu = self.nu_p
        if self.ref_rho is None:
            self.ref_rho = self.rho_p
        if self.ref_U is None:
            self.ref_U = self.uxInlet_p

    # ------------------------------------------------------------ derived --
    # Same formulas and operation order as GridClass::GridClass
    # (reference src/Grid.cpp:1247-1260).
    @property
    def c_s(self) -> float:
        return 1.0 / (3.0 ** 0.5)

    @property
    def tau(self) -> float:
        return 1.0 / self.omega

    @property
    def nu(self) -> float:
        cs = self.c_s
        return (self.tau - 0.5) * (cs * cs)

    @property
    def Dx(self) -> float:
        return self.height_p / (self.Ny - 1)

    @property
    def Dt(self) -> float:
        return (self.Dx * self.Dx) * self.nu / self.nu_p

    def replace(self, **kw) -> "CaseParams":
        return dataclasses.replace(self, **kw)

    # --------------------------------------------------------- rendering --
    def to_params_h(self) -> str:
        """Render a reference-format ``params.h`` with these exact values."""
        r = repr

        def d(name: str, on: bool, val: Optional[float] = None) -> str:
            if not on:
                return f"//#define {name}\n"
            return f"#define {name} {r(float(val))}\n" if val is not None else f"#define {name}\n"

        s = ["#ifndef PARAMS_H\n#define PARAMS_H\n#include \"defs.h\"\n"]
        s.append(d("CENTRAL_MOMENTS", self.central_moments))
        s.append(d("INLET_RAMP", self.inlet_ramp is not None, self.inlet_ramp))
        s.append(d("WOMERSLEY", self.womersley is not None, self.womersley))
        s.append(d("UNI_EPSILON", self.uni_epsilon))
        s.append(d("ORDERED", self.ordered))
        s.append(d("INITIAL_DEFLECT", self.initial_deflect is not None, self.initial_deflect))
        s.append(d("VTK", self.vtk))
        s.append(d("VTK_FEM", self.vtk_fem))
        s.append("#define FORCES\n#define TIPS\n")
        s.append(f"const int Nx = {int(self.Nx)};\nconst int Ny = {int(self.Ny)};\n")
        for name in ("height_p", "rho_p", "nu_p", "ux0_p", "uy0_p", "gravityX", "gravityY",
                     "dpdx", "dpdy"):
            s.append(f"const double {name} = {r(float(getattr(self, name)))};\n")
        s.append(f"#define WALL_LEFT {LAT_NAMES[self.wall_left]}\n")
        s.append(f"#define WALL_RIGHT {LAT_NAMES[self.wall_right]}\n")
        s.append(f"#define WALL_BOTTOM {LAT_NAMES[self.wall_bottom]}\n")
        s.append(f"#define WALL_TOP {LAT_NAMES[self.wall_top]}\n")
        if self.profile is not None:
            s.append(f"#define PROFILE {PROFILE_NAMES[self.profile]}\n")
        for name in ("uxInlet_p", "uyInlet_p", "alpha", "delta", "relaxMax", "subTol", "omega"):
            s.append(f"const double {name} = {r(float(getattr(self, name)))};\n")
        s.append("const double tStep = 1.0;\n")
        for name in ("nSteps", "tinfo", "tVTK", "tRestart"):
            s.append(f"const int {name} = {int(getattr(self, name))};\n")
        for name in ("ref_nu", "ref_rho", "ref_P", "ref_L", "ref_U"):
            s.append(f"const double {name} = {r(float(getattr(self, name)))};\n")
        s.append("const int PRECISION = 10;\n#endif\n")
        return "".join(s)


@dataclass
class Circle:
    """``CIRCLE NUMBER STARTID X Y SPACING_X SPACING_Y RADIUS`` (physical units)."""

    x: float
    y: float
    radius: float
    ID: int = 0
    number: int = 1
    dx: float = 0.0
    dy: float = 0.0

    def config_line(self) -> str:
        r = repr
        return (f"CIRCLE {self.number} {self.ID} {r(float(self.x))} {r(float(self.y))} "
                f"{r(float(self.dx))} {r(float(self.dy))} {r(float(self.radius))}")


@dataclass
class Filament:
    """``FILAMENT NUMBER STARTID X Y SPACING_X SPACING_Y LENGTH HEIGHT ANGLE
    FLEXIBLE|RIGID N_ELEMENTS|CONFORMING CLAMPED|SUPPORTED DENSITY YOUNG_MODULUS``."""

    x: float
    y: float
    length: float
    height: float
    angle_deg: float = 0.0
    flexible: bool = True
    n_elements: Optional[int] = None  # None = CONFORMING
    clamped: bool = True
    rho: float = 1.0
    E: float = 1.0
    ID: int = 0
    number: int = 1
    dx: float = 0.0
    dy: float = 0.0

    def config_line(self) -> str:
        r = repr
        nel = "CONFORMING" if self.n_elements is None else str(int(self.n_elements))
        return (f"FILAMENT {self.number} {self.ID} {r(float(self.x))} {r(float(self.y))} "
                f"{r(float(self.dx))} {r(float(self.dy))} {r(float(self.length))} "
                f"{r(float(self.height))} {r(float(self.angle_deg))} "
                f"{'FLEXIBLE' if self.flexible else 'RIGID'} {nel} "
                f"{'CLAMPED' if self.clamped else 'SUPPORTED'} {r(float(self.rho))} {r(float(self.E))}")


def _splitmix64_draws(seed: int):
    """SplitMix64 (Steele, Lea and Flood 2014), each output mapped to [0, 1)
    with 53 bits: the draws of the CANOPY keyword."""
    mask = (1 << 64) - 1
    state = seed & mask
    while True:
        state = (state + 0x9E3779B97F4A7C15) & mask
        z = state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
        z ^= z >> 31
        yield (z >> 11) * 2.0 ** -53


@dataclass
class Canopy:
    """``CANOPY NUMBER STARTID STARTX STARTY SPACING_X SPACING_Y LENGTH_MIN
    LENGTH_MAX HEIGHT ANGLE N_ELEMENTS|CONFORMING CLAMPED|SUPPORTED
    DENSITY_PER_LENGTH YOUNG_MIN YOUNG_MAX SEED``: a geometry.config keyword of
    this library (added as the reference's README, ``README.md:36-40``,
    describes) for a row of flexible stalks of random length and stiffness.
    Stalk k stands at (x + k dx, y + k dy); its length is
    ``length_min + (length_max - length_min) r``, its density
    ``density_per_length * L`` and its Young's modulus
    ``(young_min * (young_max / young_min) ** r') * (L * L * L)``, with r, r' the
    stalk's two draws of SplitMix64 seeded with ``seed``. ``expand`` gives the
    FILAMENT bodies the library's parser (life_parse_geometry) builds."""

    x: float
    y: float
    length_min: float
    length_max: float
    height: float
    density_per_length: float
    young_min: float
    young_max: float
    seed: int
    angle_deg: float = 90.0
    n_elements: Optional[int] = None
    clamped: bool = True
    ID: int = 0
    number: int = 1
    dx: float = 0.0
    dy: float = 0.0

    def config_line(self) -> str:
        r = repr
        nel = "CONFORMING" if self.n_elements is None else str(int(self.n_elements))
        return (f"CANOPY {self.number} {self.ID} {r(float(self.x))} {r(float(self.y))} {r(float(self.dx))} "
                f"{r(float(self.dy))} {r(float(self.length_min))} {r(float(self.length_max))} "
                f"{r(float(self.height))} {r(float(self.angle_deg))} {nel} "
                f"{'CLAMPED' if self.clamped else 'SUPPORTED'} {r(float(self.density_per_length))} "
                f"{r(float(self.young_min))} {r(float(self.young_max))} {int(self.seed)}")

    def expand(self) -> List["Filament"]:
        draws = _splitmix64_draws(int(self.seed))
        out = []
        for k in range(int(self.number)):
            rl, ry = next(draws), next(draws)
            L = self.length_min + (self.length_max - self.length_min) * rl
            E = (self.young_min * math.pow(self.young_max / self.young_min, ry)) * (L * L * L)
            out.append(Filament(x=self.x + k * self.dx, y=self.y + k * self.dy, length=L, height=self.height,
                                angle_deg=self.angle_deg, flexible=True, n_elements=self.n_elements,
                                clamped=self.clamped, rho=self.density_per_length * L, E=E, ID=self.ID + k))
        return out


Body = Union[Circle, Filament, Canopy]


def expand_bodies(bodies: Sequence) -> List[Body]:
    """The body lines as the C-ABI takes them: CANOPY lines expanded into their
    FILAMENT stalks (as life_parse_geometry does), other lines unchanged."""
    out: List[Body] = []
    for b in bodies:
        out += b.expand() if isinstance(b, Canopy) else [b]
    return out


def geometry_config_text(bodies: Sequence[Body]) -> str:
    lines = ["# geometry.config written by life_gb300.case"]
    lines += [b.config_line() for b in bodies]
    return "\n".join(lines) + "\n"


def parse_geometry_config(text: str) -> List[Body]:
    """Parse ``geometry.config`` text with the reference's rules.

    Leading lines that start with ``#`` are skipped (reference
    ``src/Objects.cpp:338-353``); the rest is read as whitespace-separated
    tokens, one body group per keyword (``src/Objects.cpp:399-458``).
    """
    lines = text.splitlines()
    k = 0
    while k < len(lines) and lines[k].startswith("#"):
        k += 1
    toks = " ".join(lines[k:]).split()
    out: List[Body] = []
    p = 0
    while p < len(toks):
        kw = toks[p]
        if kw == "CIRCLE":
            n, ID = int(toks[p + 1]), int(toks[p + 2])
            x, y, dx, dy, rad = map(float, toks[p + 3:p + 8])
            out.append(Circle(x=x, y=y, radius=rad, ID=ID, number=n, dx=dx, dy=dy))
            p += 8
        elif kw == "FILAMENT":
            n, ID = int(toks[p + 1]), int(toks[p + 2])
            x, y, dx, dy, L, H, ang = map(float, toks[p + 3:p + 10])
            flex, nel, bc = toks[p + 10], toks[p + 11], toks[p + 12]
            rho, E = float(toks[p + 13]), float(toks[p + 14])
            if flex not in ("FLEXIBLE", "RIGID"):
                raise ValueError("Not a proper flexible type set...exiting")
            out.append(Filament(x=x, y=y, length=L, height=H, angle_deg=ang,
                                flexible=(flex == "FLEXIBLE"),
                                n_elements=None if nel == "CONFORMING" else int(float(nel)),
                                clamped=(bc == "CLAMPED"), rho=rho, E=E, ID=ID, number=n,
                                dx=dx, dy=dy))
            p += 15
        elif kw == "CANOPY":
            n, ID = int(toks[p + 1]), int(toks[p + 2])
            x, y, dx, dy, lmin, lmax, H, ang = map(float, toks[p + 3:p + 11])
            nel, bc = toks[p + 11], toks[p + 12]
            dpl, ymin, ymax = map(float, toks[p + 13:p + 16])
            out.append(Canopy(x=x, y=y, length_min=lmin, length_max=lmax, height=H, density_per_length=dpl,
                              young_min=ymin, young_max=ymax, seed=int(toks[p + 16]), angle_deg=ang,
                              n_elements=None if nel == "CONFORMING" else int(float(nel)),
                              clamped=(bc == "CLAMPED"), ID=ID, number=n, dx=dx, dy=dy))
            p += 17
        else:
            # The reference silently ignores an unknown keyword's line; we do not
            # guess a token count for it.
            raise ValueError(f"unknown geometry keyword {kw!r}")
    return out


_PACK_FIELDS = [
    # (name, kind) in the order life_params_dump prints them
    ("Nx", "i"), ("Ny", "i"), ("height_p", "d"), ("rho_p", "d"), ("nu_p", "d"), ("omega", "d"),
    ("ux0_p", "d"), ("uy0_p", "d"), ("gravityX", "d"), ("gravityY", "d"), ("dpdx", "d"),
    ("dpdy", "d"), ("wall_left", "i"), ("wall_right", "i"), ("wall_bottom", "i"),
    ("wall_top", "i"), ("profile", "i"), ("uxInlet_p", "d"), ("uyInlet_p", "d"),
    ("alpha", "d"), ("delta", "d"), ("relaxMax", "d"), ("subTol", "d"),
    ("central_moments", "i"), ("has_inlet_ramp", "i"), ("inlet_ramp", "d"),
    ("has_womersley", "i"), ("womersley", "d"), ("uni_epsilon", "i"), ("ordered", "i"),
    ("has_initial_deflect", "i"), ("initial_deflect", "d"), ("nSteps", "i"), ("tinfo", "i"),
    ("tVTK", "i"), ("tRestart", "i"), ("ref_nu", "d"), ("ref_rho", "d"), ("ref_P", "d"),
    ("ref_L", "d"), ("ref_U", "d"),
]


def load_params_h(path: str, cxx: str = "g++") -> CaseParams:
    """Read the exact values of a reference ``params.h`` by compiling it.

    The header's constant expressions (``omega`` from ``tStep``, ``nSteps / 50``
    and so on) are evaluated by a C++ compiler exactly as in the reference
    build; ``include/life_params_pack.h`` prints them as hexadecimal floats.
    """
    here = os.path.dirname(os.path.abspath(__file__))
    inc = os.path.join(os.path.dirname(here), "include")
    src = ('#include "life_params_pack.h"\n#include <cstdio>\nint main(){\n'
           ' LifeCaseParams p; life_pack_params(&p);\n life_print_params(&p, stdout);\n return 0; }\n')
    with tempfile.TemporaryDirectory() as td:
        cpp = os.path.join(td, "dump.cpp")
        exe = os.path.join(td, "dump")
        with open(cpp, "w") as fh:
            fh.write(src)
        subprocess.run([cxx, "-std=c++17", "-O0", "-I", inc, "-I", os.path.join(inc, "life_ref_defs"),
                        "-include", os.path.abspath(path), "-o", exe, cpp], check=True,
                       capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    vals = {}
    for (name, kind), tok in zip(_PACK_FIELDS, out):
        vals[name] = int(tok) if kind == "i" else float.fromhex(tok)
    kw = {k: vals[k] for k in ("Nx", "Ny", "height_p", "rho_p", "nu_p", "omega", "ux0_p", "uy0_p",
                              "gravityX", "gravityY", "dpdx", "dpdy", "wall_left", "wall_right",
                              "wall_bottom", "wall_top", "uxInlet_p", "uyInlet_p", "alpha",
                              "delta", "relaxMax", "subTol", "nSteps", "tinfo", "tVTK",
                              "tRestart", "ref_nu", "ref_rho", "ref_P", "ref_L", "ref_U")}
    kw["profile"] = None if vals["profile"] < 0 else vals["profile"]
    kw["central_moments"] = bool(vals["central_moments"])
    kw["inlet_ramp"] = vals["inlet_ramp"] if vals["has_inlet_ramp"] else None
    kw["womersley"] = vals["womersley"] if vals["has_womersley"] else None
    kw["uni_epsilon"] = bool(vals["uni_epsilon"])
    kw["ordered"] = bool(vals["ordered"])
    kw["initial_deflect"] = vals["initial_deflect"] if vals["has_initial_deflect"] else None
    return CaseParams(**kw)


def _double_bits(x: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", x))[0]
