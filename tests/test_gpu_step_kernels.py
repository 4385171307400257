"""The one-launch step kernels of the reduced-precision forms (lattices of
2^22 sites or more) against each other and against the separate perimeter +
interior kernels of the host-driven loop: k_step_tma (TMA-staged tiles, the
default of both forms, LIFE_STEP_KERNEL=tma; BGK takes two sites per thread
with packed f32x2 arithmetic), k_step_lowp (one site per thread,
LIFE_STEP_KERNEL=site) and LIFE_CASE_HOSTLOOP=1 must give the same bits after
N steps, for BGK and central moments, with and without a step force, with a
convective outlet, periodic x walls and an odd width."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CODE = r"""
import hashlib, sys
sys.path.insert(0, '.')
from life_gb300.case import CaseParams, CONVECTIVE, FLUID, VELOCITY, WALL
from life_gb300.lib import Case
kind, prec = sys.argv[1], int(sys.argv[2])
omega = 1.0 / 0.56
nu = (1.0 / omega - 0.5) / 3.0
if kind == 'cavity':
    p = CaseParams(Nx=2049, Ny=2048, height_p=2047.0, rho_p=1.0, nu_p=nu, omega=omega, wall_left=WALL,
                   wall_right=WALL, wall_bottom=WALL, wall_top=VELOCITY, uxInlet_p=0.1, precision=prec)
elif kind == 'channel_cm_forced':
    p = CaseParams(Nx=2050, Ny=2048, height_p=2047.0, rho_p=1.0, nu_p=nu, omega=omega, wall_left=VELOCITY,
                   wall_right=CONVECTIVE, wall_bottom=WALL, wall_top=WALL, uxInlet_p=0.05, gravityY=-1e-6,
                   central_moments=True, inlet_ramp=10.0, precision=prec)
else:
    p = CaseParams(Nx=2048, Ny=2051, height_p=2050.0, rho_p=1.0, nu_p=nu, omega=omega, wall_left=FLUID,
                   wall_right=FLUID, wall_bottom=WALL, wall_top=WALL, gravityX=2e-6, precision=prec)
with Case(p) as c:
    c.step(30)
    fl = c.fields(("rho", "u"))
print("DIGEST", hashlib.sha256(fl["rho"].tobytes() + fl["u"].tobytes()).hexdigest())
"""


def digest(kind, prec, env):
    res = subprocess.run([sys.executable, "-c", CODE, kind, str(prec)], cwd=ROOT, capture_output=True, text=True,
                         env=dict(os.environ, **env))
    assert res.returncode == 0, res.stderr[-2000:]
    return [ln for ln in res.stdout.splitlines() if ln.startswith("DIGEST")][-1]


@pytest.mark.parametrize("kind", ["cavity", "channel_cm_forced", "periodic_x_forced"])
@pytest.mark.parametrize("prec", [1, 2])
def test_step_kernels_bit_identical(kind, prec):
    from life_gb300.build import build
    build()
    tma = digest(kind, prec, {"LIFE_STEP_KERNEL": "tma"})
    one = digest(kind, prec, {"LIFE_STEP_KERNEL": "site"})
    host = digest(kind, prec, {"LIFE_CASE_HOSTLOOP": "1"})
    assert one == host, "one-site step kernel vs host-driven kernels"
    assert tma == one, "TMA-staged step kernel vs one-site step kernel"


DIRECT = r"""
import hashlib, sys
sys.path.insert(0, '.'); sys.path.insert(0, 'tests/golden')
from cases import golden_cases
from life_gb300.case import CaseParams, VELOCITY, WALL
from life_gb300.lib import Case
name, split = sys.argv[1], [int(x) for x in sys.argv[2:]]
if name == 'cavity':
    omega = 1.0 / 0.56
    p = CaseParams(Nx=2049, Ny=2048, height_p=2047.0, rho_p=1.0, nu_p=(1.0 / omega - 0.5) / 3.0, omega=omega,
                   wall_left=WALL, wall_right=WALL, wall_bottom=WALL, wall_top=VELOCITY, uxInlet_p=0.1, precision=1)
    b = []
else:
    p, b = golden_cases()[name]
with Case(p, b) as c:
    for n in split:
        c.step(n)
    fl = c.fields(("rho", "u"))
print("DIGEST", hashlib.sha256(fl["rho"].tobytes() + fl["u"].tobytes()).hexdigest())
"""


@pytest.mark.parametrize("name", ["cavity", "cylinder_rigid_cm", "filament_flex_deflect", "womersley_gravity_cm"])
def test_direct_and_graph_steps_identical(name):
    """Runs shorter than 64 steps launch kernels directly until step graphs
    exist; 100 steps as one call (graphs), as 30 + 70 (direct, then graphs)
    and as 30 + 30 + 40 (direct throughout) end in the same bits."""
    from life_gb300.build import build
    build()
    out = []
    for split in (["100"], ["30", "70"], ["30", "30", "40"]):
        res = subprocess.run([sys.executable, "-c", DIRECT, name] + split, cwd=ROOT, capture_output=True, text=True)
        assert res.returncode == 0, res.stderr[-2000:]
        out.append([ln for ln in res.stdout.splitlines() if ln.startswith("DIGEST")][-1])
    assert out[0] == out[1] == out[2]


TIMED = r"""
import hashlib, sys
sys.path.insert(0, '.'); sys.path.insert(0, 'tests/golden')
from cases import golden_cases
from life_gb300.case import CaseParams, VELOCITY, WALL
from life_gb300.lib import Case
name, first, timed = sys.argv[1], int(sys.argv[2]), int(sys.argv[3])
if name == 'cavity':
    omega = 1.0 / 0.56
    p = CaseParams(Nx=2049, Ny=2048, height_p=2047.0, rho_p=1.0, nu_p=(1.0 / omega - 0.5) / 3.0, omega=omega,
                   wall_left=WALL, wall_right=WALL, wall_bottom=WALL, wall_top=VELOCITY, uxInlet_p=0.1, precision=1)
    b = []
else:
    p, b = golden_cases()[name]
with Case(p, b) as c:
    c.step(first)
    if timed:
        c.bench_steps(timed)
    fl = c.fields(("rho", "u", "f"))
print("DIGEST", hashlib.sha256(fl["rho"].tobytes() + fl["u"].tobytes() + fl["f"].tobytes()).hexdigest())
"""


@pytest.mark.parametrize("name", ["cavity", "cylinder_rigid_cm", "channel_convective_freeslip_cm"])
@pytest.mark.parametrize("first", [5, 6])
def test_interior_timing_leaves_the_state_untouched(name, first):
    """life_case_bench_steps times the interior launch alone after its steps;
    those extra launches write to scratch memory only, so the fields after
    first + 20 timed steps equal those of first + 20 plain steps, for either
    parity of the step graphs."""
    from life_gb300.build import build
    build()
    out = []
    for args in ([str(first), "20"], [str(first + 20), "0"]):
        res = subprocess.run([sys.executable, "-c", TIMED, name] + args, cwd=ROOT, capture_output=True, text=True)
        assert res.returncode == 0, res.stderr[-2000:]
        out.append([ln for ln in res.stdout.splitlines() if ln.startswith("DIGEST")][-1])
    assert out[0] == out[1]
