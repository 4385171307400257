"""The seeded synthetic workloads and the benchmark's analysis helpers (CPU).

The ensemble generator must keep the properties its documentation states
(sizes, body counts, filament spacing out of each other's reach, thin
sections, the stiffness range) and be reproducible from its seed; the canopy
generator likewise. The shedding-period helper must recover a known period.
"""
import math

import numpy as np
import pytest

from life_gb300.case import Circle, Filament
from life_gb300.ensemble import THICKNESS, canopy_case, ensemble_cases, filament_modulus, sites


def test_ensemble_is_reproducible_and_sized():
    a, b = ensemble_cases(), ensemble_cases()
    assert len(a) == 64
    assert sites(a) == sites(b)
    for (p, bodies), (q, bodies2) in zip(a, b):
        assert (p.Nx, p.Ny, p.omega, p.central_moments) == (q.Nx, q.Ny, q.omega, q.central_moments)
        assert [(x.x, x.y) for x in bodies] == [(x.x, x.y) for x in bodies2]
        assert 256 <= p.Nx <= 2048 and p.Nx % 32 == 0
        assert 128 <= p.Ny <= 512 and p.Ny % 32 == 0
        assert 1.0 / p.omega >= 0.53 - 1e-12


@pytest.mark.parametrize("k", range(64))
def test_ensemble_bodies_keep_their_spacing(k):
    p, bodies = ensemble_cases()[k]
    fil = [x for x in bodies if isinstance(x, Filament)]
    cyl = [x for x in bodies if isinstance(x, Circle)]
    assert not (fil and cyl)
    assert len(cyl) <= 4 and len(fil) <= 8
    for c in cyl:
        assert 8.0 <= c.radius <= 24.0
        assert c.radius <= p.Ny / 6.0 + 1e-9
        assert c.x + 2.0 * c.radius <= 0.75 * p.Nx + 1e-9
    if not fil:
        return
    lmax = max(f.length for f in fil)
    for f in fil:
        assert 20 <= f.length <= 60 and f.n_elements == int(f.length)
        assert f.height == THICKNESS and f.clamped and f.flexible
        # bending stiffness EI / (rho U^2 L^3) with I = H^3/12, rho_f = 1
        K = f.E * f.height ** 3 / 12.0 / (p.uxInlet_p ** 2 * f.length ** 3)
        assert 1e-2 * (1 - 1e-9) <= K <= 1e-1 * (1 + 1e-9)
        assert f.x + f.length <= p.Nx  # inside the lattice
    xs = sorted({round(f.x, 6) for f in fil})
    ys = sorted({round(f.y, 6) for f in fil})
    for a, b in zip(xs, xs[1:]):
        assert b - a >= 2.5 * lmax - 1e-6  # columns out of each other's near wake
    for a, b in zip(ys, ys[1:]):
        assert b - a >= lmax - 1e-6  # rows at least one length apart


def test_filament_modulus_is_the_stated_stiffness():
    E = filament_modulus(0.05, 0.04, 30.0)
    assert math.isclose(E * THICKNESS ** 3 / 12.0 / (0.04 ** 2 * 30.0 ** 3), 0.05, rel_tol=1e-12)


def test_canopy_requests():
    rng = np.random.Generator(np.random.PCG64(7))
    for _ in range(20):
        p, bodies, steps = canopy_case(rng)
        assert 512 <= p.Nx <= 4096 and 256 <= p.Ny <= 1024
        assert 2000 <= steps <= 20000
        assert 1 <= len(bodies) <= 32
        xs = [b.x for b in bodies]
        assert xs == sorted(xs)
        for b in bodies:
            assert b.angle_deg == 90.0 and b.y == 0.0 and b.n_elements == 20
            assert 20.0 <= b.length <= 40.0


def test_shedding_period_helper_recovers_a_period():
    import bench
    t = np.arange(0, 20000, 25, dtype=float)
    y = 0.3 * np.sin(2 * np.pi * t / 3600.0 + 0.4) + 0.01
    up = bench._upward_crossings(t, y)
    assert len(up) >= 4
    assert abs(np.mean(np.diff(up)) - 3600.0) < 1.0
