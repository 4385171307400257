"""The restart writers and readers (``life_gb300/restart.py``) on the host:
each file written from seeded data reads back to the same values, with the
byte layout of the reference's writers (native little-endian, no padding):
Fluid.restart a 44-byte header and 120 bytes per site in i-major order
(GridClass::writeRestart, src/Grid.cpp:1163-1229), IBM.restart a size_t body
count and per body an int ID, a size_t marker count and 48 bytes per marker
(ObjectsClass::writeRestart, src/Objects.cpp:1208-1265), FEM.restart an int
count, the double relaxation factor and per body the six DOF vectors, two
doubles per element and six per node (src/Objects.cpp:1267-1370). The readers
are also checked against files the reference binary wrote
(``tests/test_oracle_golden.py``, ``tests/test_drop_in_driver.py``)."""
import struct

import numpy as np
import pytest

from life_gb300.restart import (FEMBodyRestart, FEMRestart, FluidRestart, IBMRestart, read_fem_restart,
                                read_fluid_restart, read_ibm_restart, write_fem_restart, write_fluid_restart,
                                write_ibm_restart)


def fluid(nx=7, ny=5, seed=1):
    g = np.random.default_rng(seed)
    n = nx * ny
    return FluidRestart(t=4242, Nx=nx, Ny=ny, omega=1.0 / 0.62, Dx=0.0125, Dt=3.1e-4, Dm=1.9e-6,
                        rho=1.0 + 1e-3 * g.standard_normal(n), u=1e-2 * g.standard_normal((n, 2)),
                        force_ibm=1e-5 * g.standard_normal((n, 2)), f=g.random((n, 9)))


def test_fluid_restart_round_trip_and_layout(tmp_path):
    r = fluid()
    path = tmp_path / "Fluid.restart"
    write_fluid_restart(str(path), r)
    raw = path.read_bytes()
    assert len(raw) == 44 + r.Nx * r.Ny * 120
    assert struct.unpack_from("<3i", raw, 0) == (r.t, r.Nx, r.Ny)
    assert struct.unpack_from("<4d", raw, 12) == (r.omega, r.Dx, r.Dt, r.Dm)
    # the second record is site (i, j) = (0, 1): j is the inner index
    assert struct.unpack_from("<2i", raw, 44 + 120) == (0, 1)
    assert struct.unpack_from("<d", raw, 44 + 120 + 8)[0] == r.rho[1]
    back = read_fluid_restart(str(path))
    assert (back.t, back.Nx, back.Ny) == (r.t, r.Nx, r.Ny)
    assert (back.omega, back.Dx, back.Dt, back.Dm) == (r.omega, r.Dx, r.Dt, r.Dm)
    for key in ("rho", "u", "force_ibm", "f"):
        assert np.array_equal(getattr(back, key), getattr(r, key)), key


def test_fluid_restart_with_shuffled_sites_is_rejected(tmp_path):
    r = fluid()
    path = tmp_path / "Fluid.restart"
    write_fluid_restart(str(path), r)
    raw = bytearray(path.read_bytes())
    struct.pack_into("<i", raw, 44 + 120 + 4, 3)  # record 1 claims j = 3
    path.write_bytes(bytes(raw))
    with pytest.raises(ValueError, match="Grid indices do not match"):
        read_fluid_restart(str(path))


def test_ibm_restart_round_trip_and_layout(tmp_path):
    g = np.random.default_rng(2)
    sizes = [5, 1, 12]
    r = IBMRestart(ids=[0, 7, 3], pos=[g.random((n, 2)) * 100 for n in sizes],
                   vel=[g.standard_normal((n, 2)) for n in sizes], force=[g.standard_normal((n, 2)) for n in sizes])
    path = tmp_path / "IBM.restart"
    write_ibm_restart(str(path), r)
    raw = path.read_bytes()
    assert len(raw) == 8 + sum(12 + 48 * n for n in sizes)
    assert struct.unpack_from("<Q", raw, 0)[0] == 3
    assert struct.unpack_from("<iQ", raw, 8) == (0, 5)
    back = read_ibm_restart(str(path))
    assert back.ids == r.ids
    for key in ("pos", "vel", "force"):
        for a, b in zip(getattr(back, key), getattr(r, key)):
            assert np.array_equal(a, b), key


def test_fem_restart_round_trip_and_layout(tmp_path):
    g = np.random.default_rng(3)
    bodies = []
    for bid, nnode in ((2, 11), (5, 4)):
        dofs, nel = 3 * nnode, nnode - 1
        vec = lambda: g.standard_normal(dofs)
        bodies.append(FEMBodyRestart(bid, vec(), vec(), vec(), vec(), vec(), vec(), g.random(nel), g.standard_normal(nel),
                                     g.random((nnode, 2)), g.random((nnode, 2)), g.standard_normal(nnode),
                                     g.standard_normal(nnode)))
    r = FEMRestart(relax=0.37, bodies=bodies)
    path = tmp_path / "FEM.restart"
    write_fem_restart(str(path), r)
    raw = path.read_bytes()
    expect = 12 + sum(20 + 6 * 8 * 3 * len(b.pos0) + 16 * len(b.el_L) + 48 * len(b.pos0) for b in bodies)
    assert len(raw) == expect
    assert struct.unpack_from("<i", raw, 0)[0] == 2 and struct.unpack_from("<d", raw, 4)[0] == 0.37
    assert struct.unpack_from("<iQQ", raw, 12) == (2, 10, 11)
    back = read_fem_restart(str(path))
    assert back.relax == r.relax and len(back.bodies) == 2
    for a, b in zip(back.bodies, bodies):
        assert a.ID == b.ID
        for key in ("U", "Udot", "Udotdot", "U_n", "U_nm1", "R_k", "el_L", "el_angle", "pos0", "pos", "angle0",
                    "angle"):
            assert np.array_equal(getattr(a, key), getattr(b, key)), key
