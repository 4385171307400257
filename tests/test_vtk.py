"""VTK writer format (life_gb300/vtk.py) against the files the reference
itself wrote (tests/golden/make_vtk.py), with the CPU oracle as the data
source: the oracle is bit-identical to the reference on these cases, so the
writer must reproduce every byte (XML text, offsets, raw arrays). The GPU
data path is checked the same way in tests/test_gpu_vtk.py."""
import hashlib
import os
from types import SimpleNamespace

import numpy as np
import pytest

from cases import golden_cases

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


class OracleView:
    """The slice of life_gb300.lib.Case that the VTK writer reads, served by
    the oracle (reference layout converted to VTK order here, with the
    reference's operation order)."""

    def __init__(self, o, p, bodies):
        self.o, self.p, self.body_list = o, p, bodies

    @property
    def t(self):
        return self.o.t

    def info(self):
        p = self.p
        cs = 1.0 / np.sqrt(3.0)
        nu = (1.0 / p.omega - 0.5) * (cs * cs)
        Dx = p.height_p / (p.Ny - 1)
        Dt = (Dx * Dx) * nu / p.nu_p
        Drho = p.rho_p / 1.0
        Dm = (p.rho_p / 1.0) * (Dx * Dx * Dx)
        return SimpleNamespace(Nx=p.Nx, Ny=p.Ny, Dx=Dx, Dt=Dt, Dm=Dm, Drho=Drho, c_s=cs,
                               n_markers=self.o.n_markers, n_flex=self.o.n_flex, n_bodies=self.o.n_bodies)

    def vtk_fields(self):
        i = self.info()
        p = self.p
        f = self.o.fields()
        rho = f["rho"].reshape(p.Nx, p.Ny).T.ravel()
        u = f["u"].reshape(p.Nx, p.Ny, 2).transpose(1, 0, 2).reshape(-1, 2)
        dens = rho * i.Drho
        pres = p.ref_P + (rho - p.rho_p / i.Drho) * (i.c_s * i.c_s) * i.Dm / (i.Dx * (i.Dt * i.Dt))
        vel = np.zeros((len(rho), 3))
        vel[:, 0] = u[:, 0] * (i.Dx / i.Dt)
        vel[:, 1] = u[:, 1] * (i.Dx / i.Dt)
        return dens, pres, vel

    def bodies(self):
        return self.o.bodies()

    def body_nodes(self):
        from life_gb300.case import CIRCLE_KIND, FILAMENT_KIND, Circle
        kinds = []
        for b in self.body_list:
            kinds += [CIRCLE_KIND if isinstance(b, Circle) else FILAMENT_KIND] * b.number
        return np.array(kinds), np.arange(self.o.n_markers)

    def markers(self):
        return self.o.markers()

    def fem(self, k):
        return self.o.fem(k)


@pytest.mark.parametrize("name", ["cavity_cm", "cylinder_rigid_cm"])
def test_vtk_files_byte_identical_with_reference(name):
    from life_gb300 import vtk
    from oracle.pyoracle import Oracle
    p, b = golden_cases()[name]
    g = np.load(os.path.join(GOLD, f"vtk_{name}.npz"))
    o = Oracle(p, b)
    view = OracleView(o, p, b)
    for t in (0, p.nSteps // 2, p.nSteps):
        o.step(t - o.t)
        data = {f"Fluid.{t}.vti": vtk.fluid_vti_bytes(view)}
        if b:
            data[f"IBM.{t}.vtp"] = vtk.bodies_vtp_bytes(view)
        for fname, got in data.items():
            key = fname.replace(".", "_")
            assert len(got) == int(g["size_" + key]), fname
            assert hashlib.sha256(got).hexdigest() == str(g["sha_" + key]), fname
    o.close()


def test_empty_vtp_format():
    from life_gb300 import vtk
    text = vtk.empty_vtp_bytes().decode()
    assert text.startswith('<?xml version="1.0"?>\n<VTKFile type="PolyData"')
    assert '<Piece NumberOfPoints="0" NumberOfVerts="0" NumberOfLines="0"' in text
    assert text.endswith("</VTKFile>\n")
