"""VTK output in the reference's exact file format.

* ``Results/VTK/Fluid.<t>.vti`` -- ``GridClass::writeVTK`` (reference
  ``src/Grid.cpp:790-913``): XML ImageData with three appended raw Float64
  arrays (Density, Pressure, 3-component Velocity), each preceded by its byte
  count as a UInt64, points in x-fastest order.
* ``Results/VTK/IBM.<t>.vtp`` and ``FEM.<t>.vtp`` -- ``ObjectsClass::writeVTK``
  (``src/Objects.cpp:710-865``): XML PolyData, one Piece per body (IBM: every
  body's markers; FEM: the flexible bodies' FEM nodes), points and line
  connectivity appended raw; a circle's outline is closed.
* ``writeEmptyVTK`` (``src/Objects.cpp:1462-1508``): the empty PolyData file.

The field arrays come from the device already converted and in VTK point
order (``life_case_get_vtk_fields``); the bodies from the marker and FEM
getters. Numbers in the XML text follow C++ stream defaults (6 significant
digits, ``%g``), as the reference's ``ofstream`` prints them, and the raw data
is little-endian, so a file written here is byte for byte the reference's
file for the same state.
"""
from __future__ import annotations

import os
import struct
import sys
from typing import List

import numpy as np

ENDIAN = "LittleEndian" if sys.byteorder == "little" else "BigEndian"
_U64 = struct.Struct("<Q" if sys.byteorder == "little" else ">Q")


def _g(x: float) -> str:
    return format(float(x), "g")


def fluid_vti_bytes(case) -> bytes:
    """Bytes of ``Fluid.<t>.vti`` for the case's current state."""
    info = case.info()
    nx, ny, dx = info.Nx, info.Ny, info.Dx
    dens, pres, vel = case.vtk_fields()
    n8 = nx * ny * 8
    head = [
        '<?xml version="1.0"?>\n',
        f'<VTKFile type="ImageData" version="1.0" byte_order="{ENDIAN}" header_type="UInt64">\n',
        f'\t<ImageData WholeExtent="0 {nx - 1} 0 {ny - 1} 0 0" Origin="0 0 0" '
        f'Spacing="{_g(dx)} {_g(dx)} {_g(dx)}">\n',
        f'\t\t<Piece Extent="0 {nx - 1} 0 {ny - 1} 0 0">\n',
        "\t\t\t<PointData>\n",
        '\t\t\t\t<DataArray type="Float64" Name="Density" format="appended" offset="0"/>\n',
        f'\t\t\t\t<DataArray type="Float64" Name="Pressure" format="appended" offset="{1 * (n8 + 8)}"/>\n',
        f'\t\t\t\t<DataArray type="Float64" Name="Velocity" NumberOfComponents="3" format="appended" '
        f'offset="{2 * (n8 + 8)}"/>\n',
        "\t\t\t</PointData>\n",
        "\t\t</Piece>\n",
        "\t</ImageData>\n",
        '\t<AppendedData encoding="raw">\n',
        "\t\t_",
    ]
    parts: List[bytes] = ["".join(head).encode()]
    for arr, nbytes in ((dens, n8), (pres, n8), (vel, 3 * n8)):
        parts.append(_U64.pack(nbytes))
        parts.append(np.ascontiguousarray(arr, dtype="=f8").tobytes())
    parts.append(b"\n\t</AppendedData>\n</VTKFile>\n")
    return b"".join(parts)


def _polydata(pieces) -> bytes:
    """pieces: list of (points [n, 2], closed) in file order."""
    head = ['<?xml version="1.0"?>\n',
            f'<VTKFile type="PolyData" version="1.0" byte_order="{ENDIAN}" header_type="UInt64">\n',
            "\t<PolyData>\n"]
    off = 0
    for pts, closed in pieces:
        nn = len(pts)
        nl = nn if closed else nn - 1
        head.append(f'\t\t<Piece NumberOfPoints="{nn}" NumberOfVerts="0" NumberOfLines="{nl}" '
                    f'NumberOfStrips="0" NumberOfPolys="0">\n')
        head.append("\t\t\t<Points>\n")
        head.append(f'\t\t\t\t<DataArray type="Float64" Name="Points" NumberOfComponents="3" format="appended" '
                    f'offset="{off}"/>\n')
        off += 3 * nn * 8 + 8
        head.append("\t\t\t</Points>\n")
        head.append("\t\t\t<Lines>\n")
        head.append(f'\t\t\t\t<DataArray type="Int64" Name="connectivity" format="appended" offset="{off}"/>\n')
        off += 2 * nl * 8 + 8
        head.append(f'\t\t\t\t<DataArray type="Int64" Name="offsets" format="appended" offset="{off}"/>\n')
        off += nl * 8 + 8
        head.append("\t\t\t</Lines>\n")
        head.append("\t\t</Piece>\n")
    head += ["\t</PolyData>\n", '\t<AppendedData encoding="raw">\n', "\t\t_"]
    parts: List[bytes] = ["".join(head).encode()]
    for pts, closed in pieces:
        nn = len(pts)
        nl = nn if closed else nn - 1
        xyz = np.zeros((nn, 3))
        xyz[:, :2] = pts
        parts.append(_U64.pack(3 * nn * 8))
        parts.append(xyz.astype("=f8").tobytes())
        k = np.arange(nl, dtype=np.int64)
        conn = np.stack([k, (k + 1) % nn], axis=1)
        parts.append(_U64.pack(2 * nl * 8))
        parts.append(conn.astype("=i8").tobytes())
        parts.append(_U64.pack(nl * 8))
        parts.append((2 * (k + 1)).astype("=i8").tobytes())
    parts.append(b"\n\t</AppendedData>\n</VTKFile>\n")
    return b"".join(parts)


def bodies_vtp_bytes(case, fem: bool = False) -> bytes:
    """Bytes of ``IBM.<t>.vtp`` (fem=False: every body's markers) or
    ``FEM.<t>.vtp`` (fem=True: the flexible bodies' FEM nodes)."""
    from .case import CIRCLE_KIND
    b = case.bodies()
    kinds, index = case.body_nodes()
    pieces = []
    if fem:
        k = 0
        for ib in range(len(kinds)):
            if b["flexible"][ib]:
                pieces.append((case.fem(k)["pos"], False))
                k += 1
    else:
        pos = case.markers()["pos"]
        q = 0
        for ib, kind in enumerate(kinds):
            m = int(b["n_markers"][ib])
            pieces.append((pos[index[q:q + m]], kind == CIRCLE_KIND))
            q += m
    return _polydata(pieces)


def empty_vtp_bytes() -> bytes:
    return (f'<?xml version="1.0"?>\n<VTKFile type="PolyData" version="1.0" byte_order="{ENDIAN}" '
            'header_type="UInt64">\n\t<PolyData>\n\t\t<Piece NumberOfPoints="0" NumberOfVerts="0" '
            'NumberOfLines="0" NumberOfStrips="0" NumberOfPolys="0">\n\t\t</Piece>\n\t</PolyData>\n'
            '</VTKFile>\n').encode()


def write_vtk(case, directory: str = "Results/VTK", fem: bool = False) -> List[str]:
    """Utils::writeVTK (``src/Utils.cpp:150-167``) for the case's current
    state: the fluid file, then the bodies' file(s) when the case has them
    (the FEM file with fem=True, the reference's VTK_FEM). Returns the paths."""
    os.makedirs(directory, exist_ok=True)
    t = case.t
    out = []
    path = os.path.join(directory, f"Fluid.{t}.vti")
    with open(path, "wb") as fh:
        fh.write(fluid_vti_bytes(case))
    out.append(path)
    info = case.info()
    if info.n_markers > 0:
        path = os.path.join(directory, f"IBM.{t}.vtp")
        with open(path, "wb") as fh:
            fh.write(bodies_vtp_bytes(case))
        out.append(path)
        if fem and info.n_flex > 0:
            path = os.path.join(directory, f"FEM.{t}.vtp")
            with open(path, "wb") as fh:
                fh.write(bodies_vtp_bytes(case, fem=True))
            out.append(path)
    return out
