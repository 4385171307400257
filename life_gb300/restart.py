"""Readers and writers for LIFE's binary restart files.

The layouts follow the reference writers field by field (native byte order,
no padding):

* ``Fluid.restart`` -- ``GridClass::writeRestart`` (reference
  ``src/Grid.cpp:1163-1229``): ``int t, Nx, Ny; double omega, Dx, Dt, Dm``,
  then for every site in ``i``-major, ``j``-minor order
  ``int i, j; double rho, ux, uy, fx_ibm, fy_ibm, f[9]``.
* ``IBM.restart`` -- ``ObjectsClass::writeRestart`` (``src/Objects.cpp:1208-1265``):
  ``size_t nBodies``; per body ``int ID; size_t nNodes``; per marker
  ``double pos[2], vel[2], force[2]``.
* ``FEM.restart`` -- ``src/Objects.cpp:1267-1370``: ``int nFlex; double relax``;
  per flexible body ``int ID; size_t nEl, nNode``; then ``U, Udot, Udotdot, U_n,
  U_nm1, R_k`` (``3*nNode`` doubles each); per element ``double L, angle``; per
  node ``double pos0[2], pos[2], angle0, angle``.

Fields are returned in the reference's site order (``id = i*Ny + j``).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field
from typing import Dict, List

import numpy as np

_FLUID_SITE = np.dtype([("i", "<i4"), ("j", "<i4"), ("rho", "<f8"), ("u", "<f8", (2,)),
                        ("fibm", "<f8", (2,)), ("f", "<f8", (9,))])


@dataclass
class FluidRestart:
    t: int
    Nx: int
    Ny: int
    omega: float
    Dx: float
    Dt: float
    Dm: float
    rho: np.ndarray        # (Nx*Ny,)
    u: np.ndarray          # (Nx*Ny, 2)
    force_ibm: np.ndarray  # (Nx*Ny, 2)
    f: np.ndarray          # (Nx*Ny, 9)


def read_fluid_restart(path: str) -> FluidRestart:
    raw = open(path, "rb").read()
    t, nx, ny = struct.unpack_from("<3i", raw, 0)
    omega, dx, dt, dm = struct.unpack_from("<4d", raw, 12)
    sites = np.frombuffer(raw, dtype=_FLUID_SITE, offset=44, count=nx * ny)
    ii = np.repeat(np.arange(nx), ny)
    jj = np.tile(np.arange(ny), nx)
    if not (np.array_equal(sites["i"], ii) and np.array_equal(sites["j"], jj)):
        raise ValueError("Grid indices do not match Fluid.restart file...exiting")
    return FluidRestart(t, nx, ny, omega, dx, dt, dm, sites["rho"].copy(), sites["u"].copy(),
                        sites["fibm"].copy(), sites["f"].copy())


def write_fluid_restart(path: str, r: FluidRestart) -> None:
    n = r.Nx * r.Ny
    sites = np.zeros(n, dtype=_FLUID_SITE)
    sites["i"] = np.repeat(np.arange(r.Nx), r.Ny)
    sites["j"] = np.tile(np.arange(r.Ny), r.Nx)
    sites["rho"] = r.rho
    sites["u"] = r.u
    sites["fibm"] = r.force_ibm
    sites["f"] = r.f
    with open(path, "wb") as fh:
        fh.write(struct.pack("<3i", r.t, r.Nx, r.Ny))
        fh.write(struct.pack("<4d", r.omega, r.Dx, r.Dt, r.Dm))
        fh.write(sites.tobytes())


@dataclass
class IBMRestart:
    ids: List[int]
    pos: List[np.ndarray]    # per body (n, 2)
    vel: List[np.ndarray]
    force: List[np.ndarray]


def read_ibm_restart(path: str) -> IBMRestart:
    raw = open(path, "rb").read()
    (nb,) = struct.unpack_from("<Q", raw, 0)
    off = 8
    out = IBMRestart([], [], [], [])
    for _ in range(nb):
        (bid,) = struct.unpack_from("<i", raw, off)
        (nn,) = struct.unpack_from("<Q", raw, off + 4)
        off += 12
        a = np.frombuffer(raw, dtype="<f8", count=6 * nn, offset=off).reshape(nn, 6)
        off += 48 * nn
        out.ids.append(bid)
        out.pos.append(a[:, 0:2].copy())
        out.vel.append(a[:, 2:4].copy())
        out.force.append(a[:, 4:6].copy())
    return out


def write_ibm_restart(path: str, r: IBMRestart) -> None:
    with open(path, "wb") as fh:
        fh.write(struct.pack("<Q", len(r.ids)))
        for bid, p, v, f in zip(r.ids, r.pos, r.vel, r.force):
            fh.write(struct.pack("<iQ", bid, len(p)))
            fh.write(np.ascontiguousarray(np.hstack([p, v, f]), dtype="<f8").tobytes())


@dataclass
class FEMBodyRestart:
    ID: int
    U: np.ndarray
    Udot: np.ndarray
    Udotdot: np.ndarray
    U_n: np.ndarray
    U_nm1: np.ndarray
    R_k: np.ndarray
    el_L: np.ndarray       # (nEl,)
    el_angle: np.ndarray   # (nEl,)
    pos0: np.ndarray       # (nNode, 2)
    pos: np.ndarray        # (nNode, 2)
    angle0: np.ndarray     # (nNode,)
    angle: np.ndarray      # (nNode,)


@dataclass
class FEMRestart:
    relax: float
    bodies: List[FEMBodyRestart] = field(default_factory=list)


def read_fem_restart(path: str) -> FEMRestart:
    raw = open(path, "rb").read()
    (nflex,) = struct.unpack_from("<i", raw, 0)
    (relax,) = struct.unpack_from("<d", raw, 4)
    off = 12
    out = FEMRestart(relax)
    for _ in range(nflex):
        (bid,) = struct.unpack_from("<i", raw, off)
        nel, nnode = struct.unpack_from("<2Q", raw, off + 4)
        off += 20
        dofs = 3 * nnode
        vecs = []
        for _k in range(6):
            vecs.append(np.frombuffer(raw, "<f8", dofs, off).copy())
            off += 8 * dofs
        el = np.frombuffer(raw, "<f8", 2 * nel, off).reshape(nel, 2).copy()
        off += 16 * nel
        nd = np.frombuffer(raw, "<f8", 6 * nnode, off).reshape(nnode, 6).copy()
        off += 48 * nnode
        out.bodies.append(FEMBodyRestart(bid, *vecs, el[:, 0].copy(), el[:, 1].copy(),
                                         nd[:, 0:2].copy(), nd[:, 2:4].copy(),
                                         nd[:, 4].copy(), nd[:, 5].copy()))
    return out


def write_fem_restart(path: str, r: FEMRestart) -> None:
    with open(path, "wb") as fh:
        fh.write(struct.pack("<id", len(r.bodies), r.relax))
        for b in r.bodies:
            fh.write(struct.pack("<iQQ", b.ID, len(b.el_L), len(b.pos0)))
            for v in (b.U, b.Udot, b.Udotdot, b.U_n, b.U_nm1, b.R_k):
                fh.write(np.ascontiguousarray(v, dtype="<f8").tobytes())
            fh.write(np.ascontiguousarray(np.stack([b.el_L, b.el_angle], 1), "<f8").tobytes())
            nd = np.hstack([b.pos0, b.pos, b.angle0[:, None], b.angle[:, None]])
            fh.write(np.ascontiguousarray(nd, "<f8").tobytes())


def save_case(case, directory: str) -> None:
    """Writes a running case's state as the reference's restart set:
    ``Fluid.restart``, and ``IBM.restart`` / ``FEM.restart`` when it has
    bodies (ObjectsClass::writeRestart, reference src/Objects.cpp:1206-1371)."""
    import os
    os.makedirs(directory, exist_ok=True)
    inf = case.info()
    fl = case.fields()
    write_fluid_restart(os.path.join(directory, "Fluid.restart"), FluidRestart(
        inf.t, inf.Nx, inf.Ny, case.params.omega, inf.Dx, inf.Dt, inf.Dm,
        fl["rho"], fl["u"], fl["force_ibm"], fl["f"]))
    if not case.n_markers:
        return
    b = case.bodies()
    mk = case.markers()
    ibm = IBMRestart([], [], [], [])
    start = 0
    for ib in range(len(b["ids"])):
        n = int(b["n_markers"][ib])
        sl = slice(start, start + n)
        ibm.ids.append(int(b["ids"][ib]))
        ibm.pos.append(mk["pos"][sl])
        ibm.vel.append(mk["vel"][sl])
        ibm.force.append(mk["force"][sl])
        start += n
    write_ibm_restart(os.path.join(directory, "IBM.restart"), ibm)
    flex = [ib for ib in range(len(b["ids"])) if b["flexible"][ib]]
    if not flex:
        return
    fem = FEMRestart(case.relax())
    for k, ib in enumerate(flex):
        d = case.fem(k)
        fem.bodies.append(FEMBodyRestart(int(b["ids"][ib]), d["U"], d["Udot"], d["Udotdot"], d["U_n"], d["U_nm1"],
                                         d["R_k"], d["el_L"], d["el_angle"], d["pos0"], d["pos"], d["angle0"],
                                         d["angle"]))
    write_fem_restart(os.path.join(directory, "FEM.restart"), fem)


def load_case(case, directory: str) -> int:
    """Loads a restart set into a freshly created case of the same geometry,
    with the reference's rules (Utils::readRestart, src/Utils.cpp:82-101;
    GridClass::readRestart, src/Grid.cpp:1072-1160; ObjectsClass::readRestart,
    src/Objects.cpp:979-1203): bodies are matched by ID, bodies missing from
    the case are skipped, a marker or node count that differs is an error.
    Returns the restart time step."""
    import os
    fr = read_fluid_restart(os.path.join(directory, "Fluid.restart"))
    if (fr.Nx, fr.Ny) != (case.params.Nx, case.params.Ny):
        raise ValueError("Fluid.restart lattice does not match the case")
    case.set_fields(fr.t, fr.rho, fr.u, fr.f, fr.force_ibm)
    ipath, fpath = os.path.join(directory, "IBM.restart"), os.path.join(directory, "FEM.restart")
    if case.n_markers and os.path.exists(ipath):
        b = case.bodies()
        mk = case.markers()
        starts = np.concatenate([[0], np.cumsum(b["n_markers"])])
        byid = {int(bid): ib for ib, bid in enumerate(b["ids"])}
        ir = read_ibm_restart(ipath)
        for bid, p, v, f in zip(ir.ids, ir.pos, ir.vel, ir.force):
            ib = byid.get(bid)
            if ib is None:
                continue
            sl = slice(int(starts[ib]), int(starts[ib + 1]))
            if len(p) != sl.stop - sl.start:
                raise ValueError("Number of nodes in IBM.restart do not match existing number of nodes")
            mk["pos"][sl], mk["vel"][sl], mk["force"][sl] = p, v, f
        case.set_markers(mk["pos"], mk["vel"], mk["force"])
    if case.n_flex and os.path.exists(fpath):
        b = case.bodies()
        flex = [ib for ib in range(len(b["ids"])) if b["flexible"][ib]]
        kof = {int(b["ids"][ib]): k for k, ib in enumerate(flex)}
        fr2 = read_fem_restart(fpath)
        case.set_relax(fr2.relax)
        for fb in fr2.bodies:
            k = kof.get(fb.ID)
            if k is None:
                continue
            if len(fb.pos) != int(b["n_fem_nodes"][flex[k]]):
                raise ValueError("Number of nodes/elements in FEM.restart do not match existing number")
            case.set_fem(k, fb.U, fb.Udot, fb.Udotdot, fb.U_n, fb.U_nm1, fb.R_k, fb.el_L, fb.el_angle,
                         fb.pos0, fb.pos, fb.angle0, fb.angle)
    return fr.t
