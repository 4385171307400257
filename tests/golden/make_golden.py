#!/usr/bin/env python3
"""Generate the golden parity fixtures by running the LIFE reference itself.

For every case in ``cases.py`` this script

1. writes the case's ``params.h`` and ``input/geometry.config``,
2. compiles the unmodified reference sources with that ``params.h``
   (``make -C oracle ref``; the recipe reads the sources in place),
3. runs the binary single-threaded (``ORDERED`` reductions, deterministic), and
4. stores the restart dump it writes at the last step (``Fluid.restart``,
   ``IBM.restart``, ``FEM.restart`` -- full-precision binary doubles) as
   ``tests/golden/<case>.npz``.

It needs the reference tree (``LIFE_REFERENCE``, else a checkout named
``reference`` beside this repository) and is run by hand when the case list changes:

    python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

from cases import golden_cases  # noqa: E402
from life_gb300.case import geometry_config_text  # noqa: E402
from life_gb300.restart import read_fem_restart, read_fluid_restart, read_ibm_restart  # noqa: E402

REF = os.environ.get("LIFE_REFERENCE") or os.path.join(os.path.dirname(REPO), "reference")


def params_digest(text: str) -> str:
    return hashlib.sha256(text.encode()).hexdigest()[:16]


def array_digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def run_case(name: str, params, bodies, work: str, lapack: str = "openblas", threads: int = 1) -> dict:
    cdir = os.path.join(work, name + lapack, "case")
    rdir = os.path.join(work, name + lapack, "run")
    os.makedirs(cdir, exist_ok=True)
    os.makedirs(os.path.join(rdir, "input"), exist_ok=True)
    ptext = params.to_params_h()
    with open(os.path.join(cdir, "params.h"), "w") as fh:
        fh.write(ptext)
    if bodies:
        with open(os.path.join(rdir, "input", "geometry.config"), "w") as fh:
            fh.write(geometry_config_text(bodies))
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(REPO, "oracle"), "ref",
                    f"CASE={cdir}", f"NAME=golden_{name}_{lapack}", f"REF={REF}",
                    f"LAPACK={lapack}"], check=True)
    exe = os.path.join(REPO, "oracle", "_ref", f"golden_{name}_{lapack}", "LIFE")
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), OPENBLAS_NUM_THREADS="1")
    log = subprocess.run([exe], cwd=rdir, env=env, capture_output=True, text=True)
    if log.returncode != 0:
        raise RuntimeError(f"{name}: reference exited {log.returncode}\n{log.stdout[-2000:]}")
    rs = os.path.join(rdir, "Results", "Restart")
    fl = read_fluid_restart(os.path.join(rs, "Fluid.restart"))
    out = dict(t=fl.t, f=fl.f, rho=fl.rho, u=fl.u, force_ibm=fl.force_ibm,
               Dx=fl.Dx, Dt=fl.Dt, Dm=fl.Dm, omega=fl.omega,
               params_digest=params_digest(ptext))
    ibm_path = os.path.join(rs, "IBM.restart")
    if os.path.exists(ibm_path):
        ib = read_ibm_restart(ibm_path)
        out.update(ibm_ids=np.array(ib.ids), ibm_counts=np.array([len(p) for p in ib.pos]),
                   ibm_pos=np.vstack(ib.pos), ibm_vel=np.vstack(ib.vel),
                   ibm_force=np.vstack(ib.force))
    fem_path = os.path.join(rs, "FEM.restart")
    if os.path.exists(fem_path):
        fe = read_fem_restart(fem_path)
        out.update(fem_relax=fe.relax, fem_ids=np.array([b.ID for b in fe.bodies]),
                   fem_nnode=np.array([len(b.pos0) for b in fe.bodies]))
        for key in ("U", "Udot", "Udotdot", "U_n", "U_nm1", "R_k", "el_L", "el_angle",
                    "angle0", "angle"):
            out["fem_" + key] = np.concatenate([getattr(b, key) for b in fe.bodies])
        out["fem_pos0"] = np.vstack([b.pos0 for b in fe.bodies])
        out["fem_pos"] = np.vstack([b.pos for b in fe.bodies])
    vdir = os.path.join(rdir, "Results", "VTK")
    if os.path.isdir(vdir):
        out["vtk_files"] = {name: open(os.path.join(vdir, name), "rb").read() for name in sorted(os.listdir(vdir))}
    for key, fname in (("total_forces_text", "TotalForces.out"), ("tip_positions_text", "TipPositions.out"),
                       ("tip_velocities_text", "TipVelocities.out")):
        path = os.path.join(rdir, "Results", fname)
        if os.path.exists(path):
            out[key] = open(path).read()
    return out


def main(argv) -> int:
    if not os.path.isdir(os.path.join(REF, "src")):
        print(f"reference tree not found at {REF}", file=sys.stderr)
        return 2
    cases = golden_cases()
    names = argv[1:] or list(cases)
    work = tempfile.mkdtemp(prefix="life_golden_")
    try:
        for name in names:
            params, bodies = cases[name]
            res = run_case(name, params, bodies, work)
            # Same case with the reference linked against the textbook LU shim:
            # its dumps must equal the oracle's bit for bit (stored as digests).
            tb = run_case(name, params, bodies, work, lapack="textbook")
            for key in ("f", "rho", "u", "force_ibm", "ibm_pos", "ibm_vel", "ibm_force",
                        "fem_U", "fem_Udot", "fem_pos"):
                if key in tb:
                    res["sha_textbook_" + key] = array_digest(tb[key])
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **res)
            print(f"{name}: t={res['t']} sites={len(res['rho'])}"
                  + (f" markers={len(res['ibm_pos'])}" if "ibm_pos" in res else "")
                  + (f" fem_nodes={int(res['fem_nnode'].sum())}" if "fem_nnode" in res else ""))
    finally:
        shutil.rmtree(work, ignore_errors=True)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
