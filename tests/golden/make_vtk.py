#!/usr/bin/env python3
"""Golden VTK files written by the LIFE reference itself.

Three golden cases are rerun with ``VTK`` (and ``VTK_FEM``) switched on and
``tVTK = nSteps / 2``, so the reference writes ``Results/VTK/Fluid.<t>.vti``,
``IBM.<t>.vtp`` and ``FEM.<t>.vtp`` at t = 0, nSteps/2 and nSteps
(``GridClass::writeVTK``, ``src/Grid.cpp:790-913``; ``ObjectsClass::writeVTK``,
``src/Objects.cpp:710-865``). The bodies' cases link the textbook-LU LAPACK
shim, the arithmetic the GPU path reproduces bit for bit for rigid bodies.

``tests/golden/vtk_<case>.npz`` keeps, per file, its SHA-256 and size, and
the complete bytes of the last step's files (a few hundred KB at most), so a
file that differs can be compared number by number.

    python tests/golden/make_vtk.py
"""
from __future__ import annotations

import hashlib
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from cases import golden_cases  # noqa: E402
from make_golden import REF, run_case  # noqa: E402

CASES = {"cavity_cm": "openblas", "cylinder_rigid_cm": "textbook", "filament_flex_deflect": "textbook",
         "honami_like_cm": "textbook"}


def main() -> int:
    if not os.path.isdir(os.path.join(REF, "src")):
        print(f"reference tree not found at {REF}", file=sys.stderr)
        return 2
    work = tempfile.mkdtemp(prefix="life_vtk_")
    try:
        for name, lapack in CASES.items():
            p, b = golden_cases()[name]
            p = p.replace(vtk=True, vtk_fem=True, tVTK=p.nSteps // 2)
            r = run_case("vtk_" + name, p, b, work, lapack=lapack)
            files = r["vtk_files"]
            out = {"names": np.array(sorted(files)), "t": r["t"]}
            last = p.nSteps
            for fname, data in files.items():
                key = fname.replace(".", "_")
                out["sha_" + key] = hashlib.sha256(data).hexdigest()
                out["size_" + key] = len(data)
                if f".{last}." in fname:
                    out["bytes_" + key] = np.frombuffer(data, dtype=np.uint8)
            np.savez_compressed(os.path.join(HERE, f"vtk_{name}.npz"), **out)
            print(name, sorted(files))
    finally:
        shutil.rmtree(work, ignore_errors=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
