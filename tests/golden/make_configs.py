#!/usr/bin/env python3
"""Golden records of the three named single-case workloads, made by running
the LIFE reference itself at their full stated sizes.

* ``config1_cavity256.npz`` -- the 256 x 256 BGK lid-driven cavity after
  20,000 steps: SHA-256 digests of the reference's ``Fluid.restart`` arrays
  (f, rho, u in the reference layout ``id = i*Ny + j``), max |u| and every
  eighth site's u (for a diagnosis if a digest ever differs).
* ``config2_cylinder.npz`` -- the 1000 x 400 central-moments cylinder over
  50,000 steps: the reference's ``TotalForces.out`` written every 100 steps
  (``src/Objects.cpp:491-539``), and digests of the final lattice and marker
  state.
* ``config3_filament.npz`` -- the 1200 x 400 flexible filament over 2,000
  steps: ``TipPositions.out`` / ``TipVelocities.out`` / ``TotalForces.out``
  every 10 steps (``src/Objects.cpp:542-594``) and the final FEM and marker
  state.

The cases with bodies link the reference against the textbook-LU LAPACK shim
(``oracle/ref_shim/lapack_textbook.c``), whose factorisation order the GPU
path and the oracle follow, so the whole record is one deterministic
arithmetic. The reference runs with ``ORDERED`` (ordered OpenMP reductions),
so its results do not depend on the thread count; ``--check-threads``
verifies that on a small body case before the long runs.

    python tests/golden/make_configs.py [config1 config2 config3] [--threads N]

The reference tree is ``LIFE_REFERENCE``, else a checkout named ``reference``
beside this repository. The cases themselves are ``life_gb300.configs``.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

from make_golden import REF, array_digest, run_case  # noqa: E402
from life_gb300 import configs  # noqa: E402


def _series(text: str) -> np.ndarray:
    rows = [ln.split("\t") for ln in text.strip().splitlines()[1:]]
    return np.array([[float(x) for x in r] for r in rows])


def config1(work: str, threads: int) -> dict:
    p = configs.cavity(256, steps=20000)
    r = run_case("config1", p, [], work, threads=threads)
    u = r["u"].reshape(256, 256, 2)
    return dict(t=r["t"], sha_f=array_digest(r["f"]), sha_rho=array_digest(r["rho"]),
                sha_u=array_digest(r["u"]), u_max=float(np.abs(r["u"]).max()),
                u_sub=u[::8, ::8].copy(), params_digest=r["params_digest"])


def config2(work: str, threads: int) -> dict:
    p, b = configs.cylinder(steps=50000, tinfo=100)
    r = run_case("config2", p, b, work, lapack="textbook", threads=threads)
    out = dict(t=r["t"], total_forces_text=r["total_forces_text"], params_digest=r["params_digest"])
    for key in ("f", "rho", "u", "force_ibm", "ibm_pos", "ibm_vel", "ibm_force"):
        out["sha_" + key] = array_digest(r[key])
    out["ibm_force"] = r["ibm_force"]
    return out


def config3(work: str, threads: int) -> dict:
    p, b = configs.filament(steps=2000, tinfo=10)
    r = run_case("config3", p, b, work, lapack="textbook", threads=threads)
    out = dict(t=r["t"], params_digest=r["params_digest"])
    for key in ("total_forces_text", "tip_positions_text", "tip_velocities_text"):
        out[key] = r[key]
    for key in ("ibm_pos", "ibm_vel", "ibm_force", "fem_U", "fem_Udot", "fem_Udotdot", "fem_pos", "fem_relax"):
        out[key] = r[key]
    for key in ("f", "rho", "u", "force_ibm"):
        out["sha_" + key] = array_digest(r[key])
    return out


def check_threads(work: str, threads: int) -> None:
    """The reference's result on a flexible-body case must not depend on its
    thread count (ORDERED reductions)."""
    from cases import golden_cases
    p, b = golden_cases()["filament_supported_and_rigid"]
    one = run_case("thr1", p, b, work, lapack="textbook", threads=1)
    many = run_case(f"thr{threads}", p, b, work, lapack="textbook", threads=threads)
    for key in ("f", "u", "ibm_force", "fem_U"):
        if not np.array_equal(one[key], many[key]):
            raise SystemExit(f"reference result depends on the thread count ({key})")
    print(f"thread check: 1 and {threads} threads bit-identical")


def main(argv) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("which", nargs="*", default=["config1", "config2", "config3"])
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--check-threads", action="store_true")
    a = ap.parse_args(argv[1:])
    if not os.path.isdir(os.path.join(REF, "src")):
        print(f"reference tree not found at {REF}", file=sys.stderr)
        return 2
    work = tempfile.mkdtemp(prefix="life_configs_")
    try:
        if a.check_threads:
            check_threads(work, a.threads)
        names = {"config1": ("config1_cavity256", config1), "config2": ("config2_cylinder", config2),
                 "config3": ("config3_filament", config3)}
        for key in a.which:
            fname, fn = names[key]
            t0 = time.time()
            res = fn(work, a.threads)
            res["reference_seconds"] = time.time() - t0
            res["reference_threads"] = a.threads
            np.savez_compressed(os.path.join(HERE, fname + ".npz"), **res)
            print(f"{fname}: t={res['t']} ({res['reference_seconds']:.0f} s on {a.threads} threads)", flush=True)
    finally:
        shutil.rmtree(work, ignore_errors=True)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
