#!/usr/bin/env python3
"""Runs the LIFE reference itself on flexible-filament cases drawn as the
batched-ensemble configuration states them, to record which parameters its
own coupling can carry for 10,000 steps.

The ensemble configuration asks for filaments of L = 20-60 lattice units with
one element per lattice unit and a bending stiffness EI/(rho U^2 L^3)
log-uniform over 1e-3..1e-1 (no thickness or mass ratio given; the filament
configuration uses thickness 1 and mass ratio 0.5). Each case here is one
such filament (L = 40, 40 elements, clamped at its leading end) in a
512 x 256 channel, inlet 0.04 ramped in over 400 steps, convective outlet,
Re = 100 on L (tau = 0.548), BGK, sub-iteration tolerance 1e-8, run for
10,000 steps with the reference's own LAPACK (OpenBLAS) and TIPS written
every 10 steps. Two sections are swept over the stiffness range:

* thickness 1, mass ratio 0.5 (the filament configuration's values);
* thickness 0.1, mass ratio 10 (the values the ensemble workload uses).

For each run ``tests/golden/divergence_reference.json`` records whether the
reference finished, the last step whose tip line it wrote, and the last line
it printed (``Subiteration scheme hit 20 iterations...exiting`` when the
coupling diverged, src/Objects.cpp:58-59).

    python tests/golden/make_divergence_evidence.py --sweep [--canopy K ...]
        [--ensemble-thin-1e-3 K ...] [--threads N]

``--canopy K`` runs request K of the seeded serving stream at its full length
and ``--ensemble-thin-1e-3 K`` case K of the ensemble drawn with the
configured stiffness range (1e-3..1e-1), both with info and tips every 50
steps.
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

from make_golden import REF  # noqa: E402
from life_gb300.case import CONVECTIVE, VELOCITY, WALL, CaseParams, Filament, geometry_config_text  # noqa: E402
from life_gb300.ensemble import filament_modulus  # noqa: E402

STEPS = 10000
STIFFNESS = (1e-3, 3e-3, 1e-2, 3e-2, 1e-1)
SECTIONS = {"thickness1_mass0.5": (1.0, 0.5), "thickness0.1_mass10": (0.1, 10.0)}


def case(stiffness: float, height: float, mass_ratio: float):
    L, u, tau = 40.0, 0.04, 0.548
    nu = (tau - 0.5) / 3.0
    p = CaseParams(Nx=512, Ny=256, height_p=255.0, rho_p=1.0, nu_p=nu, omega=1.0 / tau, wall_left=VELOCITY,
                   wall_right=CONVECTIVE, wall_bottom=WALL, wall_top=WALL, uxInlet_p=u, inlet_ramp=400.0,
                   ref_L=L, subTol=1e-8, nSteps=STEPS, tinfo=10, tVTK=STEPS, tRestart=0)
    b = [Filament(x=80.0, y=128.0, length=L, height=height, angle_deg=0.0, flexible=True, n_elements=int(L),
                  clamped=True, rho=mass_ratio * L / height, E=filament_modulus(stiffness, u, L, height), ID=0)]
    return p, b


def run(name: str, p, b, work: str, threads: int) -> dict:
    cdir, rdir = os.path.join(work, name, "case"), os.path.join(work, name, "run")
    os.makedirs(cdir)
    os.makedirs(os.path.join(rdir, "input"))
    with open(os.path.join(cdir, "params.h"), "w") as fh:
        fh.write(p.to_params_h())
    with open(os.path.join(rdir, "input", "geometry.config"), "w") as fh:
        fh.write(geometry_config_text(b))
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(REPO, "oracle"), "ref", f"CASE={cdir}",
                    f"NAME=evidence_{name}", f"REF={REF}"], check=True)
    exe = os.path.join(REPO, "oracle", "_ref", f"evidence_{name}", "LIFE")
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), OPENBLAS_NUM_THREADS="1")
    res = subprocess.run([exe], cwd=rdir, env=env, capture_output=True, text=True)
    tips = open(os.path.join(rdir, "Results", "TipPositions.out")).read().strip().splitlines()
    lines = [ln for ln in res.stdout.strip().splitlines() if ln.strip()]
    tips = tips if tips else ["", "0"]
    return {"completed": res.returncode == 0, "exit_status": res.returncode,
            "last_tip_step": int(tips[-1].split("\t")[0]) if len(tips) > 1 else 0,
            "last_tip_line": tips[-1], "last_output_line": lines[-1] if lines else "",
            "E": b[0].E, "rho": b[0].rho, "height": b[0].height}


def canopy_request(k: int, seed: int = 7, steps=None, **kw):
    """Request k of the seeded serving stream (life_gb300.ensemble.canopy_case)."""
    import numpy as np
    from life_gb300.ensemble import canopy_case
    rng = np.random.Generator(np.random.PCG64(seed))
    for _ in range(k + 1):
        p, b, n = canopy_case(rng, precision=0, **kw)
    n = steps or n
    return p.replace(nSteps=n, tinfo=50, tVTK=n, tRestart=0), b


def ensemble_case(k: int, **kw):
    """Case k of the seeded ensemble (life_gb300.ensemble.ensemble_cases)."""
    from life_gb300.ensemble import ensemble_cases
    p, b = ensemble_cases(n=k + 1, precision=0, **kw)[k]
    return p.replace(nSteps=STEPS, tinfo=50, tVTK=STEPS, tRestart=0), b


def main(argv) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--sweep", action="store_true", help="the single-filament stiffness sweep")
    ap.add_argument("--canopy", type=int, nargs="*", default=[], help="serving-stream requests to run in full")
    ap.add_argument("--ensemble-thin-1e-3", type=int, nargs="*", default=[],
                    help="ensemble cases drawn with stiffness 1e-3..1e-1 (thickness 0.1, mass ratio 10)")
    a = ap.parse_args(argv[1:])
    if not os.path.isdir(os.path.join(REF, "src")):
        print(f"reference tree not found at {REF}", file=sys.stderr)
        return 2
    path = os.path.join(HERE, "divergence_reference.json")
    out = {"steps": STEPS, "lattice": [512, 256], "filament_length": 40, "elements": 40, "inlet": 0.04,
           "tau": 0.548, "lapack": "openblas", "runs": {}}
    if os.path.exists(path):
        with open(path) as fh:
            out = json.load(fh)
    jobs = []
    if a.sweep:
        for sec, (h, mr) in SECTIONS.items():
            for s in STIFFNESS:
                p, b = case(s, h, mr)
                jobs.append((f"{sec}_stiffness{s:g}", p, b, dict(stiffness=s, section=sec, mass_ratio=mr)))
    for k in a.canopy:
        p, b = canopy_request(k)
        jobs.append((f"canopy_request{k}", p, b, dict(request=k, steps=p.nSteps, lattice=[p.Nx, p.Ny],
                                                     stalks=len(b))))
    for k in a.ensemble_thin_1e_3:
        p, b = ensemble_case(k, stiffness=(1e-3, 1e-1))
        jobs.append((f"ensemble_stiffness1e-3_case{k}", p, b,
                     dict(case=k, lattice=[p.Nx, p.Ny], filaments=len(b),
                          min_stiffness_E=min(x.E for x in b))))
    work = tempfile.mkdtemp(prefix="life_evidence_")
    try:
        for name, p, b, meta in jobs:
            r = run(name, p, b, work, a.threads)
            r.update(meta)
            out["runs"][name] = r
            print(name, "completed" if r["completed"] else f"failed after step {r['last_tip_step']}",
                  "|", r["last_output_line"], flush=True)
            with open(path, "w") as fh:
                json.dump(out, fh, indent=1, sort_keys=True)
    finally:
        shutil.rmtree(work, ignore_errors=True)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
