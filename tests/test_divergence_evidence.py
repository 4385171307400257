"""The recorded runs of the LIFE reference itself on the flexible-body
parameters the batched and served workloads leave out
(tests/golden/divergence_reference.json, made by
tests/golden/make_divergence_evidence.py with the reference's own OpenBLAS
LAPACK): where the reference's coupling diverges it stops with
"Subiteration scheme hit 20 iterations...exiting" (src/Objects.cpp:58-59),
exit status 99.

* One filament of L = 40 with one element per lattice unit, thickness 1 and
  mass ratio 0.5 (the filament configuration's section): the reference stops
  at stiffness 1e-3 and 3e-3 and runs 10,000 steps at 1e-2 and above -- the
  stiffness range the ensemble and serving workloads draw from starts at 1e-2.
* With thickness 0.1 and mass ratio 10 (the workloads' section) one such
  filament runs 10,000 steps across the whole 1e-3..1e-1 range.
* Request 9 of the seeded serving stream (1088 x 384, 22 stalks, 17,489
  steps) stops near step 10,100 in the reference as on the GPU, so requests
  are served at a fraction of their drawn length by default.
"""
import json
import os

import pytest

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "divergence_reference.json")
CAP = "Subiteration scheme hit 20 iterations...exiting"


@pytest.fixture(scope="module")
def runs():
    with open(PATH) as fh:
        return json.load(fh)["runs"]


def test_thick_soft_filaments_diverge_in_the_reference(runs):
    for s in ("0.001", "0.003"):
        r = runs[f"thickness1_mass0.5_stiffness{s}"]
        assert not r["completed"] and r["exit_status"] == 99 and r["last_output_line"] == CAP
        assert 0 < r["last_tip_step"] < 10000
    for s in ("0.01", "0.03", "0.1"):
        assert runs[f"thickness1_mass0.5_stiffness{s}"]["completed"]


def test_thin_heavy_filaments_run_in_the_reference(runs):
    for s in ("0.001", "0.003", "0.01", "0.03", "0.1"):
        assert runs[f"thickness0.1_mass10_stiffness{s}"]["completed"]


def test_long_canopy_request_diverges_in_the_reference(runs):
    r = runs["canopy_request9"]
    assert not r["completed"] and r["last_output_line"] == CAP
    assert 9000 <= r["last_tip_step"] <= 11000 < r["steps"]
