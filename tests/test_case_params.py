"""params.h round trip: CaseParams -> params.h text -> compiled by
include/life_params_pack.h -> identical values; and the reference's own
example params.h files (when the reference tree is present) pack cleanly."""
import glob
import os

import pytest

from cases import golden_cases
from life_gb300.case import load_params_h

REF = os.environ.get("LIFE_REFERENCE") or os.path.join(
    os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))), "reference")


@pytest.mark.parametrize("name", sorted(golden_cases()))
def test_params_h_round_trip(tmp_path, name):
    p, _ = golden_cases()[name]
    path = tmp_path / "params.h"
    path.write_text(p.to_params_h())
    q = load_params_h(str(path))
    for field in ("Nx", "Ny", "height_p", "rho_p", "nu_p", "omega", "ux0_p", "uy0_p", "gravityX", "gravityY",
                  "dpdx", "dpdy", "wall_left", "wall_right", "wall_bottom", "wall_top", "profile",
                  "uxInlet_p", "uyInlet_p", "alpha", "delta", "relaxMax", "subTol", "central_moments",
                  "inlet_ramp", "womersley", "uni_epsilon", "ordered", "initial_deflect", "nSteps",
                  "ref_nu", "ref_rho", "ref_P", "ref_L", "ref_U"):
        assert getattr(q, field) == getattr(p, field), field
    assert q.Dx == p.Dx and q.Dt == p.Dt


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "examples")), reason="reference tree not present")
@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(REF, "examples", "*", "params.h"))))
def test_reference_example_params_pack(path):
    q = load_params_h(path)
    assert q.Nx > 4 and q.Ny > 4 and q.omega > 0
    if "LidDrivenCavity" in path:
        assert q.central_moments and q.wall_top == 2 and q.Nx == 101
    if "PELskin" in path:
        assert q.womersley == 7.52 and q.wall_left == 0
    if "TurekHron" in path:
        assert q.inlet_ramp == 2.0 and q.profile == 0 and q.uni_epsilon
