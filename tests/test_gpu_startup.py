"""Body start-up (ObjectsClass ctor: removeOverlapMarkers, initialiseObjects
with the static pre-deflection of every flexible body) on the GPU path.

* The marker overlap test runs as a device kernel over all marker pairs for
  sets of 2048 markers or more (LIFE_OVERLAP_SCAN=device forces it for any
  set, =host keeps it on the host). Both sides apply the reference's test to
  the same values, so the markers left, their order, the bodies' node lists
  and everything built on them (support, ds, epsilon) must be the same bits
  either way, and equal to the oracle's.
* The static pre-deflection runs on host threads, one body per thread (the
  feedback loop is a serial chain of small band solves). With several
  flexible bodies the result must equal the oracle's sequential loop bit for
  bit.
"""
import dataclasses
import os

import numpy as np
import pytest

from cases import golden_cases, lattice_case
from life_gb300.case import CONVECTIVE, VELOCITY, Circle, Filament

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from life_gb300.build import build
    build()


def startup_state(p, b, scan=None):
    from life_gb300.lib import Case
    old = os.environ.get("LIFE_OVERLAP_SCAN")
    if scan:
        os.environ["LIFE_OVERLAP_SCAN"] = scan
    try:
        with Case(p, b) as c:
            out = dict(c.markers())
            bo = c.bodies()
            out.update({"body_" + k: np.asarray(v) for k, v in bo.items()})
            for k in range(c.n_flex):
                fm = c.fem(k)
                out[f"fem{k}_U"], out[f"fem{k}_pos"] = fm["U"], fm["pos"]
            out["n_markers"] = np.array([c.info().n_markers])
    finally:
        if old is None:
            os.environ.pop("LIFE_OVERLAP_SCAN", None)
        else:
            os.environ["LIFE_OVERLAP_SCAN"] = old
    return out


def assert_same(a, b):
    assert a.keys() == b.keys()
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def crowded_case():
    """100 rigid circles in a row (12 lattice units apart), ten more circles
    each overlapping one of them (centres 3 apart), and a flexible filament
    threaded through one circle of the row: about 2300 markers, with
    rigid-rigid and flexible-rigid close pairs."""
    p = lattice_case(1300, 80, 1.0 / 0.6, 10, wall_left=VELOCITY, wall_right=CONVECTIVE, uxInlet_p=0.03,
                     ref_L=10.0)
    b = [Circle(x=20.0, y=40.0, radius=3.5, ID=0, number=100, dx=12.0, dy=0.0),
         Circle(x=23.0, y=40.0, radius=3.5, ID=200, number=10, dx=120.0, dy=0.0),
         Filament(x=37.6, y=40.0, length=12.0, height=1.0, angle_deg=0.0, flexible=True, n_elements=12,
                  clamped=False, rho=10.0, E=1e4, ID=500)]
    return p, b


@pytest.mark.parametrize("name", ["cylinders_uni_bgk", "turek_like_uni", "filament_supported_and_rigid"])
def test_overlap_scan_device_equals_host_and_oracle(name):
    from oracle.pyoracle import Oracle
    p, b = golden_cases()[name]
    dev, host = startup_state(p, b, "device"), startup_state(p, b, "host")
    assert_same(dev, host)
    o = Oracle(p, b)
    mo = o.markers()
    for key in ("pos", "epsilon", "ds"):
        assert np.array_equal(dev[key], mo[key]), key
    o.close()


def test_overlap_scan_large_marker_set():
    p, b = crowded_case()
    dev, host = startup_state(p, b), startup_state(p, b, "host")
    assert int(dev["n_markers"][0]) >= 2048  # the default takes the device path
    assert_same(dev, host)


def test_flexible_overlap_is_refused_on_both_paths():
    from life_gb300.lib import LifeError, Case
    p, _ = golden_cases()["cavity_bgk"]
    b = [Filament(x=10.0, y=20.0, length=10.0, height=1.0, angle_deg=0.0, flexible=True, n_elements=10,
                  clamped=True, rho=10.0, E=1e4, ID=0),
         Filament(x=15.0, y=15.0, length=10.0, height=1.0, angle_deg=90.0, flexible=True, n_elements=10,
                  clamped=True, rho=10.0, E=1e4, ID=1)]
    for scan in ("device", "host"):
        os.environ["LIFE_OVERLAP_SCAN"] = scan
        try:
            with pytest.raises(LifeError, match="Cannot place two flexible bodies"):
                Case(p, b)
        finally:
            os.environ.pop("LIFE_OVERLAP_SCAN", None)


def test_static_deflection_of_several_bodies_on_threads_equals_oracle():
    from oracle.pyoracle import Oracle
    p, b = golden_cases()["honami_like_cm"]
    p = dataclasses.replace(p, initial_deflect=0.05)
    got = startup_state(p, b)
    o = Oracle(p, b)
    mo = o.markers()
    for key in ("pos", "vel", "epsilon", "ds"):
        assert np.array_equal(got[key], mo[key]), key
    for k in range(o.n_flex):
        fo = o.fem(k)
        assert np.array_equal(got[f"fem{k}_U"], fo["U"]), k
        assert np.array_equal(got[f"fem{k}_pos"], fo["pos"]), k
    o.close()
