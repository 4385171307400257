"""Serving (``life_server_*``): requests that arrive while others run are
admitted against the HBM budget and stepped together, regrouped each time a
request is admitted or finishes. Each request's final state must equal the
same case run alone (bit for bit: inside a batch a case runs the same
kernels with the same arguments in the same order; the scheduling rounds only
split its steps), in either storage form, whatever else is in the mix.
"""
import dataclasses
import time

import numpy as np
import pytest

from cases import golden_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from life_gb300.build import build
    build()


def _state(c):
    out = dict(c.fields(("u", "f")))
    if c.n_markers:
        out["marker_pos"] = c.markers()["pos"]
    return out


def _alone(p, b, steps):
    from life_gb300.lib import Case
    with Case(p, b) as c:
        c.step(steps)
        c.sync()
        return _state(c)


def _mix():
    cs = golden_cases()
    names = ["cavity_bgk", "cylinder_rigid_cm", "filament_flex_deflect", "channel_convective_freeslip_cm",
             "honami_like_cm", "periodic_womersley", "turek_like_uni", "velocity_walls_shear"]
    steps = [53, 120, 75, 31, 90, 64, 47, 110]
    precs = [1, 1, 0, 1, 1, 0, 1, 2]
    return [(dataclasses.replace(cs[n][0], precision=pr), cs[n][1], s) for n, s, pr in zip(names, steps, precs)]


def test_each_request_equals_its_solo_run():
    from life_gb300.lib import REQ_DONE, Server
    reqs = _mix()
    with Server(hbm_budget=8 << 30, steps_per_round=16) as S:
        ids = []
        for k, (p, b, n) in enumerate(reqs):
            ids.append(S.submit(p, b, n))
            if k % 3 == 2:
                time.sleep(0.05)  # later requests arrive while earlier ones run
        S.drain(timeout=300)
        st = S.stats()
        assert st.completed == len(reqs) and st.failed == 0
        assert st.regroups >= 2
        for rid, (p, b, n) in zip(ids, reqs):
            inf = S.query(rid)
            assert inf.state == REQ_DONE and inf.steps_done == n
            assert inf.submit_s <= inf.start_s <= inf.done_s
            with S.take(rid) as c:
                assert c.t == n
                got = _state(c)
            ref = _alone(p, b, n)
            for key in ref:
                assert np.array_equal(got[key], ref[key]), (rid, key)


def test_admission_respects_budget_in_arrival_order():
    from life_gb300.lib import Server
    cs = golden_cases()
    p, b = cs["cylinder_rigid_cm"]
    p = dataclasses.replace(p, precision=1)
    from life_gb300.lib import Case
    with Case(p, b) as c:
        one = c.info().device_bytes
    # the admission estimate is above the exact footprint; this budget holds
    # a few such requests at a time, not all six
    with Server(hbm_budget=int(4 * one), steps_per_round=8) as S:
        ids = [S.submit(p, b, 40) for _ in range(6)]
        starts = []
        for i in ids:  # a finished request holds its memory until released
            S.wait(i, timeout=300)
            starts.append(S.query(i).start_s)
            S.release(i)
        st = S.stats()
        assert st.completed == 6 and 0 < st.bytes_peak <= 4 * one
        assert starts == sorted(starts)  # admitted in arrival order
        assert st.bytes_in_use == 0


def test_failed_request_does_not_disturb_others():
    from life_gb300.lib import REQ_DONE, REQ_FAILED, LifeError, Server
    cs = golden_cases()
    p, b = cs["cavity_bgk"]
    bad = dataclasses.replace(p, Nx=2)  # rejected at creation
    with Server(hbm_budget=1 << 30) as S:
        a = S.submit(p, b, 20)
        x = S.submit(bad, [], 20)
        c2 = S.submit(p, b, 30)
        S.drain(timeout=120)
        assert S.query(a).state == REQ_DONE and S.query(c2).state == REQ_DONE
        with pytest.raises(LifeError):
            S.wait(x, 1.0)
        assert S.query(x).state == REQ_FAILED
        with S.take(c2) as c:
            got = _state(c)
    ref = _alone(p, b, 30)
    for key in ref:
        assert np.array_equal(got[key], ref[key]), key
