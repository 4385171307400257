"""Batched ensembles (``life_batch_*``): the batch steps all golden cases
together (uneven lattices, BGK and central moments, every wall type, rigid
and flexible bodies, uniform epsilon) through one persistent interior launch
and one replayed graph per step, and every case must come out exactly as it
does when run alone through ``life_case_step``: the per-case kernels, their
arguments and their order within a case are the same, so the comparison is
bit for bit.

The step counts are split over two calls with an odd first count, so both
step graphs (the two buffer parities) run and a second call resumes from the
first; a tile autotune between the calls re-cuts the interior launch.
"""
import dataclasses

import numpy as np
import pytest

from cases import golden_cases

pytestmark = pytest.mark.gpu
STEPS = (37, 24)


@pytest.fixture(scope="module", autouse=True)
def built():
    from life_gb300.build import build
    build()


def _state(c):
    out = dict(c.fields())
    if c.n_markers:
        mk = c.markers()
        out["marker_pos"], out["marker_force"] = mk["pos"], mk["force"]
    for k in range(c.n_flex):
        out[f"fem{k}_U"] = c.fem(k)["U"]
    return out


def _alone(p, b):
    from life_gb300.lib import Case
    with Case(p, b) as c:
        for n in STEPS:
            c.step(n)
        c.sync()
        return _state(c)


@pytest.mark.parametrize("prec", [0, 1, 2], ids=["f64", "f32", "f16"])
def test_batch_equals_each_case_alone(prec):
    from life_gb300.lib import Batch
    items = [(dataclasses.replace(p, precision=prec), b) for p, b in golden_cases().values()]
    with Batch(items) as B:
        B.step(STEPS[0])
        w, h, ms = B.autotune()
        assert w in (64, 128, 256) and h in (1, 2, 4, 8) and ms > 0
        B.step(STEPS[1])
        info = B.info()
        assert info.n_cases == len(items) and info.tile_w == w and info.tile_h == h
        assert info.sites == sum(p.Nx * p.Ny for p, _ in items)
        assert info.kernel_nodes > len(items)
        for k, (p, b) in enumerate(items):
            c = B.case(k)
            assert c.t == sum(STEPS)
            got, ref = _state(c), _alone(p, b)
            for key in ref:
                assert np.array_equal(got[key], ref[key]), (k, key)


def test_batch_rejects_mixed_storage():
    from life_gb300.lib import Batch, LifeError
    cs = list(golden_cases().values())[:2]
    items = [(dataclasses.replace(cs[0][0], precision=0), cs[0][1]),
             (dataclasses.replace(cs[1][0], precision=1), cs[1][1])]
    with pytest.raises(LifeError):
        Batch(items)
