"""The CANOPY geometry.config keyword (a keyword of this library, added the
way the reference's README describes, README.md:36-40): the C parser
(life_parse_geometry) and the Python description (life_gb300.case.Canopy)
expand it into the same FILAMENT bodies bit for bit, the text round-trips,
the SplitMix64 draws follow the published generator, and a case built from
a CANOPY line holds the same bodies as one built from its FILAMENT lines."""
import numpy as np
import pytest

from life_gb300.case import Canopy, expand_bodies, geometry_config_text, parse_geometry_config


def canopy():
    return Canopy(x=40.0, y=0.0, dx=23.5, length_min=20.0, length_max=40.0, height=0.1,
                  density_per_length=100.0, young_min=1.2e-2, young_max=1.2e-1, seed=20260101,
                  angle_deg=90.0, n_elements=20, clamped=True, ID=3, number=16)


def test_splitmix64_reference_values():
    from life_gb300.case import _splitmix64_draws
    # SplitMix64 from seed 0: first outputs 0xe220a8397b1dcdaf, 0x6e789e6aa1b965f4
    d = _splitmix64_draws(0)
    assert next(d) == (0xe220a8397b1dcdaf >> 11) * 2.0 ** -53
    assert next(d) == (0x6e789e6aa1b965f4 >> 11) * 2.0 ** -53


def test_text_round_trip():
    c = canopy()
    back = parse_geometry_config(geometry_config_text([c]))
    assert back == [c]


def test_c_parser_expands_like_python():
    from life_gb300.build import build
    build()
    from life_gb300.lib import parse_geometry
    c = canopy()
    got = parse_geometry(geometry_config_text([c]))
    want = c.expand()
    assert len(got) == len(want) == 16
    for d, f in zip(got, want):
        assert d.kind == 1 and d.number == 1 and d.id == f.ID and d.flexible == 1 and d.clamped == 1
        assert d.n_elements == 20
        for a, b in ((d.x, f.x), (d.y, f.y), (d.length, f.length), (d.height, f.height),
                     (d.angle_deg, f.angle_deg), (d.rho, f.rho), (d.E, f.E)):
            assert a == b
    lengths = np.array([f.length for f in want])
    assert lengths.min() >= 20.0 and lengths.max() < 40.0
    y = np.array([f.E / f.length ** 3 for f in want])
    assert y.min() >= 1.2e-2 * (1 - 1e-12) and y.max() < 1.2e-1


@pytest.mark.gpu
def test_case_from_canopy_equals_case_from_filaments():
    from life_gb300 import configs
    from life_gb300.lib import Case
    p, _ = configs.cylinder()
    p = p.replace(Nx=512, Ny=128, height_p=127.0)
    c = canopy()
    with Case(p, [c]) as a, Case(p, expand_bodies([c])) as b:
        ma, mb = a.markers(), b.markers()
        for key in ("pos", "epsilon", "ds"):
            assert np.array_equal(ma[key], mb[key])
        a.step(20)
        b.step(20)
        assert np.array_equal(a.fields(("u",))["u"], b.fields(("u",))["u"])
