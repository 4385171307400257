"""Argument checks of the C-ABI that run before any device work, so they are
exercised here without a GPU: every rejected call returns LIFE_ERR_INVALID,
leaves the output handle NULL and sets a message naming the problem. The
convective-wall message is the reference's own (GridClass::initialiseGrid,
src/Grid.cpp:918-920: only the right boundary may be convective)."""
import ctypes as C
import dataclasses

import pytest

from life_gb300.abi import body_structs, params_struct
from life_gb300.case import CONVECTIVE, FLUID, PREC_F32, PREC_F64, Circle

LIFE_ERR_INVALID = 1


@pytest.fixture(scope="module")
def L():
    from life_gb300.lib import lib
    return lib()


def base():
    from life_gb300 import configs
    return configs.cavity(64, PREC_F64)


def create(L, p, bodies=()):
    ps = params_struct(p) if p is not None else None
    bs = body_structs(list(bodies))
    h = C.c_void_p(12345)
    rc = L.life_case_create(C.byref(ps) if ps is not None else None, C.byref(bs), len(bodies), C.byref(h))
    return rc, h.value, L.life_last_error().decode()


@pytest.mark.parametrize("change, message", [
    (dict(Nx=3), "at least 4 x 4"),
    (dict(Ny=2), "at least 4 x 4"),
    (dict(Ny=70000), "Ny above 65535"),
    (dict(wall_left=9), "unknown wall type"),
    (dict(wall_top=-1), "unknown wall type"),
    (dict(wall_left=CONVECTIVE), "Currently convective BC only supported for right boundary...exiting"),
    (dict(wall_bottom=CONVECTIVE), "Currently convective BC only supported for right boundary...exiting"),
    (dict(wall_top=CONVECTIVE), "Currently convective BC only supported for right boundary...exiting"),
    (dict(precision=7), "unknown precision"),
    (dict(omega=0.0), "omega must be positive"),
    (dict(omega=-1.5), "omega must be positive"),
])
def test_case_create_rejects_bad_parameters(L, change, message):
    rc, h, msg = create(L, dataclasses.replace(base(), **change))
    assert rc == LIFE_ERR_INVALID and h is None
    assert message in msg, msg


def test_case_create_rejects_null_arguments(L):
    rc, h, msg = create(L, None)
    assert rc == LIFE_ERR_INVALID and h is None and "params is NULL" in msg
    ps = params_struct(base())
    assert L.life_case_create(C.byref(ps), None, 0, None) == LIFE_ERR_INVALID
    assert "out is NULL" in L.life_last_error().decode()
    h = C.c_void_p(7)
    assert L.life_case_create(C.byref(ps), None, 2, C.byref(h)) == LIFE_ERR_INVALID  # bodies missing
    assert h.value is None and "bad body list" in L.life_last_error().decode()
    assert L.life_case_create(C.byref(ps), None, -1, C.byref(h)) == LIFE_ERR_INVALID


def test_valid_parameters_pass_the_checks(L):
    # the checks accept the reference's own combinations; periodic walls and
    # a convective right wall are fine (creation may then fail later only for
    # want of a device)
    for change in (dict(), dict(wall_left=FLUID, wall_right=FLUID), dict(wall_right=CONVECTIVE),
                   dict(precision=PREC_F32)):
        rc, h, msg = create(L, dataclasses.replace(base(), **change))
        assert rc != LIFE_ERR_INVALID or "device" in msg.lower(), msg
        if h:
            L.life_case_destroy(C.c_void_p(h))


def test_null_handles_are_rejected(L):
    assert L.life_case_step(None, 1) == LIFE_ERR_INVALID
    assert L.life_case_destroy(None) == 0
    assert L.life_batch_step(None, 1) == LIFE_ERR_INVALID
    assert L.life_batch_sync(None) == LIFE_ERR_INVALID
    assert L.life_case_get_fields(None, None, None, None, None) == LIFE_ERR_INVALID


def test_batch_create_rejects_mixed_storage_and_empty_lists(L):
    from life_gb300.abi import LifeCaseParams
    ps = (LifeCaseParams * 2)(params_struct(base()), params_struct(dataclasses.replace(base(), precision=PREC_F32)))
    nb = (C.c_int32 * 2)(0, 0)
    h = C.c_void_p(5)
    assert L.life_batch_create(ps, None, nb, 2, C.byref(h)) == LIFE_ERR_INVALID
    assert h.value is None and "same population storage form" in L.life_last_error().decode()
    assert L.life_batch_create(ps, None, nb, 0, C.byref(h)) == LIFE_ERR_INVALID
    assert L.life_batch_create(None, None, nb, 2, C.byref(h)) == LIFE_ERR_INVALID


def test_body_list_type_is_checked_before_the_device(L):
    # a negative body count is refused whatever the bodies
    p = base()
    ps = params_struct(p)
    bs = body_structs([Circle(x=30.0, y=30.0, radius=5.0)])
    h = C.c_void_p(3)
    assert L.life_case_create(C.byref(ps), C.byref(bs), -2, C.byref(h)) == LIFE_ERR_INVALID
    assert h.value is None
