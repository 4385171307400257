"""TEST INFRASTRUCTURE ONLY -- Python handle on the C oracle (liblife_oracle.so).

Imported by tests/, bench.py's CPU-baseline leg and the smoke check, never by
the product package. Builds the oracle on first use if the shared library is
missing.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from typing import Dict, Optional, Sequence

import numpy as np

from life_gb300.abi import body_structs, params_struct
from life_gb300.case import CaseParams, expand_bodies

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblife_oracle.so")
CR_LIB_PATH = os.path.join(HERE, "_build", "liblife_oracle_cr.so")
_libs: Dict[str, C.CDLL] = {}
_lock = threading.Lock()


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    return LIB_PATH


def lib(trig: str = "libm") -> C.CDLL:
    """The oracle library. trig="libm" is the restatement pinned to the
    reference (C library trigonometry); trig="cr" is the same restatement
    with the GPU's correctly rounded per-step trigonometry."""
    with _lock:
        if trig not in _libs:
            path = LIB_PATH if trig == "libm" else CR_LIB_PATH
            if not os.path.exists(path):
                build()
            L = C.CDLL(path)
            dp = C.POINTER(C.c_double)
            ip = C.POINTER(C.c_int)
            L.oracle_last_error.restype = C.c_char_p
            L.oracle_create.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]
            L.oracle_destroy.argtypes = [C.c_void_p]
            L.oracle_destroy.restype = None
            L.oracle_step.argtypes = [C.c_void_p, C.c_int]
            L.oracle_time.argtypes = [C.c_void_p]
            L.oracle_counts.argtypes = [C.c_void_p, ip, ip, ip, ip]
            L.oracle_get_fields.argtypes = [C.c_void_p, dp, dp, dp, dp]
            L.oracle_set_fields.argtypes = [C.c_void_p, C.c_int, dp, dp, dp, dp]
            L.oracle_get_markers.argtypes = [C.c_void_p, dp, dp, dp, dp, dp, ip]
            L.oracle_get_bodies.argtypes = [C.c_void_p, ip, ip, ip, ip]
            L.oracle_get_fem.argtypes = [C.c_void_p, C.c_int] + [dp] * 10
            L.oracle_get_relax.argtypes = [C.c_void_p, dp, ip, dp]
            L.oracle_solve.argtypes = [C.c_int, dp, dp, C.c_int, dp]
            L.oracle_get_nr.argtypes = [C.c_void_p, C.c_int, ip, dp]
            if trig == "cr":
                for name in ("oracle_cr_sin", "oracle_cr_cos"):
                    getattr(L, name).argtypes = [C.c_double]
                    getattr(L, name).restype = C.c_double
                L.oracle_cr_atan2.argtypes = [C.c_double, C.c_double]
                L.oracle_cr_atan2.restype = C.c_double
            _libs[trig] = L
    return _libs[trig]


def _dp(a: Optional[np.ndarray]):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a: Optional[np.ndarray]):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(C.c_int))


class OracleError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class Oracle:
    """A LIFE case run by the CPU oracle (reference layout, FP64)."""

    def __init__(self, params: CaseParams, bodies: Sequence = (), trig: str = "libm"):
        self._L = L = lib(trig)
        self.params = params
        bodies = expand_bodies(bodies)
        ps = params_struct(params)
        bs = body_structs(bodies)
        h = C.c_void_p()
        rc = L.oracle_create(C.byref(ps), C.byref(bs), len(bodies), C.byref(h))
        if rc:
            raise OracleError(rc, L.oracle_last_error().decode())
        self._h = h
        n = [C.c_int() for _ in range(4)]
        L.oracle_counts(h, *[C.byref(x) for x in n])
        self.n_markers, self.n_bodies, self.n_flex, self.sim_dofs = (x.value for x in n)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.oracle_destroy(self._h)
            self._h = None

    __del__ = close

    @property
    def t(self) -> int:
        return self._L.oracle_time(self._h)

    def step(self, n: int = 1) -> None:
        rc = self._L.oracle_step(self._h, int(n))
        if rc:
            raise OracleError(rc, self._L.oracle_last_error().decode())

    def fields(self) -> Dict[str, np.ndarray]:
        n = self.params.Nx * self.params.Ny
        rho, u = np.empty(n), np.empty((n, 2))
        f, fibm = np.empty((n, 9)), np.empty((n, 2))
        self._L.oracle_get_fields(self._h, _dp(rho), _dp(u), _dp(f), _dp(fibm))
        return dict(rho=rho, u=u, f=f, force_ibm=fibm)

    def set_fields(self, t: int, rho, u, f, force_ibm) -> None:
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (rho, u, f, force_ibm)]
        self._L.oracle_set_fields(self._h, int(t), *[_dp(a) for a in arrs])

    def markers(self) -> Dict[str, np.ndarray]:
        n = self.n_markers
        pos, vel, force = np.empty((n, 2)), np.empty((n, 2)), np.empty((n, 2))
        eps, ds = np.empty(n), np.empty(n)
        bidx = np.empty(n, dtype=np.int32)
        self._L.oracle_get_markers(self._h, _dp(pos), _dp(vel), _dp(force), _dp(eps), _dp(ds), _ip(bidx))
        return dict(pos=pos, vel=vel, force=force, epsilon=eps, ds=ds, body=bidx)

    def bodies(self) -> Dict[str, np.ndarray]:
        nb = self.n_bodies
        out = {k: np.empty(nb, dtype=np.int32) for k in ("ids", "flexible", "n_markers", "n_fem_nodes")}
        self._L.oracle_get_bodies(self._h, *[_ip(out[k]) for k in ("ids", "flexible", "n_markers", "n_fem_nodes")])
        return out

    def fem(self, k: int) -> Dict[str, np.ndarray]:
        nn = int(self.bodies()["n_fem_nodes"][np.flatnonzero(self.bodies()["flexible"])[k]])
        dofs = 3 * nn
        keys = ("U", "Udot", "Udotdot", "U_n", "U_nm1", "R_k")
        out = {key: np.empty(dofs) for key in keys}
        out["el_L"], out["el_angle"] = np.empty(nn - 1), np.empty(nn - 1)
        out["pos"], out["angle"] = np.empty((nn, 2)), np.empty(nn)
        rc = self._L.oracle_get_fem(self._h, k, *[_dp(out[key]) for key in keys], _dp(out["el_L"]),
                                  _dp(out["el_angle"]), _dp(out["pos"]), _dp(out["angle"]))
        if rc:
            raise OracleError(rc, self._L.oracle_last_error().decode())
        return out

    def nr(self, k: int = 0):
        it, res = C.c_int(), C.c_double()
        self._L.oracle_get_nr(self._h, k, C.byref(it), C.byref(res))
        return it.value, res.value

    def relax(self):
        r, s, res = C.c_double(), C.c_int(), C.c_double()
        self._L.oracle_get_relax(self._h, C.byref(r), C.byref(s), C.byref(res))
        return r.value, s.value, res.value


def solve(A: np.ndarray, b: np.ndarray, bc: int = 0) -> np.ndarray:
    A = np.ascontiguousarray(A, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.empty_like(b)
    lib().oracle_solve(A.shape[0], _dp(A), _dp(b), bc, _dp(x))
    return x
