"""Python handle on the C-ABI (``liblife_gb300.so``).

:class:`Case` mirrors how the reference's ``main()`` drives a run
(reference ``src/main.cpp:42-86``): construct it from a ``params.h`` value set
and the geometry (``GridClass()`` + ``ObjectsClass(grid)``), advance it with
:meth:`Case.step` (``grid.solver()`` per step) and read the restart-format
fields, markers and FEM state back. Every call goes through the exported C
functions; there is no Python or CPU compute path.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from typing import Dict, Optional, Sequence

import numpy as np

from .abi import (ERRORS, LifeBatchInfo, LifeCaseInfo, LifeRequestInfo, LifeServerConfig, LifeServerStats,
                  LifeStatus, body_structs, params_struct)
from .case import CaseParams, expand_bodies

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "liblife_gb300.so")
_lib: Optional[C.CDLL] = None
_lock = threading.Lock()

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)

# Every function the header declares, with its ctypes signature.
SIGNATURES = {
    "life_abi_version": (C.c_int, []),
    "life_last_error": (C.c_char_p, []),
    "life_case_create": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_void_p)]),
    "life_case_destroy": (C.c_int, [C.c_void_p]),
    "life_case_step": (C.c_int, [C.c_void_p, C.c_int32]),
    "life_case_sync": (C.c_int, [C.c_void_p]),
    "life_case_info": (C.c_int, [C.c_void_p, C.c_void_p]),
    "life_case_status": (C.c_int, [C.c_void_p, C.c_void_p]),
    "life_case_get_fields": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp]),
    "life_case_set_fields": (C.c_int, [C.c_void_p, C.c_int32, _dp, _dp, _dp, _dp]),
    "life_case_get_markers": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp, _dp, _ip]),
    "life_case_get_bodies": (C.c_int, [C.c_void_p, _ip, _ip, _ip, _ip]),
    "life_case_get_fem": (C.c_int, [C.c_void_p, C.c_int32] + [_dp] * 10),
    "life_case_get_relax": (C.c_int, [C.c_void_p, _dp]),
    "life_case_set_markers": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "life_case_set_fem": (C.c_int, [C.c_void_p, C.c_int32] + [_dp] * 12),
    "life_case_set_relax": (C.c_int, [C.c_void_p, C.c_double]),
    "life_case_get_fem0": (C.c_int, [C.c_void_p, C.c_int32, _dp, _dp]),
    "life_selftest_division": (C.c_int, [C.c_int64, C.c_uint64, C.POINTER(C.c_int64)]),
    "life_case_max_velocity": (C.c_int, [C.c_void_p, _dp, _ip]),
    "life_case_total_force": (C.c_int, [C.c_void_p, _dp, _dp]),
    "life_case_record": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "life_case_get_body_nodes": (C.c_int, [C.c_void_p, _ip, _ip]),
    "life_case_get_vtk_fields": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "life_measure_fp64_rate": (C.c_int, [_dp]),
    "life_selftest_trig": (C.c_int, [C.c_int32, C.c_int64, _dp, _dp, _dp]),
    "life_case_records": (C.c_int, [C.c_void_p, C.c_int32, _ip, _ip, _ip, _dp, _ip]),
    "life_parse_geometry": (C.c_int, [C.c_char_p, C.c_void_p, C.c_int32, _ip]),
    "life_case_bench_steps": (C.c_int, [C.c_void_p, C.c_int32, _dp, _dp, _ip]),
    "life_case_get_support": (C.c_int, [C.c_void_p, _ip, _ip, _ip, _dp]),
    "life_ibm_epsilon": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_int32, C.c_double, C.c_void_p, C.c_void_p]),
    "life_ibm_epsilon_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_int32, C.c_double, C.c_void_p, C.c_void_p]),
    "life_batch_create": (C.c_int, [C.c_void_p, C.c_void_p, _ip, C.c_int32, C.POINTER(C.c_void_p)]),
    "life_batch_destroy": (C.c_int, [C.c_void_p]),
    "life_batch_step": (C.c_int, [C.c_void_p, C.c_int32]),
    "life_batch_sync": (C.c_int, [C.c_void_p]),
    "life_batch_case": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p)]),
    "life_batch_info": (C.c_int, [C.c_void_p, C.c_void_p]),
    "life_batch_set_tile": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "life_batch_autotune": (C.c_int, [C.c_void_p, _ip, _ip, C.POINTER(C.c_float)]),
    "life_batch_interior_ms": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float)]),
    "life_batch_bench_steps": (C.c_int, [C.c_void_p, C.c_int32, _dp, _ip]),
    "life_server_create": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "life_server_submit": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                                     C.POINTER(C.c_int64)]),
    "life_server_query": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p]),
    "life_server_wait": (C.c_int, [C.c_void_p, C.c_int64, C.c_double]),
    "life_server_take": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_void_p)]),
    "life_server_release": (C.c_int, [C.c_void_p, C.c_int64]),
    "life_server_stats": (C.c_int, [C.c_void_p, C.c_void_p]),
    "life_server_drain": (C.c_int, [C.c_void_p, C.c_double]),
    "life_server_destroy": (C.c_int, [C.c_void_p]),
}


class LifeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def lib() -> C.CDLL:
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"{LIB_PATH} is missing: run `python -m life_gb300.build` "
                                   "(the GPU path has no fallback)")
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def _check(rc: int) -> None:
    if rc:
        raise LifeError(rc, lib().life_last_error().decode())


def _p(a: Optional[np.ndarray]):
    if a is None:
        return None
    if a.dtype == np.float64:
        return a.ctypes.data_as(_dp)
    return a.ctypes.data_as(_ip)


class Case:
    """A LIFE case running on the GPU through the C-ABI."""

    def __init__(self, params: CaseParams, bodies: Sequence = (), _handle=None):
        L = lib()
        self.params = params
        self._owned = _handle is None
        if _handle is None:
            bodies = expand_bodies(bodies)
            ps = params_struct(params)
            bs = body_structs(bodies)
            h = C.c_void_p()
            _check(L.life_case_create(C.byref(ps), C.byref(bs), len(bodies), C.byref(h)))
            _handle = h
        self._h = _handle
        info = self.info()
        self.n_markers, self.n_bodies, self.n_flex = info.n_markers, info.n_bodies, info.n_flex

    def close(self) -> None:
        if getattr(self, "_h", None):
            if self._owned:
                lib().life_case_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def info(self) -> LifeCaseInfo:
        inf = LifeCaseInfo()
        _check(lib().life_case_info(self._h, C.byref(inf)))
        return inf

    def status(self) -> LifeStatus:
        st = LifeStatus()
        _check(lib().life_case_status(self._h, C.byref(st)))
        return st

    @property
    def t(self) -> int:
        return self.info().t

    def step(self, n: int = 1) -> None:
        _check(lib().life_case_step(self._h, int(n)))

    def sync(self) -> None:
        _check(lib().life_case_sync(self._h))

    def fields(self, which=("rho", "u", "f", "force_ibm"), out: Optional[Dict[str, np.ndarray]] = None
               ) -> Dict[str, np.ndarray]:
        """The fields of `which` in the reference layout. `out` may hold
        caller-owned arrays to fill (C-contiguous float64 of the right shape),
        as a host program reuses its own buffers from step to step."""
        n = self.params.Nx * self.params.Ny
        shapes = {"rho": (n,), "u": (n, 2), "f": (n, 9), "force_ibm": (n, 2)}
        given = out or {}
        for k, a in given.items():
            if k not in shapes or a.shape != shapes[k] or a.dtype != np.float64 or not a.flags.c_contiguous:
                raise ValueError(f"out[{k!r}] must be a C-contiguous float64 array of shape {shapes.get(k)}")
        out = {}

        def buf(k):
            if k not in which:
                return None
            return given[k] if k in given else np.empty(shapes[k])
        rho, u, f, fi = buf("rho"), buf("u"), buf("f"), buf("force_ibm")
        _check(lib().life_case_get_fields(self._h, _p(rho), _p(u), _p(f), _p(fi)))
        for k, v in (("rho", rho), ("u", u), ("f", f), ("force_ibm", fi)):
            if v is not None:
                out[k] = v
        return out

    def set_fields(self, t: int, rho, u, f, force_ibm=None) -> None:
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (rho, u, f)]
        fi = None if force_ibm is None else np.ascontiguousarray(force_ibm, dtype=np.float64)
        _check(lib().life_case_set_fields(self._h, int(t), *[_p(a) for a in arrs], _p(fi)))

    def markers(self) -> Dict[str, np.ndarray]:
        n = self.n_markers
        pos, vel, force = np.empty((n, 2)), np.empty((n, 2)), np.empty((n, 2))
        eps, ds = np.empty(n), np.empty(n)
        body = np.empty(n, dtype=np.int32)
        _check(lib().life_case_get_markers(self._h, _p(pos), _p(vel), _p(force), _p(eps), _p(ds), _p(body)))
        return dict(pos=pos, vel=vel, force=force, epsilon=eps, ds=ds, body=body)

    def support(self) -> Dict[str, np.ndarray]:
        n = self.n_markers
        ns = np.empty(n, dtype=np.int32)
        si, sj = np.empty((n, 9), dtype=np.int32), np.empty((n, 9), dtype=np.int32)
        sd = np.empty((n, 9))
        _check(lib().life_case_get_support(self._h, _p(ns), _p(si), _p(sj), _p(sd)))
        return dict(nsupp=ns, si=si, sj=sj, sd=sd)

    def bodies(self) -> Dict[str, np.ndarray]:
        nb = self.n_bodies
        out = {k: np.empty(nb, dtype=np.int32) for k in ("ids", "flexible", "n_markers", "n_fem_nodes")}
        _check(lib().life_case_get_bodies(self._h, *[_p(out[k]) for k in
                                                     ("ids", "flexible", "n_markers", "n_fem_nodes")]))
        return out

    def fem(self, k: int) -> Dict[str, np.ndarray]:
        b = self.bodies()
        nn = int(b["n_fem_nodes"][np.flatnonzero(b["flexible"])[k]])
        dofs = 3 * nn
        keys = ("U", "Udot", "Udotdot", "U_n", "U_nm1", "R_k")
        out = {key: np.empty(dofs) for key in keys}
        out["el_L"], out["el_angle"] = np.empty(nn - 1), np.empty(nn - 1)
        out["pos"], out["angle"] = np.empty((nn, 2)), np.empty(nn)
        _check(lib().life_case_get_fem(self._h, k, *[_p(out[key]) for key in keys], _p(out["el_L"]),
                                       _p(out["el_angle"]), _p(out["pos"]), _p(out["angle"])))
        out["pos0"], out["angle0"] = np.empty((nn, 2)), np.empty(nn)
        _check(lib().life_case_get_fem0(self._h, k, _p(out["pos0"]), _p(out["angle0"])))
        return out

    def set_markers(self, pos=None, vel=None, force=None) -> None:
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (pos, vel, force)]
        _check(lib().life_case_set_markers(self._h, *[_p(a) for a in arrs]))

    def set_fem(self, k: int, U=None, Udot=None, Udotdot=None, U_n=None, U_nm1=None, R_k=None, el_L=None,
                el_angle=None, pos0=None, pos=None, angle0=None, angle=None) -> None:
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64)
                for a in (U, Udot, Udotdot, U_n, U_nm1, R_k, el_L, el_angle, pos0, pos, angle0, angle)]
        _check(lib().life_case_set_fem(self._h, int(k), *[_p(a) for a in arrs]))

    def set_relax(self, relax: float) -> None:
        _check(lib().life_case_set_relax(self._h, float(relax)))

    def relax(self) -> float:
        r = C.c_double()
        _check(lib().life_case_get_relax(self._h, C.byref(r)))
        return r.value

    def max_velocity(self):
        m, nan = C.c_double(), C.c_int32()
        _check(lib().life_case_max_velocity(self._h, C.byref(m), C.byref(nan)))
        return m.value, bool(nan.value)

    def bench_steps(self, n: int):
        """Run n steps; return (total_ms, mean interior-kernel ms, kernel launches),
        all measured with CUDA events on the case's stream."""
        tot, inner, launches = C.c_double(), C.c_double(), C.c_int32()
        _check(lib().life_case_bench_steps(self._h, int(n), C.byref(tot), C.byref(inner), C.byref(launches)))
        return tot.value, inner.value, launches.value

    def vtk_fields(self):
        """(density, pressure, velocity[.., 3]) as GridClass::writeVTK writes
        them, in VTK point order (``life_case_get_vtk_fields``)."""
        i = self.info()
        n = i.Nx * i.Ny
        dens, pres, vel = np.empty(n), np.empty(n), np.empty((n, 3))
        _check(lib().life_case_get_vtk_fields(self._h, _p(dens), _p(pres), _p(vel)))
        return dens, pres, vel

    def body_nodes(self):
        """(kind per body, global marker index of each body's markers in body
        order) (``life_case_get_body_nodes``)."""
        i = self.info()
        kind = np.zeros(max(i.n_bodies, 1), dtype=np.int32)
        idx = np.zeros(max(i.n_markers, 1), dtype=np.int32)
        _check(lib().life_case_get_body_nodes(self._h, _p(kind), _p(idx)))
        return kind[:i.n_bodies], idx[:i.n_markers]

    def total_force(self):
        fx, fy = C.c_double(), C.c_double()
        _check(lib().life_case_total_force(self._h, C.byref(fx), C.byref(fy)))
        return fx.value, fy.value

    def record(self, every: int, capacity: int = 4096) -> None:
        """Record the total force and the flexible bodies' tips every `every`
        steps on the device (``life_case_record``); 0 removes the recorder."""
        _check(lib().life_case_record(self._h, int(every), int(capacity)))

    def records(self, max_rows: int = 1 << 20) -> Dict[str, np.ndarray]:
        """Rows recorded since the last call (``life_case_records``): ``t``,
        ``force`` [n, 2], ``tip_pos`` / ``tip_vel`` [n, bodies, 2], ``dropped``."""
        n, cols, dropped = C.c_int32(), C.c_int32(), C.c_int32()
        _check(lib().life_case_records(self._h, 0, C.byref(n), C.byref(cols), None, None, C.byref(dropped)))
        max_rows = max(max_rows, n.value)
        t = np.zeros(max(max_rows, 1), dtype=np.int32)
        rows = np.zeros((max(max_rows, 1), max(cols.value, 1)))
        _check(lib().life_case_records(self._h, int(max_rows), C.byref(n), C.byref(cols), _p(t), _p(rows),
                                       C.byref(dropped)))
        k, nc = n.value, cols.value
        rows = rows[:k, :nc]
        nb = (nc - 2) // 4
        tips = rows[:, 2:].reshape(k, nb, 4) if nb else np.zeros((k, 0, 4))
        return {"t": t[:k].copy(), "force": rows[:, :2].copy(), "tip_pos": tips[:, :, :2].copy(),
                "tip_vel": tips[:, :, 2:].copy(), "dropped": dropped.value}


def measure_fp64_rate() -> float:
    """FP64 GFLOP/s this GPU sustains on independent FMA chains
    (``life_measure_fp64_rate``)."""
    g = C.c_double()
    _check(lib().life_measure_fp64_rate(C.byref(g)))
    return g.value


class Batch:
    """Many independent cases stepped together (``life_batch_*``).

    ``cases`` is a sequence of ``(params, bodies)``. :meth:`case` returns a
    borrowed :class:`Case` view of case k for the field, marker and FEM getters.
    """

    def __init__(self, cases: Sequence):
        L = lib()
        self._cases = [(p, expand_bodies(b)) for p, b in cases]
        n = len(self._cases)
        ps = (type(params_struct(self._cases[0][0])) * n)()
        for k, (p, _) in enumerate(self._cases):
            ps[k] = params_struct(p)
        allb = [b for _, bl in self._cases for b in bl]
        bs = body_structs(allb)
        nb = (C.c_int32 * n)(*[len(bl) for _, bl in self._cases])
        h = C.c_void_p()
        _check(L.life_batch_create(ps, C.byref(bs), nb, n, C.byref(h)))
        self._h = h
        self._views = {}

    def close(self) -> None:
        if getattr(self, "_h", None):
            for v in self._views.values():
                v._h = None
            lib().life_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __len__(self) -> int:
        return len(self._cases)

    def step(self, n: int = 1) -> None:
        _check(lib().life_batch_step(self._h, int(n)))

    def sync(self) -> None:
        _check(lib().life_batch_sync(self._h))

    def case(self, k: int) -> Case:
        if k not in self._views:
            h = C.c_void_p()
            _check(lib().life_batch_case(self._h, int(k), C.byref(h)))
            self._views[k] = Case(self._cases[k][0], _handle=h)
        _check(lib().life_batch_sync(self._h))
        return self._views[k]

    def info(self) -> LifeBatchInfo:
        inf = LifeBatchInfo()
        _check(lib().life_batch_info(self._h, C.byref(inf)))
        return inf

    def set_tile(self, w: int, h: int) -> None:
        _check(lib().life_batch_set_tile(self._h, int(w), int(h)))

    def autotune(self):
        w, h, ms = C.c_int32(), C.c_int32(), C.c_float()
        _check(lib().life_batch_autotune(self._h, C.byref(w), C.byref(h), C.byref(ms)))
        return w.value, h.value, ms.value

    def interior_ms(self, reps: int = 10) -> float:
        ms = C.c_float()
        _check(lib().life_batch_interior_ms(self._h, int(reps), C.byref(ms)))
        return ms.value

    def bench_steps(self, n: int):
        """Run n batch steps; return (device ms, kernel nodes per step graph)."""
        tot, kn = C.c_double(), C.c_int32()
        _check(lib().life_batch_bench_steps(self._h, int(n), C.byref(tot), C.byref(kn)))
        return tot.value, kn.value


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = range(4)


class Server:
    """Request loop on the GPU (``life_server_*``): submit cases, wait for
    them, take their final state as a :class:`Case`."""

    def __init__(self, hbm_budget: int, max_active: int = 0, steps_per_round: int = 0):
        cfg = LifeServerConfig(int(hbm_budget), int(max_active), int(steps_per_round))
        h = C.c_void_p()
        _check(lib().life_server_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self._params = {}

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().life_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, params: CaseParams, bodies: Sequence, steps: int) -> int:
        bodies = expand_bodies(bodies)
        ps = params_struct(params)
        bs = body_structs(bodies)
        rid = C.c_int64()
        _check(lib().life_server_submit(self._h, C.byref(ps), C.byref(bs), len(bodies), int(steps),
                                        C.byref(rid)))
        self._params[rid.value] = params
        return rid.value

    def query(self, rid: int) -> LifeRequestInfo:
        inf = LifeRequestInfo()
        _check(lib().life_server_query(self._h, int(rid), C.byref(inf)))
        return inf

    def wait(self, rid: int, timeout: float = -1.0) -> None:
        _check(lib().life_server_wait(self._h, int(rid), float(timeout)))

    def take(self, rid: int) -> Case:
        h = C.c_void_p()
        _check(lib().life_server_take(self._h, int(rid), C.byref(h)))
        c = Case(self._params[rid], _handle=h)
        c._owned = True
        return c

    def release(self, rid: int) -> None:
        _check(lib().life_server_release(self._h, int(rid)))

    def stats(self) -> LifeServerStats:
        st = LifeServerStats()
        _check(lib().life_server_stats(self._h, C.byref(st)))
        return st

    def drain(self, timeout: float = -1.0) -> None:
        _check(lib().life_server_drain(self._h, float(timeout)))


def parse_geometry(text: str):
    from .abi import LifeBodyDesc
    n = C.c_int32()
    _check(lib().life_parse_geometry(text.encode(), None, 0, C.byref(n)))
    arr = (LifeBodyDesc * max(1, n.value))()
    _check(lib().life_parse_geometry(text.encode(), C.byref(arr), n.value, C.byref(n)))
    return [arr[k] for k in range(n.value)]
