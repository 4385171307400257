"""Body start-up (ObjectsClass ctor: geometryReadIn, removeOverlapMarkers,
initialiseObjects with findSupport, computeDs, the epsilon solve and the
static pre-deflection of flexible bodies) is host code in the library
(``life_gb300/csrc/objects.cpp``). Here it is compiled for the host on its
own, with a small C wrapper, and run without a GPU: the markers (position,
velocity, epsilon, ds) and the flexible bodies' FEM state (U, node positions)
must equal the oracle's bit for bit, for the golden body cases (rigid and
flexible, uniform epsilon, overlapping markers) and for a case whose static
pre-deflection runs on several host threads. The marker overlap test runs
on the host here (the library sends sets of 2048 markers or more to a device
kernel that applies the same test; ``tests/test_gpu_startup.py`` checks that
the two agree)."""
import ctypes as C
import dataclasses
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from cases import golden_cases
from life_gb300.abi import LifeBodyDesc, LifeCaseParams, body_structs, params_struct

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "life_gb300", "csrc")

WRAPPER = r"""
#include "objects.h"
#include <cmath>
#include <cstring>
using namespace life;

// the lattice scalars as life_case_create forms them (GridClass ctor)
static Grid0 grid_of(const LifeCaseParams* p) {
    const double rho0 = 1.0, cs = 1.0 / std::sqrt(3.0), tau = 1.0 / p->omega;
    const double nu = (tau - 0.5) * (cs * cs);
    const double Dx = p->height_p / (p->Ny - 1);
    const double Dt = (Dx * Dx) * nu / p->nu_p;
    const double Dm = (p->rho_p / rho0) * (Dx * Dx * Dx);
    return Grid0{p->Nx, p->Ny, Dx, Dt, Dm, p->gravityX, p->gravityY, p->ref_L, p->alpha, p->delta};
}

extern "C" int startup_host(const LifeCaseParams* p, const LifeBodyDesc* d, int nd, int cap, double* pos,
                            double* vel, double* eps, double* ds, int* nm, int fcap, double* U, double* npos,
                            int* dofs, int* nflex, char* err, int errcap) {
    HObjects o;
    std::string e;
    const int rc = build_objects(grid_of(p), *p, d, nd, o, &e, nullptr, 0);
    if (rc) {
        std::strncpy(err, e.c_str(), errcap - 1);
        err[errcap - 1] = 0;
        return rc;
    }
    *nm = (int)o.m.size();
    if (*nm > cap) return -1;
    for (int k = 0; k < *nm; k++) {
        for (int c = 0; c < 2; c++) {
            pos[2 * k + c] = o.m[k].pos[c];
            vel[2 * k + c] = o.m[k].vel[c];
        }
        eps[k] = o.m[k].eps;
        ds[k] = o.m[k].ds;
    }
    int f = 0, off = 0;
    for (const HBody& b : o.b) {
        if (!b.flex || !b.fem) continue;
        const HFem& F = *b.fem;
        if (off + F.dofs > fcap) return -2;
        dofs[f] = F.dofs;
        for (int q = 0; q < F.dofs; q++) U[off + q] = F.U[q];
        for (int q = 0; q < 2 * F.nNodes; q++) npos[2 * off / 3 + q] = F.pos[q];
        off += F.dofs;
        f++;
    }
    *nflex = f;
    return 0;
}
"""


@pytest.fixture(scope="module")
def lib():
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not found")
    d = tempfile.mkdtemp(prefix="startup_host_")
    src, so = os.path.join(d, "wrapper.cpp"), os.path.join(d, "libstartup.so")
    with open(src, "w") as fh:
        fh.write(WRAPPER)
    cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-I", CSRC,
           "-I", os.path.join(ROOT, "include"), src, os.path.join(CSRC, "objects.cpp"), "-o", so]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    L = C.CDLL(so)
    L.startup_host.restype = C.c_int
    yield L
    shutil.rmtree(d, ignore_errors=True)


def host_startup(L, p, b):
    ps = params_struct(p)
    bs = body_structs(list(b))
    cap, fcap = 20000, 20000
    pos, vel = np.empty((cap, 2)), np.empty((cap, 2))
    eps, ds = np.empty(cap), np.empty(cap)
    U, npos = np.empty(fcap), np.empty(fcap)
    dofs = np.zeros(256, dtype=np.int32)
    nm, nflex = C.c_int(0), C.c_int(0)
    err = C.create_string_buffer(512)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    rc = L.startup_host(C.byref(ps), bs, len(b), cap, dp(pos), dp(vel), dp(eps), dp(ds), C.byref(nm), fcap,
                        dp(U), dp(npos), dofs.ctypes.data_as(C.POINTER(C.c_int)), C.byref(nflex), err, 512)
    assert rc == 0, (rc, err.value)
    n = nm.value
    out = dict(pos=pos[:n], vel=vel[:n], epsilon=eps[:n], ds=ds[:n], fem=[])
    off = 0
    for k in range(nflex.value):
        m = int(dofs[k])
        out["fem"].append(dict(U=U[off:off + m].copy(), pos=npos[2 * off // 3:2 * off // 3 + 2 * (m // 3)].reshape(-1, 2)))
        off += m
    return out


def compare_with_oracle(got, p, b):
    from oracle.pyoracle import Oracle
    o = Oracle(p, b)
    try:
        mo = o.markers()
        assert len(got["pos"]) == o.n_markers
        for key in ("pos", "vel", "epsilon", "ds"):
            assert np.array_equal(got[key], mo[key]), key
        assert len(got["fem"]) == o.n_flex
        for k in range(o.n_flex):
            fo = o.fem(k)
            assert np.array_equal(got["fem"][k]["U"], fo["U"]), k
            assert np.array_equal(got["fem"][k]["pos"], fo["pos"]), k
    finally:
        o.close()


BODY_CASES = [k for k, (_, b) in golden_cases().items() if b]


@pytest.mark.parametrize("name", BODY_CASES)
def test_host_startup_equals_oracle(lib, name):
    p, b = golden_cases()[name]
    compare_with_oracle(host_startup(lib, p, b), p, b)


def test_host_startup_with_static_deflection_of_several_bodies_equals_oracle(lib):
    p, b = golden_cases()["honami_like_cm"]
    p = dataclasses.replace(p, initial_deflect=0.05)
    got = host_startup(lib, p, b)
    assert len(got["fem"]) > 1  # several flexible bodies: one host thread each
    compare_with_oracle(got, p, b)
