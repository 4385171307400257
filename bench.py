#!/usr/bin/env python3
"""Benchmark of the GB300 LIFE hot path (D2Q9 stream-collide + boundary conditions).

Workload: the lid-driven cavity of the reference's plain-method configuration
(regularised velocity lid u = 0.1, regularised no-slip walls, BGK, tau = 0.5768)
scaled to a 4096 x 4096 lattice, the size the headline roofline target is
quoted on. One "step" is one time step of the whole lattice. The headline form
is the FP32 shifted-population storage; FP64 (bit-exact with the reference)
and FP16 storage are measured beside it, with their velocity error against the
FP64 run after the same steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Each rank runs an independent replica (the reference has no domain
decomposition and the path is timed replicas-only); `value` is the sum over
ranks. Timing: W untimed steps, then K steps bracketed by a barrier and a
device synchronise, measured with CUDA events on the case's stream. The lattice
state (2 x 9 x 4 B x 16.8M sites = 1.2 GB) is far larger than L2, so no flush
is needed between steps.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MLUPS & HBM-roofline %, FP32 vs FP64 at stated error; p50/p99 solve latency"
WORKLOAD = "lid_driven_cavity_4096x4096_d2q9_bgk"


def cavity_params(n: int, precision: int, cm: bool = False):
    """The lid-driven cavity (BGK, lid 0.1, tau 0.5768) on an n x n lattice."""
    from life_gb300 import configs
    return configs.cavity(n, precision, cm)


def cylinder_params(precision: int):
    """Rigid cylinder channel: 1000 x 400, central moments, D = 40, inlet 0.04,
    convective outlet, Re = 100 (tau = 0.548)."""
    from life_gb300 import configs
    return configs.cylinder(precision)


def filament_params(precision: int):
    """Flexible filament channel: 1200 x 400 BGK, inlet 0.05, convective outlet,
    one filament L = 80 clamped at (300, 200), 80 corotational elements,
    EI/(rho U^2 L^3) = 0.2 (E = 3072 with H = 1), mass ratio 0.5 (rho_s = 40),
    Re = 100 on L (tau = 0.62), initial tip deflection 0.03 L."""
    from life_gb300 import configs
    return configs.filament(precision)


def _pinned_array(shape):
    """A page-locked float64 host array (zeroed), through torch's pinned host
    allocator; a plain array when no pinned memory can be had."""
    import numpy as np
    try:
        import torch
        t = torch.zeros(int(np.prod(shape)), dtype=torch.float64, pin_memory=True)
        a = t.numpy().reshape(shape)
        _pinned_array.keep.append(t)  # the array borrows the tensor's memory
        return a
    except Exception:
        return np.zeros(shape)


_pinned_array.keep = []


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class NvmlSampler:
    """SM clock and clock-event reasons read through NVML (libnvidia-ml, read
    only) every `period` seconds on a thread, so that timed regions of tens of
    milliseconds still get many samples."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, device: int, period: float = 0.002):
        import ctypes
        import threading
        self.C, self.period = ctypes, period
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        if self.lib.nvmlDeviceGetHandleByIndex_v2(device, ctypes.byref(self.h)) != 0:
            raise RuntimeError("no NVML handle")
        self.reason_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.lib.nvmlDeviceGetCurrentClocksThrottleReasons
        self.rows, self.stop, self.th = [], threading.Event(), None
        self.threading = threading

    def _read(self):
        C = self.C
        mhz, mx, rs = C.c_uint(), C.c_uint(), C.c_ulonglong()
        self.lib.nvmlDeviceGetClockInfo(self.h, 1, C.byref(mhz))
        self.lib.nvmlDeviceGetMaxClockInfo(self.h, 1, C.byref(mx))
        self.reason_fn(self.h, C.byref(rs))
        return mhz.value, mx.value, rs.value

    def __enter__(self):
        def run():
            while not self.stop.is_set():
                self.rows.append(self._read())
                self.stop.wait(self.period)
        self.rows.append(self._read())
        self.th = self.threading.Thread(target=run, daemon=True)
        self.th.start()
        return self

    def __exit__(self, *exc):
        self.stop.set()
        self.th.join()
        self.rows.append(self._read())

    def summary(self):
        sm = sorted(r[0] for r in self.rows)
        reasons = sorted({name for r in self.rows for bit, name in self.REASONS.items() if r[2] & bit})
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(r[1] for r in self.rows), "reasons": reasons,
                "samples": len(self.rows), "source": "nvml"}


class ClockSampler:
    """Clocks and throttle reasons during the timed region: NVML when it
    loads, else nvidia-smi at 200 ms."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        vis = os.environ.get("CUDA_VISIBLE_DEVICES")
        if vis:
            ids = [x.strip() for x in vis.split(",") if x.strip()]
            if device < len(ids) and ids[device].isdigit():
                device = int(ids[device])
        self.device = device
        self.proc = None
        self.path = None
        self.nvml = None

    def __enter__(self):
        try:
            self.nvml = NvmlSampler(self.device).__enter__()
            return self
        except Exception:
            self.nvml = None
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.nvml is not None:
            self.nvml.__exit__(*exc)
            return
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.nvml is not None:
            return self.nvml.summary()
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except Exception:
            pass
        finally:
            if self.path and os.path.exists(self.path):
                os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = sorted(float(r[1]) for r in rows if r[1].replace(".", "").isdigit())
        smax = max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": smax, "reasons": reasons,
                "samples": len(rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_oracle_mlups(params, steps: int, warmup: int):
    """The oracle (C restatement of the reference, OpenMP over all host
    cores) timed on the same lattice."""
    from oracle.pyoracle import Oracle
    o = Oracle(params)
    o.step(warmup)
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    o.close()
    return params.Nx * params.Ny * steps / dt / 1e6, dt


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    from life_gb300.case import PREC_F64
    n = args.nx
    p = cavity_params(n, PREC_F64)
    mlups, dt = cpu_oracle_mlups(p, args.steps, args.warmup)
    cores = os.cpu_count()
    line = {
        "impl": "reference", "metric": METRIC, "value": round(mlups, 3), "unit": "MLUPS",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dt * 1e3 / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (analytic initial state)",
        "config": {"workload": f"lid_driven_cavity_{n}x{n}_d2q9_bgk", "lattice": [n, n], "collision": "BGK",
                   "l2": "state larger than L2"},
        "cpu_baseline": {"value": round(mlups, 3), "unit": "MLUPS", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full steps of the {n}x{n} lattice after {args.warmup} warm-up"},
        "e2e": {"value": round(mlups, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_workload(args, world, rank):
    """Single-workload timing (--workload cylinder|filament): FP64 and FP32
    MLUPS of one IBM case, used for profiling the immersed-body path."""
    from life_gb300.build import build
    from life_gb300.case import PREC_F32, PREC_F64
    build()
    from life_gb300.lib import Case
    if args.workload == "ensemble":
        tile = tuple(int(x) for x in args.tile.split("x")) if args.tile else None
        out = {"workload": f"ensemble{args.cases}",
               **ensemble_leg(args.steps, args.warmup, args.cases, tile, not args.batch_only)}
        if rank == 0:
            print(json.dumps(out), flush=True)
        return 0
    if args.workload == "serve":
        out = {"workload": "serving_canopy", **serving_leg(args.requests, args.step_scale)}
        if rank == 0:
            print(json.dumps(out), flush=True)
        return 0
    if args.workload == "spread":
        out = {"workload": "spread_scaling", **spread_leg(steps=args.steps, warmup=args.warmup)}
        if rank == 0:
            print(json.dumps(out), flush=True)
        return 0
    if args.workload == "accuracy":
        out = {"workload": "accuracy", **accuracy_leg(args.steps, max(args.steps // 25, 50))}
        if rank == 0:
            print(json.dumps(out), flush=True)
        return 0
    make = cylinder_params if args.workload == "cylinder" else filament_params
    out = {"workload": args.workload}
    for prec, tag in ((PREC_F64, "fp64"), (PREC_F32, "fp32")):
        p, b = make(prec)
        c = Case(p, b)
        c.step(args.warmup)
        tt, inner, launches = c.bench_steps(args.steps)
        st = c.status()
        out[f"{tag}_mlups"] = round(p.Nx * p.Ny * args.steps / (tt * 1e-3) / 1e6, 1)
        out[f"{tag}_ms_per_step"] = round(tt / args.steps, 4)
        out[f"{tag}_lattice_ms"] = round(inner, 4)
        out[f"{tag}_launches_per_step"] = launches / args.steps
        out["last_subiterations"] = st.last_subits
        out["last_nr_iterations"] = st.last_nr_its
        del c
    if rank == 0:
        print(json.dumps(out), flush=True)
    return 0


def spread_leg(counts=(0, 16, 32, 64, 128), steps: int = 200, warmup: int = 5) -> dict:
    """IBM cost against marker count: a row of N rigid stalks (30 lattice
    units, 31 markers each, the Honami example's stalks) clamped on the
    bottom wall of a 3106 x 91 boundary-layer channel (the Honami example's
    lattice), central moments, FP64. ms per step for each N; the IBM cost is
    the difference to the same lattice without bodies."""
    from life_gb300.case import BOUNDARY_LAYER, CONVECTIVE, FREESLIP, VELOCITY, WALL, CaseParams, Filament
    from life_gb300.lib import Case
    tau = 0.55
    out = {"lattice": [3106, 91], "steps": steps, "points": []}
    base = None
    for n in counts:
        p = CaseParams(Nx=3106, Ny=91, height_p=90.0, rho_p=1.0, nu_p=(tau - 0.5) / 3.0, omega=1.0 / tau,
                       wall_left=VELOCITY, wall_right=CONVECTIVE, wall_bottom=WALL, wall_top=FREESLIP,
                       profile=BOUNDARY_LAYER, uxInlet_p=0.04, inlet_ramp=50.0, central_moments=True, ref_L=30.0)
        gap = 2900.0 / max(n, 1)
        b = ([Filament(x=100.0, y=0.0, length=30.0, height=1.0, angle_deg=90.0, flexible=False, n_elements=None,
                       clamped=True, rho=1.0, E=1.0, ID=0, number=n, dx=gap)] if n else [])
        with Case(p, b) as c:
            c.step(warmup)
            tt, _, launches = c.bench_steps(steps)
            markers = c.info().n_markers
        ms = tt / steps
        if n == 0:
            base = ms
        out["points"].append({"stalks": n, "markers": markers, "ms_per_step": round(ms, 4),
                              "ibm_ms_per_step": round(ms - base, 4) if base is not None else None})
    return out


def _upward_crossings(t, y):
    """Times at which y - mean(y) crosses zero upwards (linear interpolation)."""
    import numpy as np
    y = np.asarray(y) - float(np.mean(y))
    k = np.flatnonzero((y[:-1] < 0.0) & (y[1:] >= 0.0))
    return [t[i] + (t[i + 1] - t[i]) * (-y[i]) / (y[i + 1] - y[i]) for i in k]


def cylinder_forces(precision: int, steps: int, every: int = 25) -> dict:
    """Drag and lift coefficients of the 1000 x 400 cylinder over `steps`
    steps: C = F / (0.5 rho U^2 D) with F the total force on the body as
    ObjectsClass::writeTotalForces forms it (src/Objects.cpp:518-528),
    sampled every `every` steps. Statistics over the second half: mean Cd,
    lift amplitude (half the peak-to-peak), shedding period from the upward
    zero crossings of Cl."""
    import numpy as np
    from life_gb300.lib import Case
    p, b = cylinder_params(precision)
    nd = 0.5 * 1.0 * 0.04 ** 2 * 40.0
    ts, cd, cl = [], [], []
    with Case(p, b) as c:
        while c.t < steps:
            c.step(min(every, steps - c.t))
            fx, fy = c.total_force()
            ts.append(c.t)
            cd.append(fx / nd)
            cl.append(fy / nd)
    ts, cd, cl = np.array(ts, dtype=float), np.array(cd), np.array(cl)
    h = len(ts) // 2
    up = _upward_crossings(ts[h:], cl[h:])
    period = float(np.mean(np.diff(up))) if len(up) >= 2 else None
    return {"t": ts, "cd": cd, "cl": cl, "cd_mean": float(cd[h:].mean()),
            "cl_amp": float(0.5 * (cl[h:].max() - cl[h:].min())), "period_steps": period}


def filament_tip(precision: int, steps: int, every: int = 50) -> dict:
    """Transverse tip displacement (y of the last FEM node minus its
    undeformed y, over L) of the 1200 x 400 filament, sampled every `every`
    steps."""
    import numpy as np
    from life_gb300.lib import Case
    p, b = filament_params(precision)
    L = b[0].length
    ys = []
    with Case(p, b) as c:
        while c.t < steps:
            c.step(min(every, steps - c.t))
            fm = c.fem(0)
            ys.append((fm["pos"][-1, 1] - fm["pos0"][-1, 1]) / L)
    return {"tip": np.array(ys)}


def accuracy_leg(cyl_steps: int = 50000, fil_steps: int = 2000) -> dict:
    """FP32 shifted populations against the FP64 form (bit-identical to the
    reference) on the two immersed-body workloads: cylinder drag, lift and
    shedding period after cyl_steps steps; filament tip displacement over
    fil_steps steps (FEM, epsilon and Aitken in FP64 in both)."""
    import numpy as np
    out = {"cylinder_steps": cyl_steps}
    t0 = time.perf_counter()
    r = {tag: cylinder_forces(prec, cyl_steps) for prec, tag in ((0, "fp64"), (1, "fp32"))}
    for tag in ("fp64", "fp32"):
        out[f"cylinder_{tag}_cd"] = round(r[tag]["cd_mean"], 6)
        out[f"cylinder_{tag}_cl_amp"] = round(r[tag]["cl_amp"], 6)
        per = r[tag]["period_steps"]
        out[f"cylinder_{tag}_shedding_period_steps"] = None if per is None else round(per, 1)
        out[f"cylinder_{tag}_strouhal"] = None if per is None else round(40.0 / (0.04 * per), 5)
    a, b = r["fp64"], r["fp32"]
    out["cylinder_cd_rel_err"] = abs(b["cd_mean"] - a["cd_mean"]) / abs(a["cd_mean"])
    out["cylinder_cl_amp_rel_err"] = (abs(b["cl_amp"] - a["cl_amp"]) / a["cl_amp"]) if a["cl_amp"] > 0 else None
    if a["period_steps"] and b["period_steps"]:
        out["cylinder_period_rel_err"] = abs(b["period_steps"] - a["period_steps"]) / a["period_steps"]
    # pointwise, relative to the lift amplitude (drag: to its mean)
    out["cylinder_cd_series_max_rel_err"] = float(np.abs(b["cd"] - a["cd"]).max() / abs(a["cd_mean"]))
    if a["cl_amp"] > 0:
        out["cylinder_cl_series_max_err_over_amp"] = float(np.abs(b["cl"] - a["cl"]).max() / a["cl_amp"])
    out["filament_steps"] = fil_steps
    f64, f32 = filament_tip(0, fil_steps)["tip"], filament_tip(1, fil_steps)["tip"]
    out["filament_fp64_tip_over_L_final"] = round(float(f64[-1]), 6)
    out["filament_fp64_tip_over_L_range"] = [round(float(f64.min()), 6), round(float(f64.max()), 6)]
    out["filament_tip_max_err_over_L"] = float(np.abs(f32 - f64).max())
    span = float(f64.max() - f64.min())
    out["filament_tip_max_err_over_swing"] = float(np.abs(f32 - f64).max() / span) if span > 0 else None
    out["seconds"] = round(time.perf_counter() - t0, 1)
    return out


def ensemble_leg(steps: int, warmup: int, n_cases: int = 64, tile=None, sequential: bool = True,
                 fp16_steps: int = None, seq_steps: int = None, long_error: bool = False) -> dict:
    """The 64-case batched ensemble (uneven lattices, cylinders or filament
    rows, BGK/CM, Re 50-300): batched FP32 over `steps` steps and FP16 over
    `fp16_steps` (one persistent interior launch and one replayed graph per
    batch step, autotuned tiles) against the same cases stepped one after
    another through life_case_step in FP64 and FP32 over `seq_steps` steps
    each (a bounded sample). MLUPS = sum of lattice sites x steps / device
    time. With long_error, the same cases are also run as an FP64 batch for
    the FP32 batch's whole length and every case's final velocity field is
    compared: the FP32 error after the configured run, not a short sample."""
    import numpy as np
    from life_gb300.ensemble import ensemble_cases, sites
    from life_gb300.lib import Batch, Case
    out = {}
    u32 = {}
    total32 = 0
    nsteps = {1: steps, 2: steps if fp16_steps is None else fp16_steps}
    for prec, tag in ((1, "fp32"), (2, "fp16")):
        steps = nsteps[prec]
        cs = ensemble_cases(n=n_cases, precision=prec)
        with Batch(cs) as B:
            B.step(warmup)
            if tile:
                w, h = tile
                B.set_tile(w, h)
            else:
                w, h, ms = B.autotune()
            B.step(warmup)
            tot, kn = B.bench_steps(steps)
            inf = B.info()
            out[f"batched_{tag}_steps"] = steps
            out[f"batched_{tag}_mlups"] = round(inf.sites * steps / (tot * 1e-3) / 1e6, 1)
            out[f"batched_{tag}_ms_per_step"] = round(tot / steps, 4)
            out[f"batched_{tag}_interior_ms"] = round(B.interior_ms(10), 4)
            out[f"batched_{tag}_tile"] = [w, h]
            out[f"batched_{tag}_kernel_nodes_per_step"] = kn
            out[f"batched_{tag}_device_gb"] = round(inf.device_bytes / 1e9, 3)
            if prec == 1 and long_error:
                total32 = B.case(0).t
                u32 = {k: B.case(k).fields(("u",))["u"] for k in range(len(cs))}
    if long_error:
        # the FP64 batch (the reference's arithmetic) over the same steps
        t0 = time.perf_counter()
        errs = []
        with Batch(ensemble_cases(n=n_cases, precision=0)) as B:
            B.step(total32)
            for k in range(n_cases):
                u64 = B.case(k).fields(("u",))["u"]
                errs.append(float(np.abs(u32[k] - u64).max() / np.abs(u64).max()))
        out["fp32_velocity_rel_err_after_full_run"] = {
            "steps": total32, "max_over_cases": max(errs), "median_over_cases": float(np.median(errs)),
            "cases_above_1e-5": int(sum(e > 1e-5 for e in errs)), "fp64_batch_seconds": round(time.perf_counter() - t0, 1)}
        del u32
    cs = ensemble_cases(n=n_cases)
    out["cases"] = len(cs)
    out["sites"] = sites(cs)
    out["bodies"] = sum(len(b) for _, b in cs)
    if not sequential:
        return out
    # sequential per-case runs; the FP32 and FP16 states are compared with the
    # FP64 state after the same steps (a case in a batch is bit-identical to
    # the case alone, so this is the batched forms' error too)
    import numpy as np
    import dataclasses
    k = seq_steps if seq_steps else max(10, nsteps[1] // 5)
    n_ss, ms = 0, {0: 0.0, 1: 0.0}
    err = {1: 0.0, 2: 0.0}
    for p, b in ensemble_cases(n=n_cases, precision=0):
        u = {}
        for prec in (0, 1, 2):
            with Case(dataclasses.replace(p, precision=prec), b) as c:
                c.step(warmup)
                if prec in ms:
                    tt, _, _ = c.bench_steps(k)
                    ms[prec] += tt
                else:
                    c.step(k)
                u[prec] = c.fields(("u",))["u"]
        n_ss += p.Nx * p.Ny * k
        umax = float(np.abs(u[0]).max())
        for prec in (1, 2):
            err[prec] = max(err[prec], float(np.abs(u[prec] - u[0]).max()) / umax)
    for prec, tag in ((0, "fp64"), (1, "fp32")):
        out[f"sequential_{tag}_mlups"] = round(n_ss / (ms[prec] * 1e-3) / 1e6, 1)
    out["fp32_velocity_rel_err_max_over_cases"] = err[1]
    out["fp16_velocity_rel_err_max_over_cases"] = err[2]
    out["error_after_steps"] = warmup + k
    out["batched_fp32_over_sequential_fp64"] = round(out["batched_fp32_mlups"] / out["sequential_fp64_mlups"], 2)
    out["batched_fp32_over_sequential_fp32"] = round(out["batched_fp32_mlups"] / out["sequential_fp32_mlups"], 2)
    return out


def serving_leg(n_requests: int = 24, step_scale: float = 0.25, seed: int = 7, load: float = 0.8,
                error_samples: int = 4) -> dict:
    """Serving: a seeded Poisson stream of canopy requests (8-32 stalks of 20
    elements, 512-4096 x 256-1024 lattices, FP32 lattice / FP64 FEM) against
    a 160 GB admission budget, continuous batching on one GB300.

    1. capacity: the first 8 requests submitted at once, aggregate site
       updates per second until they drain;
    2. stream: arrivals at rate load x capacity / mean request work, each
       request released as soon as it finishes; latency = finish - submit;
    3. baseline: the same kind of request solved alone in FP64 through
       life_case_step, one after another (bounded sample of steps);
    4. error: the `error_samples` requests with the least work are taken from
       the server when they finish and compared with the same request solved
       alone in FP64 (the reference's arithmetic) for the same steps: max
       |u - u64| / max |u64| per request.
    Step counts are the request's 2000-20000 steps times step_scale."""
    import numpy as np
    from life_gb300.ensemble import canopy_case
    from life_gb300.lib import REQ_DONE, Case, LifeError, Server
    rng = np.random.Generator(np.random.PCG64(seed))
    reqs = []
    for _ in range(n_requests):
        p, b, steps = canopy_case(rng, precision=1)
        reqs.append((p, b, max(10, int(round(steps * step_scale)))))
    work = [p.Nx * p.Ny * s for p, _, s in reqs]
    budget = 160 << 30
    out = {"requests": n_requests, "step_scale": step_scale, "hbm_budget_gb": 160, "load": load}
    # 0. one short untimed request, so that loading the kernels of this
    # request type happens before anything is timed
    with Server(hbm_budget=budget, steps_per_round=100) as S:
        p, b, _ = reqs[0]
        S.wait(S.submit(p, b, 10), timeout=600)
    # 1. capacity at saturation
    with Server(hbm_budget=budget, steps_per_round=100) as S:
        burst = reqs[:8]
        ids = [S.submit(p, b, s) for p, b, s in burst]
        S.drain(timeout=3600)
        infos = [S.query(i) for i in ids]
        span = max(i.done_s for i in infos) - min(i.submit_s for i in infos)
        # a request that fails (the subiteration cap) does not count as work
        cap = sum(w for w, i in zip(work[:8], infos) if i.state == REQ_DONE) / span
        for i in ids:
            S.release(i)
    out["capacity_mlups"] = round(cap / 1e6, 1)
    # 2. Poisson stream at `load` of capacity
    lam = load * cap / float(np.mean(work))
    gaps = rng.exponential(1.0 / lam, size=n_requests)
    sampled = set(sorted(range(n_requests), key=lambda k: work[k])[:error_samples])
    u_served = {}
    with Server(hbm_budget=budget, steps_per_round=100) as S:
        t0 = time.perf_counter()
        ids = []
        for k, (p, b, s) in enumerate(reqs):
            due = t0 + float(np.sum(gaps[:k + 1]))
            while True:
                dt = due - time.perf_counter()
                if dt <= 0:
                    break
                time.sleep(min(dt, 0.01))
            ids.append(S.submit(p, b, s))
        lat, infos, done_work = [], [], 0
        for k, (i, w) in enumerate(zip(ids, work)):
            try:
                S.wait(i, timeout=7200)
            except LifeError:
                pass  # a failed request fails alone; counted in st.failed
            inf = S.query(i)
            infos.append(inf)
            if inf.state == REQ_DONE:
                lat.append(inf.done_s - inf.submit_s)
                done_work += w
            if k in sampled and inf.state == REQ_DONE:
                with S.take(i) as c:
                    u_served[k] = c.fields(("u",))["u"]
            else:
                S.release(i)
        st = S.stats()
    span = max(i.done_s for i in infos) - min(i.submit_s for i in infos)
    lat = np.array(lat if lat else [float("nan")])
    out.update({
        "arrival_rate_per_s": round(lam, 3),
        "latency_s_p50": round(float(np.percentile(lat, 50)), 4),
        "latency_s_p95": round(float(np.percentile(lat, 95)), 4),
        "latency_s_p99": round(float(np.percentile(lat, 99)), 4),
        "latency_s_max": round(float(lat.max()), 4),
        "aggregate_mlups": round(done_work / span / 1e6, 1),
        "busy_fraction": round(st.busy_s / max(st.clock_s, 1e-9), 3),
        "peak_device_gb": round(st.bytes_peak / 1e9, 2),
        "rounds": st.rounds, "regroups": st.regroups, "failed": st.failed,
    })
    # 3. sequential plain FP64, bounded sample
    n_ss, ms_tot = 0, 0.0
    for p, b, s in reqs[:4]:
        import dataclasses
        p64 = dataclasses.replace(p, precision=0)
        with Case(p64, b) as c:
            c.step(3)
            k = min(s, 40)
            tt, _, _ = c.bench_steps(k)
        ms_tot += tt
        n_ss += p.Nx * p.Ny * k
    out["sequential_fp64_mlups"] = round(n_ss / (ms_tot * 1e-3) / 1e6, 1)
    # 4. served FP32 result against the request solved alone in FP64
    import dataclasses
    errs = {}
    for k, u in u_served.items():
        p, b, s = reqs[k]
        with Case(dataclasses.replace(p, precision=0), b) as c:
            c.step(s)
            u64 = c.fields(("u",))["u"]
        errs[k] = float(np.abs(u - u64).max() / np.abs(u64).max())
    out["served_fp32_velocity_rel_err_vs_fp64_solo"] = {
        "requests": sorted(errs), "steps": [reqs[k][2] for k in sorted(errs)],
        "errors": [errs[k] for k in sorted(errs)], "max": max(errs.values()) if errs else None}
    out["aggregate_over_sequential_fp64"] = round(out["aggregate_mlups"] / out["sequential_fp64_mlups"], 2)
    # under an open (Poisson) stream the aggregate follows the arrival rate;
    # the capacity is what the server sustains
    out["capacity_over_sequential_fp64"] = round(out["capacity_mlups"] / out["sequential_fp64_mlups"], 2)
    return out


def fp64_block(args, n: int, world: int) -> dict:
    """The FP64 form (the reference's arithmetic, bit for bit) on the same
    lattice: device MLUPS, its interior kernel against the FP64 rate this GPU
    sustains (the bound) and against HBM, and its own end-to-end figure
    through the C-ABI (create, K steps, velocity field to host)."""
    from life_gb300.case import PREC_F64
    from life_gb300.lib import Case, measure_fp64_rate
    sites = n * n
    k = args.steps
    c = Case(cavity_params(n, PREC_F64))
    c.step(args.warmup)
    c.sync()
    tot, inner, launches = c.bench_steps(k)
    del c
    out = {"value": round(sites * k / (tot * 1e-3) / 1e6, 1), "unit": "MLUPS", "steps": k,
           "ms_per_step": round(tot / k, 4), "kernel_ms": round(inner, 4), "gpu_launches": launches}
    hbm, hbm_kind = peaks()
    gbs = 144 * sites / (inner * 1e-3) / 1e9
    out["hbm"] = {"achieved": round(gbs, 1), "peak": hbm, "unit": "GB/s", "frac": round(gbs / hbm, 4),
                  "peak_source": f"{hbm_kind} hbm_gbs", "algorithmic_bytes_per_site": 144}
    # the FP64 unit issues one add, multiply or FMA per slot: the bound is
    # FP64 instructions per second, the peak the FMA probe's rate / 2
    rate = measure_fp64_rate()
    fl = None
    fpath = os.path.join(ROOT, "profiles", "interior_f64_flops.json")
    if os.path.exists(fpath):
        with open(fpath) as fh:
            fl = json.load(fh)
    roof = {"bound": "fp64", "peak": round(rate / 2, 1), "unit": "G FP64 instr/s",
            "peak_source": f"measured here: life_measure_fp64_rate {rate:.0f} GFLOP/s of FMA chains = "
                           f"{rate / 2:.0f} G FMA instr/s, all SMs",
            "kernel": "k_interior_f64<BGK>"}
    if fl:
        per = float(fl["fp64_instructions_per_site"])
        ach = per * sites / (inner * 1e-3) / 1e9
        roof.update({"achieved": round(ach, 1), "frac": round(ach / (rate / 2), 4),
                     "fp64_instructions_per_site": per, "fp64_flops_per_site": fl.get("fp64_flops_per_site"),
                     "per_site_source": fl.get("source")})
    out["roofline"] = roof
    # end to end through the C-ABI, as the headline's e2e
    u = _pinned_array((sites, 2))
    t0 = time.perf_counter()
    ce = Case(cavity_params(n, PREC_F64))
    ce.step(k)
    ce.fields(("u",), out={"u": u})
    e2e_s = time.perf_counter() - t0
    del ce, u
    out["e2e"] = {"value": round(world * sites * k / e2e_s / 1e6, 1), "unit": "MLUPS",
                  "h2d_bytes_per_step": round((376 + 16 * n + 32 * (k + 2)) / k),
                  "d2h_bytes_per_step": round(sites * 16 / k),
                  "what": "create from params + K steps + velocity field to host, wall clock"}
    return out


def run_gb300(args, world, rank, local):
    import numpy as np
    from life_gb300.build import build
    from life_gb300.case import PREC_F16, PREC_F32, PREC_F64
    build()
    from life_gb300.lib import Case
    n = args.nx
    sites = n * n
    hbm, hbm_kind = peaks()

    # ---- headline: FP32 shifted populations (--storage selects another form
    # for a headline-only run, e.g. to profile that form's kernel)
    form = {"fp32": (PREC_F32, 4, "f32", "fp32 shifted populations (f - w)"),
            "fp16": (PREC_F16, 2, "f16", "fp16 scaled shifted populations ((f - w) / s_v)"),
            "fp64": (PREC_F64, 8, "f64", "fp64 populations (reference arithmetic)")}[args.storage]
    if args.storage != "fp32" and not args.quick:
        raise SystemExit("--storage other than fp32 needs --quick (the extras compare the forms themselves)")
    c32 = Case(cavity_params(n, form[0]))
    c32.step(args.warmup)
    c32.sync()
    barrier(world)
    with ClockSampler(local) as clk:
        tot_ms, inner_ms, launches = c32.bench_steps(args.steps)
    barrier(world)
    tot_ms = max_over_ranks(world, tot_ms)
    clocks = clk.summary()
    ms_step = tot_ms / args.steps
    value = world * sites * args.steps / (tot_ms * 1e-3) / 1e6
    bytes_per_site = 18 * form[1]
    achieved = bytes_per_site * sites / (inner_ms * 1e-3) / 1e9

    extras = {}
    fp64 = fp64_block(args, n, world) if args.storage == "fp32" else None
    if not args.quick:
        # ---- FP64 (reference-exact) and FP16 storage on the same lattice
        k2 = max(10, args.steps // 2)
        c64 = Case(cavity_params(n, PREC_F64))
        c64.step(args.warmup)
        t64, i64, _ = c64.bench_steps(k2)
        extras["fp64_mlups"] = round(sites * k2 / (t64 * 1e-3) / 1e6, 1)
        extras["fp64_interior_gbs"] = round(144 * sites / (i64 * 1e-3) / 1e9, 1)
        c16 = Case(cavity_params(n, PREC_F16))
        c16.step(args.warmup)
        t16, i16, _ = c16.bench_steps(k2)
        extras["fp16_mlups"] = round(sites * k2 / (t16 * 1e-3) / 1e6, 1)
        extras["fp16_interior_gbs"] = round(36 * sites / (i16 * 1e-3) / 1e9, 1)
        extras["fp32_over_fp64"] = round(value / world / extras["fp64_mlups"], 3)
        # velocity error after the same number of steps (FP64 GPU = reference bits)
        done = args.warmup + args.steps
        c64.step(done - c64.t)
        c16.step(done - c16.t)
        ref = c64.fields(("rho", "u", "f"))
        umax = np.abs(ref["u"]).max()
        for name, c in (("fp32", c32), ("fp16", c16)):
            got = c.fields(("rho", "u", "f"))
            extras[f"{name}_velocity_rel_err"] = float(np.abs(got["u"] - ref["u"]).max() / umax)
            # the other error measures: L2 (relative to the FP64 field's
            # norm) of u and f, max-relative of f, max of rho - rho64
            extras[f"{name}_velocity_l2_rel_err"] = float(np.linalg.norm(got["u"] - ref["u"]) / np.linalg.norm(ref["u"]))
            extras[f"{name}_f_max_rel_err"] = float(np.abs(got["f"] - ref["f"]).max() / np.abs(ref["f"]).max())
            extras[f"{name}_f_l2_rel_err"] = float(np.linalg.norm(got["f"] - ref["f"]) / np.linalg.norm(ref["f"]))
            extras[f"{name}_rho_max_abs_err"] = float(np.abs(got["rho"] - ref["rho"]).max())
            del got
        extras["error_after_steps"] = done
        del c64, c16, ref
        # ---- rigid cylinder channel (1000 x 400, CM, IBM) and flexible
        # filament channel (1200 x 400, BGK, FEM), FP64 and FP32
        for prec, tag in ((PREC_F64, "fp64"), (PREC_F32, "fp32")):
            p, b = cylinder_params(prec)
            cc = Case(p, b)
            cc.step(args.warmup)
            tt, _, _ = cc.bench_steps(200)
            extras[f"cylinder_1000x400_cm_{tag}_mlups"] = round(1000 * 400 * 200 / (tt * 1e-3) / 1e6, 1)
            del cc
            p, b = filament_params(prec)
            cf = Case(p, b)
            cf.step(args.warmup)
            tt, _, _ = cf.bench_steps(50)
            st = cf.status()
            extras[f"filament_1200x400_bgk_{tag}_mlups"] = round(1200 * 400 * 50 / (tt * 1e-3) / 1e6, 1)
            extras[f"filament_1200x400_bgk_{tag}_ms_per_step"] = round(tt / 50, 3)
            extras["filament_subiterations_last_step"] = st.last_subits
            del cf
        # ---- FP32 vs FP64 on the immersed-body workloads: drag, lift,
        # shedding period, filament tip displacement
        extras["accuracy"] = accuracy_leg()
        # ---- 64-case batched ensemble
        # (FP32 over the configured 10,000 steps; FP16 storage over 100, since
        # it does not carry long FSI runs)
        extras["ensemble"] = ensemble_leg(10000, args.warmup, fp16_steps=100, seq_steps=20, long_error=True)
        # ---- serving: Poisson stream of canopy requests
        extras["serving"] = serving_leg()

    # ---- end to end through the C-ABI: create from params (host), K steps,
    # read the velocity field back into host memory. The host buffer is
    # page-locked and exists before the timed region, as the output arrays of
    # a host program do; allocating 268 MB of fresh pages inside the region
    # would time the operating system's page faults.
    u = _pinned_array((sites, 2))
    t0 = time.perf_counter()
    ce = Case(cavity_params(n, form[0]))
    ce.step(args.steps)
    ce.fields(("u",), out={"u": u})
    e2e_s = time.perf_counter() - t0
    e2e = world * sites * args.steps / e2e_s / 1e6
    h2d = 376 + 16 * n + 32 * (args.steps + 2)  # params struct, inlet profile, step scalars
    d2h = u.nbytes
    del ce, u

    traffic = None
    tpath = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if os.path.exists(tpath) and args.storage == "fp32":
        with open(tpath) as fh:
            tr = json.load(fh)
        traffic = round(float(tr["dram_bytes_per_site"]) * sites)

    cpu = None
    if rank == 0 and world == 1 and not args.quick:
        cp = cavity_params(n, PREC_F64)
        m1, d1 = cpu_oracle_mlups(cp, 1, 1)
        k = max(2, min(400, int(10.0 / max(d1, 1e-3))))  # about 10 s of CPU work
        mlups, dt = cpu_oracle_mlups(cp, k, 1)
        cpu = {"value": round(mlups, 3), "unit": "MLUPS", "cores": os.cpu_count(), "kind": "port",
               "sample": f"{k} full steps of the {n}x{n} FP64 lattice after 1 warm-up ({dt:.1f} s)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 1), "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": form[2],
            "data": "synthetic (analytic initial state of the cavity)",
            "config": {"workload": f"lid_driven_cavity_{n}x{n}_d2q9_bgk", "lattice": [n, n], "collision": "BGK",
                       "storage": form[3], "lid_velocity": 0.1, "tau": 0.5768,
                       "parallelism": f"replicas{world}", "l2": f"state {2 * 9 * form[1] * sites / 1e9:.2f} GB > L2 (no flush needed)"},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                         "frac": round(achieved / hbm, 4), "traffic": traffic,
                         "peak_source": f"{hbm_kind} hbm_gbs",
                         "kernel": ("k_interior_f64<BGK> + k_perimeter" if args.storage == "fp64" else
                                    f"k_step_tma<BGK,{form[2].upper()}> (boundary perimeter + TMA-staged interior tiles, one launch per step)"),
                         "algorithmic_bytes_per_site": bytes_per_site, "kernel_ms": round(inner_ms, 4)},
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e, 1), "unit": "MLUPS", "h2d_bytes_per_step": round(h2d / args.steps),
                    "d2h_bytes_per_step": round(d2h / args.steps),
                    "what": "create from params + K steps + velocity field to host, wall clock"},
            "gpu_launches": launches,
            "fp64": fp64,
            "clocks": clocks,
            "extras": extras,
        }
        if "fp64_mlups" in extras:
            line["fp32_vs_fp64"] = {"fp32_over_fp64_mlups": extras["fp32_over_fp64"],
                                    "fp32_velocity_rel_err": extras["fp32_velocity_rel_err"],
                                    "fp32_velocity_l2_rel_err": extras["fp32_velocity_l2_rel_err"],
                                    "fp32_f_max_rel_err": extras["fp32_f_max_rel_err"],
                                    "fp16_velocity_rel_err": extras["fp16_velocity_rel_err"]}
            ac = extras.get("accuracy", {})
            for key in ("cylinder_cd_rel_err", "cylinder_cl_amp_rel_err", "cylinder_period_rel_err",
                        "filament_tip_max_err_over_L"):
                if key in ac:
                    line["fp32_vs_fp64"][key] = ac[key]
        if "serving" in extras:
            sv = extras["serving"]
            line["latency"] = {"p50_s": sv["latency_s_p50"], "p95_s": sv["latency_s_p95"],
                               "p99_s": sv["latency_s_p99"],
                               "workload": f"Poisson stream of {sv['requests']} canopy solves at "
                                           f"{sv['load']:.0%} of measured capacity"}
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nx", type=int, default=4096)
    ap.add_argument("--quick", action="store_true", help="headline measurement only")
    ap.add_argument("--storage", default="fp32", choices=["fp32", "fp16", "fp64"],
                    help="population storage of the headline case (other than fp32 only with --quick)")
    ap.add_argument("--requests", type=int, default=24, help="serve: requests in the stream")
    ap.add_argument("--cases", type=int, default=64, help="ensemble: cases in the batch")
    ap.add_argument("--tile", default="", help="ensemble: fixed tile WxH instead of the autotuner")
    ap.add_argument("--batch-only", action="store_true", help="ensemble: skip the sequential per-case runs")
    ap.add_argument("--step-scale", type=float, default=0.25, help="serve: fraction of each request's steps")
    ap.add_argument("--workload", default="cavity", choices=["cavity", "cylinder", "filament", "ensemble", "serve", "accuracy", "spread"],
                    help="cavity: the headline line; cylinder/filament: timing of one IBM case; "
                         "ensemble: the 64-case batch against sequential per-case runs; "
                         "serve: the Poisson request stream; accuracy: FP32 vs FP64 cylinder "
                         "Cd/Cl/shedding period over --steps steps and filament tip displacement")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup()
    try:
        if args.impl == "reference":
            return run_reference(args, world, rank)
        if args.workload != "cavity":
            return run_workload(args, world, rank)
        return run_gb300(args, world, rank, local)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
