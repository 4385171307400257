"""Build the GB300 CUDA library ``life_gb300/_lib/liblife_gb300.so`` in-tree.

Every translation unit is compiled for sm_103a only, in parallel, and linked
into one shared library that exports the C-ABI of ``include/life_gb300.h``.

* Every CUDA unit is compiled with ``--fmad=false`` (no a*b+c contraction, as
  g++ on x86-64 does), so the FP64 code shared by all storage forms rounds
  identically everywhere; the reduced-precision kernels spell out the fused
  multiply-adds they want with ``fmaf``.
* Host C++ is compiled with ``-ffp-contract=off`` so start-up arithmetic is
  identical on x86-64 and aarch64 hosts.

``python -m life_gb300.build`` rebuilds when a source or flag changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from typing import List, Tuple

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "liblife_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


# (source, extra flags)
UNITS: List[Tuple[str, List[str]]] = [
    ("lbm_f64.cu", ["--fmad=false"]),
    ("ibm_f64.cu", ["--fmad=false"]),
    ("fem_f64.cu", ["--fmad=false"]),
    ("lbm_lowp.cu", ["--fmad=false"]),
    ("life_case.cu", ["--fmad=false"]),
    ("ibm_host.cu", ["--fmad=false"]),
    ("fem_host.cu", ["--fmad=false"]),
    ("ibm_noalloc.cu", ["--fmad=false"]),
    ("batch.cu", ["--fmad=false"]),
    ("server.cu", ["--fmad=false"]),
    ("observe.cu", ["--fmad=false"]),
    ("measure.cu", ["--fmad=false"]),
    ("objects.cpp", []),
]


def _cmd(src: str, extra: List[str], obj: str) -> List[str]:
    path = os.path.join(CSRC, src)
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-lineinfo",
              "-I", CSRC, "-I", os.path.join(os.path.dirname(HERE), "include")]
    if src.endswith(".cpp"):
        return [nvcc(), "-x", "c++", *common, "-c", path, "-o", obj]
    return [nvcc(), *ARCH, *common, *extra, "-c", path, "-o", obj]


def _digest(units) -> str:
    h = hashlib.sha256()
    for src, extra in units:
        h.update(src.encode())
        h.update(" ".join(extra).encode())
    for name in sorted(os.listdir(CSRC)):
        with open(os.path.join(CSRC, name), "rb") as fh:
            h.update(name.encode())
            h.update(fh.read())
    with open(os.path.join(os.path.dirname(HERE), "include", "life_gb300.h"), "rb") as fh:
        h.update(fh.read())
    h.update(" ".join(ARCH).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> str:
    units = [(s, e) for s, e in UNITS if os.path.exists(os.path.join(CSRC, s))]
    os.makedirs(OUT, exist_ok=True)
    stamp = os.path.join(OUT, "build.sha256")
    dig = _digest(units)
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == dig:
        return LIB
    objs = []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        futs = {}
        for src, extra in units:
            obj = os.path.join(OUT, src.replace(".", "_") + ".o")
            objs.append(obj)
            cmd = _cmd(src, extra, obj)
            if verbose:
                print(" ".join(cmd), flush=True)
            futs[ex.submit(subprocess.run, cmd, capture_output=True, text=True)] = src
        errors = []
        for fut in cf.as_completed(futs):
            res = fut.result()
            if res.returncode != 0:
                errors.append(f"--- {futs[fut]} ---\n{res.stderr}")
            elif verbose and res.stderr.strip():
                print(res.stderr, flush=True)
        if errors:
            raise RuntimeError("CUDA library build failed:\n" + "\n".join(errors))
    tmp = LIB + ".tmp"
    link = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    res = subprocess.run(link, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n" + res.stderr)
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(dig)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
