"""The multi-rank bench path on CPU (gloo, world size 2): under
torch.distributed.run every rank joins the process group, the timing
reduction takes the maximum over ranks, and rank 0 alone prints the one JSON
line. The reference arm runs here because it times the CPU oracle."""
import json
import os
import re
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(args, timeout=600):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port())] + args
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="2")
    return subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=timeout, env=env)


def test_reference_arm_two_ranks_prints_one_line():
    res = _torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "2", "--warmup", "3",
                     "--nx", "128"])
    assert res.returncode == 0, res.stderr[-3000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, res.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["steps"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"


RANK_SCRIPT = r"""
import os, sys
sys.path.insert(0, os.environ["ROOT"])
import bench
world, rank, local = bench.dist_setup()
bench.barrier(world)
v = bench.max_over_ranks(world, float(rank + 1) * 10.0)
sys.stdout.write(f"rank {rank} max {v}\n")  # one write: the ranks share the pipe
sys.stdout.flush()
import torch.distributed as dist
dist.destroy_process_group()
"""


def test_max_over_ranks_gloo(tmp_path):
    script = tmp_path / "ranks.py"
    script.write_text(RANK_SCRIPT)
    os.environ["ROOT"] = ROOT
    res = _torchrun([str(script)], timeout=300)
    assert res.returncode == 0, res.stderr[-3000:]
    got = sorted(re.findall(r"rank (\d+) max ([0-9.]+)", res.stdout))
    assert got == [("0", "20.0"), ("1", "20.0")], res.stdout
