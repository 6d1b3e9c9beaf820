"""The N > 1 path of bench.py on the CPU with gloo, world size 2: the helpers
(barrier, max over ranks) and the reference arm under torchrun, where rank 0
alone runs the CPU oracle and prints one JSON line and rank 1 exits 0 without
work (replicas only: the path has no data-path collective)."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _env(port: int) -> dict:
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
    env["PYTHONPATH"] = ROOT + os.pathsep + env.get("PYTHONPATH", "")
    return env


HELPER = r"""
import json, os, sys
sys.path.insert(0, os.environ["PYTHONPATH"].split(os.pathsep)[0])
import bench
dist, rank, world = bench.dist_setup(2)
bench.barrier(dist)
m = bench.reduce_max(dist, 1.5 + rank)
print(json.dumps({"rank": rank, "world": world, "max": m, "backend": dist.get_backend()}), flush=True)
dist.destroy_process_group()
"""


def test_dist_helpers_two_ranks():
    pytest.importorskip("torch.distributed")
    port = _free_port()
    procs = []
    for r in range(2):
        env = _env(port)
        env.update(RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r))
        procs.append(subprocess.Popen([sys.executable, "-c", HELPER], env=env, cwd=ROOT,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e[-2000:]
    lines = [json.loads(o.strip().splitlines()[-1]) for o, _ in outs]
    assert sorted(l["rank"] for l in lines) == [0, 1]
    assert all(l["world"] == 2 and l["max"] == 2.5 and l["backend"] == "gloo" for l in lines)


def test_reference_arm_under_torchrun_two_ranks():
    pytest.importorskip("torch.distributed.run")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1"]
    r = subprocess.run(cmd, env=_env(port), cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
