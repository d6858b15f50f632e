"""The benchmark's multi-rank plumbing on CPU: two gloo ranks (replicas)
agree on the slowest rank's time and pass the barriers the timed region uses;
the reference arm runs on rank 0 only.  No GPU needed."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    bench.barrier(ws)
    slowest = bench.max_over_ranks(ws, 10.0 + rank)
    bench.barrier(ws)
    out.put((rank, slowest))
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 11.0), (1, 11.0)]


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    args = bench.parse()
    # rank 1 returns before touching the GPU, the oracle or the network
    assert bench.run_reference(args) is None


def test_reference_arm_line_loads_no_product_code(tmp_path):
    """The reference arm on a small workload (in a child process): it prints
    one line with the GPU arm's config keys and the volume digest, and maps
    the oracle but not libtvk.so."""
    import json
    import subprocess
    code = f"""
import sys, json, dataclasses
sys.path.insert(0, {str(ROOT)!r})
import bench
from tuvok_gb300 import workloads as W
small = dataclasses.replace(W.WORKLOADS["plain_small"], name="plain_tiny", dims=(48, 40, 36),
                            width=64, height=48, n_poses=4, brick_core=16)
W.WORKLOADS["plain_tiny"] = small
sys.argv = ["bench.py", "--impl", "reference", "--workload", "plain_tiny", "--steps", "2",
            "--warmup", "1"]
bench.run_reference(bench.parse())
maps = open("/proc/self/maps").read()
print("MAPS", int("libtvk" in maps), int("liboracle" in maps))
"""
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300,
                       cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = r.stdout.strip().splitlines()
    line = json.loads([x for x in lines if x.startswith("{")][-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["config"]["workload"] == "plain_tiny"
    assert len(line["config"]["volume_fnv1a"]) == 16
    import bench  # noqa: F401  (same keys as the GPU arm's config builder)
    from tuvok_gb300 import workloads as W
    import dataclasses
    small = dataclasses.replace(W.WORKLOADS["plain_small"], name="plain_tiny", dims=(48, 40, 36),
                                width=64, height=48, n_poses=4, brick_core=16)
    assert set(line["config"]) == set(bench.workload_config(small, 1, 1.0, "x"))
    assert [x for x in lines if x.startswith("MAPS")][-1] == "MAPS 0 1"
