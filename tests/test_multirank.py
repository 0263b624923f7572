"""The N-GPU path on CPU: replicas only (no collective on the data path), so
what N > 1 adds is host logic -- the slowest rank's time (max over ranks) and
rank 0 alone printing the reference arm's line.  Both run here as two `gloo`
processes on 127.0.0.1."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _max_worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    v = bench.max_over_ranks(1.5 + rank, dist, torch, "cpu")
    with open(out + ".%d" % rank, "w") as f:
        f.write(repr(v))
    dist.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp
    out = str(tmp_path / "v")
    mp.start_processes(_max_worker, args=(2, _free_port(), out), nprocs=2,
                       start_method="spawn")
    got = [float(open(out + ".%d" % r).read()) for r in range(2)]
    assert got == [2.5, 2.5]


def test_max_over_ranks_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25, None, None, "cpu") == 3.25


def test_reference_arm_two_ranks():
    # torchrun with two ranks: rank 0 runs the CPU reference arm and prints
    # one line, rank 1 exits 0 without work
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1",
           "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
           "--master-port", str(_free_port()), "bench.py", "--impl",
           "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
           "--ref-moves-per-step", "5", "--small"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"
