"""The N-rank bench path on CPU (gloo, world size 2): replicas with no data-path collective,
the timing taken as the maximum over ranks, and the reference arm run by rank 0 alone."""

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


def _rank_main(rank, world, port, values, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    out[rank] = bench.max_over_ranks(values[rank], dist)
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_world2():
    import torch.multiprocessing as mp
    port = _free_port()
    manager = mp.Manager()
    out = manager.dict()
    values = [3.5, 7.25]
    mp.spawn(_rank_main, args=(2, port, values, out), nprocs=2, join=True)
    assert out[0] == out[1] == 7.25


def test_reference_arm_under_torchrun_world2():
    """--impl reference launched on two ranks: rank 0 alone times the CPU reference and
    prints one JSON line; the other rank exits 0 without work."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--grid", "16", "--steps", "1", "--warmup", "1"]
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert p.returncode == 0, p.stdout + p.stderr
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 2
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
