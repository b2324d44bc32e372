"""The multi-process side of bench.py on CPU (gloo, world size 2): the
slowest-rank timing reduction and the replica throughput the line reports,
and the reference arm under torchrun (rank 0 alone works and prints one
line; the other rank exits 0)."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank)
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out, f"r{rank}"), "w") as f:
        f.write(repr(ms))


def test_max_over_ranks_and_replica_throughput(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    got = [float(open(tmp_path / f"r{r}").read()) for r in range(world)]
    assert got == [15.0, 15.0]
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.5) == 3.5  # one process: no reduction
    # 2 replicas x 100 cells x 10 steps in 1 ms
    assert bench.replica_throughput(100, 10, 2, 1.0) == pytest.approx(2e-3)
    _ = torch


def test_reference_arm_under_torchrun(tmp_path, oracle_lib):
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "2", "--warmup", "1", "--cpu-seconds", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=str(tmp_path), env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
