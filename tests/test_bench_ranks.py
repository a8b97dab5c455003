"""The multi-rank paths of bench.py, on CPU with gloo at world size 2.  The
path does not shard (replicas only): each rank renders its own frame, and
rank 0 reports the whole job as every rank's rays over the slowest rank's
time.  The reference arm is launched the same way, and rank 0 alone runs it
and prints its line."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def aggregate_worker(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=2)
    ws, r, _ = bench.dist_env()
    q.put((r, bench.aggregate_ranks(10.0 * (rank + 1), 100 * (rank + 1), ws, "cpu")))
    dist.barrier()
    dist.destroy_process_group()


def test_aggregate_ranks_over_gloo():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=aggregate_worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # slowest rank's time, every rank's rays, on both ranks
    assert got == {0: (20.0, 300.0), 1: (20.0, 300.0)}


def test_aggregate_ranks_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.aggregate_ranks(12.5, 77, 1, "cpu") == (12.5, 77)


def test_reference_arm_under_torchrun_prints_once():
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3", "--scene", "box4k",
           "--width", "64", "--height", "32", "--spp", "1", "--cpu-seconds", "0.2"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
