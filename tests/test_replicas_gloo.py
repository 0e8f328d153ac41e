"""The multi-GPU form of the benchmark is replicas (independent meshes, no
data exchange): per-rank timing reduced by MAX, whole-job throughput summed.
The host logic runs here as two gloo ranks on the CPU; the reference arm
runs on rank 0 only and the other ranks exit without work."""
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


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.replica_barrier(torch, world)
    t = bench.replica_max(torch, 1.0 + rank, world, "cpu")
    v = bench.replica_value(world, 1000, 10, t)
    out.put((rank, t, v))
    dist.destroy_process_group()


def test_replica_max_and_value_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.0, 2.0]  # the slowest rank's time on every rank
    assert [r[2] for r in res] == [2 * 1000 * 10 / 2.0] * 2


def test_reference_arm_rank0_only():
    """`bench.py --impl reference` under two ranks: rank 0 prints the line,
    rank 1 exits 0 without work."""
    env = dict(os.environ, WORLD_SIZE="2", LOCAL_RANK="1", RANK="1")
    r1 = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--n", "4,4,6", "--steps", "1",
                         "--warmup", "0"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r1.returncode == 0 and r1.stdout.strip() == ""
    env.update(LOCAL_RANK="0", RANK="0")
    r0 = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--n", "4,4,6", "--steps", "1",
                         "--warmup", "0"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r0.returncode == 0, r0.stderr
    line = json.loads(r0.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port"
