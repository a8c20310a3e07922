"""bench.py under several ranks, on the CPU with the gloo backend (world size 2): replicas take
disjoint history ranges, the job's time is the slowest rank's, and the reference arm runs
and prints on rank 0 alone."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        total = 1.0 + rank  # rank 1 is the slower one
        value, slowest = bench.job_rate(dist, world, 3, 1000, total, device="cpu")
        out.put((rank, value, slowest, [bench.replica_first(rank, i, 1000) for i in range(3)]))
    finally:
        dist.destroy_process_group()


def test_job_rate_is_the_slowest_rank_and_ranges_are_disjoint():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, slowest, firsts in got:
        assert slowest == 2.0
        assert value == pytest.approx(2 * 3 * 1000 / 2.0)
    ranges = [set(range(f, f + 1000)) for _, _, _, firsts in got for f in firsts]
    assert sum(len(r) for r in ranges) == len(set().union(*ranges))  # no history id twice


def test_job_rate_single_rank():
    value, slowest = bench.job_rate(None, 1, 5, 2000, 4.0)
    assert (value, slowest) == (2500.0, 4.0)


def test_reference_arm_prints_once_under_two_ranks():
    """torchrun with two ranks (gloo here): rank 0 times the CPU restatement and prints one
    JSON line; rank 1 exits 0 without work."""
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-sample", "500"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
