"""The N > 1 path of bench.py on CPU: replicas with no data-path collective,
the job's time is the slowest rank's (max over ranks, gloo, world size 2),
and the reference arm runs on rank 0 only."""
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


def _rank_main(rank, ws, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=ws)
    try:
        # rank r took (r + 1) seconds per step for 10 particles x 3 elements
        value, t = bench.job_value(float(rank + 1), ws, 10, 3)
        q.put((rank, value, t))
    finally:
        dist.destroy_process_group()


def test_job_value_is_all_ranks_over_the_slowest():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, value, t in got:
        assert t == 2.0                      # the slower rank's time on every rank
        assert value == 2 * 10 * 3 / 2.0     # both replicas' steps over that time


def test_job_value_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_value(0.5, 1, 4, 5) == (40.0, 0.5)


@pytest.mark.timeout(600)
def test_reference_arm_prints_once_under_torchrun():
    """bench.py --impl reference launched like the driver launches it at
    N = 2: rank 0 times the CPU reference and prints one JSON line, the other
    rank exits 0 without work."""
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1",
           "--particles", "2048", "--gaps", "4"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["value"] > 0 and d["e2e"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] == "port"
