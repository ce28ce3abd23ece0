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


def test_partition_beams_balances_and_covers():
    from hpsim_gb300 import lattices as L
    nums = [b.num for b in L.batched_scan(256)]
    for ranks in (1, 2, 3, 4, 8):
        parts = L.partition_beams(nums, ranks)
        assert sorted(i for p in parts for i in p) == list(range(len(nums)))
        loads = [sum(nums[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(nums)  # greedy largest-first bound
    assert L.partition_beams([5, 5, 5, 5], 2) == [[0, 2], [1, 3]]


def _part_rank(rank, ws, port, q):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    from hpsim_gb300 import lattices as L
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=ws)
    try:
        nums = [b.num for b in L.batched_scan(64)]
        mine = L.partition_beams(nums, ws)[rank]
        # every beam counted once over the ranks; particles add up to the batch
        seen = torch.zeros(len(nums), dtype=torch.int64)
        seen[mine] = 1
        dist.all_reduce(seen)
        tot = torch.tensor([sum(nums[i] for i in mine)], dtype=torch.int64)
        dist.all_reduce(tot)
        q.put((rank, seen.tolist(), int(tot.item()), sum(nums)))
    finally:
        dist.destroy_process_group()


def test_batch_partition_across_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_part_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, seen, tot, want in out:
        assert all(s == 1 for s in seen) and tot == want
