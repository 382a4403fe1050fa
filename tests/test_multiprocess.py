"""The replicas-only multi-GPU path, on the CPU: two `gloo` ranks agree on
the job time (the maximum over ranks, which `bench.py` divides the
aggregate work by), and the reference arm under a multi-rank launch runs on
rank 0 alone while the other ranks exit 0 without work."""

import os
import socket
import subprocess
import sys
from pathlib import Path

import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(dist, 1.0 + 0.5 * rank, "cpu")
        dist.barrier()
        q.put((rank, t))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
    assert [p.exitcode for p in procs] == [0, 0]
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 1.5), (1, 1.5)]


def test_max_over_ranks_without_a_group_is_the_value():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(None, 2.25, "cpu") == 2.25


def test_reference_arm_on_a_nonzero_rank_does_no_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1",
               MASTER_ADDR="127.0.0.1", MASTER_PORT=str(_free_port()))
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1",
                          "--warmup", "1"], cwd=ROOT, env=env, capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip() == ""
