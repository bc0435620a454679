"""Multi-GPU is replicas only (each rank runs its own copy of the scene, no
data-path collective): the bench's only exchange is the max-over-ranks of
the timed region, and the job's throughput counts every rank's steps over
the slowest rank's time.  Checked with world_size 2 on the gloo backend
(CPU), and the reference arm's non-zero ranks exit without output."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
ROOT = Path(__file__).resolve().parent.parent


def _rank(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, str(ROOT))
    import bench

    seconds = 1.0 + rank  # rank 1 is the slow one
    t = bench.max_over_ranks(seconds, world)
    out.put((rank, t, bench.job_throughput(10, world, t)))
    dist.destroy_process_group()


def test_max_over_ranks_and_job_throughput_two_ranks():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 2000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert [r[1] for r in res] == [2.0, 2.0]          # both see the slowest rank's time
    assert [r[2] for r in res] == [10.0, 10.0]        # 2 ranks x 10 steps / 2 s


def test_reference_arm_other_ranks_print_nothing():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    res = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1"],
                         capture_output=True, text=True, env=env, timeout=300)
    assert res.returncode == 0
    assert res.stdout.strip() == ""
