"""Multi-GPU bench logic on CPU (gloo, world size 2): replicas share no data,
the timing collective returns the slowest rank's time to every rank, the
whole-job rate counts every rank's units, and the reference arm runs on rank 0
only (other ranks exit 0 without work)."""
import os
import subprocess
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(0.5 + rank, torch.device("cpu"))
    out.put((rank, t, bench.whole_job_rate(1.0, world, t)))
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    import random
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + random.randint(0, 2000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [1.5, 1.5]          # both ranks see the slowest time
    assert all(abs(r[2] - 2 / 1.5) < 1e-12 for r in res)


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""
