"""The replicas path of bench.py on CPU ranks (gloo, world size 2): the job's
time per step is the slowest rank's and its throughput the work of all ranks
over that time; under torchrun the reference arm runs on rank 0 alone."""
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    dist.barrier()
    ms, value = bench.job_rate(10.0 + 5.0 * rank, 1000 * (rank + 1), dist, "cpu")
    out[rank] = (ms, value)
    dist.barrier()
    dist.destroy_process_group()


def test_job_rate_two_gloo_ranks():
    import torch.multiprocessing as tmp

    # spawn, not fork: other tests may have started threads (the oracle's OpenMP pool) in this process
    mgr = tmp.get_context("spawn").Manager()
    out = mgr.dict()
    tmp.spawn(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True)
    for r in range(2):
        ms, value = out[r]
        assert ms == 15.0  # the slower rank
        assert abs(value - 3000 / 0.015) < 1e-6 * value


def test_job_rate_single_rank():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.job_rate(20.0, 1000) == (20.0, 50000.0)


def test_reference_arm_rank1_does_no_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], env=env, capture_output=True, text=True, timeout=120)
    assert p.returncode == 0 and p.stdout.strip() == ""
