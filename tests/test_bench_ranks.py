"""The N > 1 host logic of bench.py on CPU: two gloo ranks (world size 2)
aggregate their device times (max) and pixels (sum) into the whole-job
throughput, as the NCCL ranks of a multi-GPU run do.  The path is replicas
only (every request is independent), so this reduction is the only
cross-rank step."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=2)
    ms, px = (10.0, 100.0) if rank == 0 else (20.0, 300.0)
    q.put((rank, bench.job_throughput(ms, px, dist, "cpu")))
    dist.barrier()
    dist.destroy_process_group()


def test_job_throughput_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        value, ms, px = out[r]
        assert ms == 20.0 and px == 400.0
        assert value == pytest.approx(400.0 / 0.020 / 1e6)


def test_job_throughput_one_process():
    sys.path.insert(0, ROOT)
    import bench
    value, ms, px = bench.job_throughput(8.0, 4e6)
    assert (ms, px) == (8.0, 4e6) and value == pytest.approx(500.0)
