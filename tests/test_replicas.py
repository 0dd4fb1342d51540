"""Multi-GPU form of bench.py: independent replicas, one per rank, with no collective on the data
path; the job time is the slowest replica's (max over ranks) and the throughput is the whole
job's.  The rank logic runs here on CPU with two gloo ranks."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = [40.0, 55.0][rank]
    ms = bench.max_over_ranks(local_ms, dist, "cpu")
    value = bench.job_throughput(world, 512 * 512 * 513, 2 * 10, ms * 1e-3)
    out.put((rank, ms, value))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_max_time_and_job_throughput():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [55.0, 55.0]
    expect = 2 * 512 * 512 * 513 * 20 / 0.055 / 1e6
    assert all(r[2] == pytest.approx(expect) for r in res)


def test_reference_arm_only_rank0_prints(capsys, monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")

    class A:
        steps, warmup, gpus = 2, 1, 2
    bench.run_reference(A())
    assert capsys.readouterr().out == ""
