"""The multi-GPU path of bench.py on the CPU: N ranks run independent replicas
of the solve (the path needs no exchange), the timed region is the slowest
rank's (max over ranks through a gloo all-reduce), and the reported value is
the whole job's edge-sweeps over that time.  Two gloo ranks on 127.0.0.1."""
import multiprocessing as mp
import os
import socket

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(10.0 + 5.0 * rank, world)
    v = bench.whole_job_gteps(world, 1_000_000, 20, t)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, t, v))


def test_two_replicas_report_the_slowest_rank_and_the_whole_job():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [t for _, t, _ in out] == [15.0, 15.0]
    want = 2 * 1_000_000 * 20 / 0.015 / 1e9
    assert all(abs(v - want) < 1e-9 for _, _, v in out)


def test_one_rank_needs_no_process_group():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, 1) == 12.5
    assert bench.whole_job_gteps(1, 10, 3, 1000.0) == 10 * 3 / 1.0 / 1e9
