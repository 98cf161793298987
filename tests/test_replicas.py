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


def test_clock_samples_outside_the_timed_region_are_dropped():
    # bench.Clocks keeps only the nvidia-smi samples stamped inside the timed
    # region, and reports a slowdown reason seen in any of them
    import datetime
    import sys
    import time
    sys.path.insert(0, ROOT)
    import bench

    def stamp(t):
        return datetime.datetime.fromtimestamp(t).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]

    now = time.time()
    c = bench.Clocks(0)
    c.lines = [
        f"{stamp(now - 2)}, 1100, 2070, 300.0, Not Active, Not Active, Not Active, Not Active",
        f"{stamp(now + 0.05)}, 2070, 2070, 900.0, Not Active, Not Active, Not Active, Active",
        f"{stamp(now + 0.10)}, 2040, 2070, 950.0, Not Active, Not Active, Not Active, Not Active",
        f"{stamp(now + 0.15)}, [N/A], 2070, 950.0, Not Active, Not Active, Not Active, Not Active",
        f"{stamp(now + 9)}, 900, 2070, 200.0, Active, Not Active, Not Active, Not Active",
    ]
    c.t0, c.t1 = now, now + 1.0
    s = c.summary()
    assert s["samples"] == 2
    assert s["sm_mhz"] == 2055.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
    c.t0, c.t1 = now + 5, now + 6  # nothing inside: no summary
    assert c.summary() is None
