"""The multi-GPU form is one replica per rank (independent jobs, weak
scaling, no data-path collective): bench.py times every rank, takes the max
over ranks and reports the visibilities of all ranks over that time.  This
checks that host-side logic with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as td  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world))
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    td.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seconds = [1.5, 2.5][rank]           # rank 1 is the slower replica
        t = bench.max_over_ranks(seconds, td)
        rate = bench.replica_rate(1_000_000, world, t)
        q.put((rank, t, rate))
    finally:
        td.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate_with_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    for rank, t, rate in out:
        assert t == 2.5                      # every rank sees the slowest time
        assert rate == pytest.approx(2 * 1_000_000 / 2.5 / 1e6)


def test_single_process_is_unchanged():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench.max_over_ranks(3.0, None) == 3.0
    assert bench.replica_rate(2_000_000, 1, 0.5) == pytest.approx(4.0)
