"""The multi-GPU path of bench.py is replicas only: every rank runs the same
extraction and the ranks share nothing but the timing barrier and a MAX
all-reduce of the step time.  That host logic runs here on two CPU ranks
with the gloo backend (no GPU)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, _ = bench.dist_info()
    dist.barrier()
    ms = bench.max_over_ranks(100.0 + 50.0 * r, w, device="cpu")      # rank 1 is the slow replica
    value = bench.whole_job_value(8, w, ms)
    out.put((r, w, ms, value))
    dist.destroy_process_group()


def test_two_replicas_time_by_the_slowest_rank_and_sum_the_work():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, w, ms, value in res:
        assert w == 2
        assert ms == 150.0                    # every rank sees the slowest step
        assert value == pytest.approx(2 * 8 / 0.150)


def test_one_rank_needs_no_process_group():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench.max_over_ranks(123.0, 1) == 123.0
    assert bench.whole_job_value(8, 1, 250.0) == pytest.approx(32.0)
