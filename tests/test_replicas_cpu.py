"""The N > 1 path of bench.py on the CPU: one process per GPU runs an
independent replica, and the ranks coordinate only on the host -- a barrier
around the timed region and a max over ranks of its duration, through gloo.
No collective touches the data path.  Two gloo ranks at 127.0.0.1 check the
environment reading, the barrier, the max and the whole-job aggregate."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    try:
        assert bench.dist_env() == (ws, rank, rank)
        dist.init_process_group("gloo")
        bench.barrier(True)
        ms = 100.0 + 10.0 * rank  # rank 1 is the slowest
        ms_max = bench.max_over_ranks(ms, True)
        bench.barrier(True)
        q.put((rank, ms_max, bench.aggregate_rate(1000, 20, ws, ms_max)))
        dist.destroy_process_group()
    except Exception as e:  # report to the parent instead of hanging it
        q.put((rank, "error", repr(e)))


def test_two_replicas_coordinate_on_the_host():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    for rank, ms_max, rate in out:
        assert ms_max == 110.0, (rank, ms_max, rate)
        # 2 replicas x 1000 cells x 20 steps over the slowest rank's 110 ms
        assert rate == pytest.approx(2 * 1000 * 20 / 0.110)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, None) == 3.5
    bench.barrier(None)
    assert bench.aggregate_rate(10, 2, 1, 1.0) == pytest.approx(20000.0)
