"""bench.py on N GPUs runs N independent replicas of the design loop (the
path has no exchange step); the only cross-rank step is the timing
reduction. Here two gloo ranks on the CPU check it: the job time is the
slowest rank's and the throughput counts both ranks' iterations."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch.distributed as td
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    td.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    assert bench.dist() == (world, rank, rank)
    K = 17
    times, values = bench.whole_job([1.0 + rank, 2.0 + 0.5 * rank], K, world, device="cpu")
    out.put((rank, times, values))
    td.barrier()
    td.destroy_process_group()


def test_replica_timing_two_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for rank, times, values in res:
        assert times == [2.0, 2.5]  # the slower rank's times, on both ranks
        assert values == pytest.approx([2 * 17 / 2.0, 2 * 17 / 2.5])


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    times, values = bench.whole_job([0.5, 0.25], 4, 1)
    assert times == [0.5, 0.25] and values == [8.0, 16.0]
