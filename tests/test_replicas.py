"""Multi-GPU path of bench.py on CPU: pairs are independent, so N GPUs run
N replicas (one pair each, seed 2000 + rank) with no collective on the data
path; the time is the slowest rank's and the rate sums the replicas.  The
reduction runs here over two gloo ranks."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as tdist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = [250.0, 310.5][rank]
        ms = bench.max_over_ranks(local_ms, True, "cpu")
        sc = bench.scene_for(rank)
        out.put((rank, ms, bench.replica_rate(world, 1242, 375, 8, ms * 1e-3), float(sc.left[10, 10, 0])))
    finally:
        tdist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
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
    (r0, ms0, v0, px0), (r1, ms1, v1, px1) = res
    assert ms0 == ms1 == 310.5                      # max over ranks
    assert v0 == pytest.approx(2 * 1242 * 375 * 8 / 0.3105 / 1e6)
    assert px0 != px1                                # each rank its own pair
