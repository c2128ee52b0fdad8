"""The multi-GPU path is N independent replicas (no data-path collective);
its host side -- rank discovery, max-over-ranks timing, one pack per rank --
runs here as two gloo processes on the CPU."""

import os
import socket

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys

    sys.path.insert(0, REPO)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, local = bench.dist_setup(None)
    slowest = bench.max_over_ranks(10.0 * (rank + 1), dist, "cpu")
    pack = bench.make_pack(1234 + r)
    dist.barrier()
    dist.destroy_process_group()
    q.put((r, w, local, slowest, float(pack[:, 3].sum())))


def test_two_replicas_over_gloo():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert [o[2] for o in out] == [0, 1]
    assert all(o[3] == 20.0 for o in out)  # every rank reports the slowest time
    assert out[0][4] != out[1][4]  # each replica drains its own pack


def test_single_process_needs_no_group():
    import sys

    sys.path.insert(0, REPO)
    import bench

    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert np.array_equal(bench.make_pack(7), bench.make_pack(7))
