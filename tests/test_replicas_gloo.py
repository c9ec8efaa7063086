"""The multi-rank path of bench.py on CPU: N ranks run independent replicas
(the sampling path does not shard), joined only by a gloo barrier and a
max-reduce of the timed region.  Two ranks over gloo check the reduction,
the barrier and that each rank's replica is seeded differently."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, REPO)
    import bench
    r, local, w = bench.dist_env()
    d = bench.dist_init(w)
    try:
        # each rank's "timed region" differs; every rank must see the maximum
        mx = bench.reduce_max(d, 10.0 * (rank + 1))
        bench.barrier(d)
        wl = bench.workload(r)
        out.put((r, local, w, mx, float(wl.coords.ravel()[0])))
    except Exception as e:                     # reported to the parent at once
        out.put((rank, -1, -1, -1.0, repr(e)))
    finally:
        d.destroy_process_group()


def test_two_ranks_reduce_the_slowest_time_and_seed_independently():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1]
    assert all(r[2] == 2 for r in res)
    assert all(r[3] == 20.0 for r in res)          # max over ranks
    assert res[0][4] != res[1][4]                  # independently seeded replicas


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, REPO)
    import bench
    assert bench.dist_init(1) is None
    assert bench.reduce_max(None, 3.5) == 3.5
    bench.barrier(None)
