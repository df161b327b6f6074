"""The multi-process host logic of bench.py on CPU (gloo, world size 2): the
rendezvous, the barrier and the max-over-ranks timing that the replicas
scaling uses.  The data path has no collective (independent replicas), so
this is all the N > 1 path needs; no GPU is involved."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    import bench
    import torch.distributed as dist
    r, w = bench.dist_setup("gloo")
    bench.barrier(w)
    t = bench.max_over_ranks(1.5 + rank, w)            # per-rank "timings"
    units = bench.max_over_ranks(float(10 * (rank + 1)), w)
    q.put((r, w, t, units))
    dist.destroy_process_group()


def test_gloo_two_ranks_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 for o in out)
    assert all(o[2] == pytest.approx(2.5) for o in out)     # every rank sees the slowest rank's time
    assert all(o[3] == pytest.approx(20.0) for o in out)


def test_single_process_needs_no_process_group():
    import bench
    os.environ.pop("WORLD_SIZE", None)
    r, w = bench.dist_setup("gloo")
    assert (r, w) == (0, 1)
    assert bench.max_over_ranks(3.25, w) == 3.25
    bench.barrier(w)
