"""The bench's multi-rank host logic on CPU with two gloo ranks: replicas get
distinct fields, the timing is the maximum over ranks, the barrier passes.
(The interpolation has no data-path collective: every rank runs its own
batch.)"""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    w, r, local = bench.dist_setup()
    dist.init_process_group("gloo", rank=r, world_size=w)
    bench.barrier(w)
    t = bench.max_over_ranks(w, 10.0 + r)
    pts, val = bench.field_inputs(bench.field_seed(r, 0))
    q.put((r, t, float(val[:5].sum())))
    bench.barrier(w)
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=100) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert [o[1] for o in out] == [11.0, 11.0]          # max over ranks
    assert out[0][2] != out[1][2]                      # distinct replica data
    assert not np.isnan(out[0][2])
