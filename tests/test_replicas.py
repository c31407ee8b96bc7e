"""Multi-process path of bench.py on the CPU: two gloo ranks, each solving an
independent replica (the GB300 design shards independent problems, with no
data-path collective), joined by the barrier and the max-over-ranks
reduction bench.py uses.  Each rank's solve is checked against the same
solve run alone."""
import os
import pathlib
import socket
import sys

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _replica(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "saras-cc_gb300"))
    sys.path.insert(0, str(ROOT / "oracle"))
    sys.path.insert(0, str(ROOT / "tests"))
    import torch.distributed as dist
    import bench
    import pyoracle as O
    import saras_gb300 as S
    from helpers import random_rhs

    dist.init_process_group("gloo", rank=rank, world_size=world)
    g = S.grid_desc(n=(16, 16, 16), mesh="UUD", beta=(1, 1, 1.2), domain="NNN")
    rhs = random_rhs(g, 100 + rank)
    lhs = S.padded_field(g)
    r = O.mg_solve(g, S.mg_params(vc_count=5, vc_tolerance=1e-30, pre_smooth=2, post_smooth=2), lhs, rhs)
    dist.barrier()
    t = bench.max_over_ranks(float(rank + 1), dist, "cpu")
    out[rank] = (t, r.history.tolist(), float(lhs.sum()))
    dist.destroy_process_group()


def test_two_gloo_replicas():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    sys.path.insert(0, str(ROOT / "tests"))
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle as O
    import saras_gb300 as S
    from helpers import random_rhs

    port = _free_port()
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    procs = [ctx.Process(target=_replica, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for rank in range(2):
        t, hist, tot = out[rank]
        assert t == 2.0  # max over ranks of (rank + 1)
        g = S.grid_desc(n=(16, 16, 16), mesh="UUD", beta=(1, 1, 1.2), domain="NNN")
        lhs = S.padded_field(g)
        r = O.mg_solve(g, S.mg_params(vc_count=5, vc_tolerance=1e-30, pre_smooth=2, post_smooth=2), lhs,
                       random_rhs(g, 100 + rank))
        assert np.array_equal(np.array(hist), r.history) and tot == float(lhs.sum())
