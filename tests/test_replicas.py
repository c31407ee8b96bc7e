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


def _gpu_replica(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "saras-cc_gb300"))
    sys.path.insert(0, str(ROOT / "tests"))
    import torch
    import torch.distributed as dist
    import bench
    import saras_gb300 as S
    from helpers import random_rhs

    dist.init_process_group("gloo", rank=rank, world_size=world)
    torch.cuda.set_device(0)
    g = S.grid_desc(n=(64, 64, 64), mesh="UUD", beta=(1, 1, 1.2), domain="NNN")
    mg = S.Multigrid(g, S.mg_params(precision=S.PREC_MIXED, vc_count=50, vc_tolerance=1e-10, pre_smooth=2,
                                    post_smooth=2, mg_tolerance=1e-6, inner_cycles=-8))
    lhs = S.padded_field(g)
    dist.barrier()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    st = mg.mg_solve(lhs, random_rhs(g, 200 + rank))
    t1.record()
    torch.cuda.synchronize()
    dist.barrier()
    ms = bench.max_over_ranks(t0.elapsed_time(t1), dist, "cpu")
    out[rank] = (st, ms, lhs.tobytes(), mg.history.tolist())
    mg.close()
    dist.destroy_process_group()


@pytest.mark.gpu
def test_two_gloo_replicas_through_the_cuda_library():
    """The same two-rank path with each replica's solve on the GPU through
    the CUDA library (both ranks on device 0; the replicas never wait on each
    other's kernels, only on the host-side gloo barrier): the max-over-ranks
    time is the larger of the two, and each rank's solution and residual
    history are bit for bit those of the same solve in this process."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    sys.path.insert(0, str(ROOT / "tests"))
    import saras_gb300 as S
    from helpers import random_rhs

    port = _free_port()
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    procs = [ctx.Process(target=_gpu_replica, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(300)
        assert p.exitcode == 0
    assert out[0][1] == out[1][1] > 0.0
    g = S.grid_desc(n=(64, 64, 64), mesh="UUD", beta=(1, 1, 1.2), domain="NNN")
    for rank in range(2):
        st, _, sol, hist = out[rank]
        assert st == S.OK
        mg = S.Multigrid(g, S.mg_params(precision=S.PREC_MIXED, vc_count=50, vc_tolerance=1e-10, pre_smooth=2,
                                        post_smooth=2, mg_tolerance=1e-6, inner_cycles=-8))
        lhs = S.padded_field(g)
        mg.mg_solve(lhs, random_rhs(g, 200 + rank))
        assert lhs.tobytes() == sol and mg.history.tolist() == hist
        mg.close()
