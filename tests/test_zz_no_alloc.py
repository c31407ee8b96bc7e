"""saras_mg_solve_static, the multigrid solve that allocates no device
memory (its scratch is a file-scope __device__ array), called through the C
ABI and compared with the handle-based entry point saras_mg_solve_dev on the
same inputs, for two calls in a row.  Tolerance: 1e-12 relative in the
solution and the residual history (the two run the same kernels in the same
order, so they normally agree bit for bit).  The second call must leave the
device's free memory unchanged: the entry point allocates nothing."""
import ctypes as C

import numpy as np
import pytest

import saras_gb300 as S
from helpers import random_rhs

pytestmark = pytest.mark.gpu

RTOL = 1e-12
CASES = [
    ("fp64_3d", dict(n=(32, 32, 32), mesh="UUD", beta=(1, 1, 1.2), domain="NNN"), S.PREC_FP64),
    ("mixed_2d", dict(n=(64, 1, 64), mesh="UUD", beta=(1, 1, 1.1), domain="NNN", dims=2), S.PREC_MIXED),
    # 3-D MIXED: the paired red-black iterations (second e buffer), the
    # single-block bottom and adaptive inner counts, all in the scratch
    ("mixed_3d", dict(n=(64, 64, 64), mesh="UUD", beta=(1, 1, 1.2), domain="NNN"), S.PREC_MIXED),
    ("fp64_dirichlet", dict(n=(16, 16, 32), mesh="UUD", beta=(1, 1, 1.3), domain="PPN"), S.PREC_FP64),
]


def _entry():
    lib = S.load()
    f = lib.saras_mg_solve_static
    f.argtypes = [C.POINTER(S.GridDesc), C.POINTER(S.MgParams), C.c_void_p, C.c_void_p, C.c_void_p,
                  C.POINTER(C.c_int64), C.POINTER(C.c_double), C.c_int32, C.POINTER(C.c_int32)]
    f.restype = C.c_int
    return lib, f


def _params(precision, gk):
    bc = [0, 0, 0, 0, 1, 1] if gk.get("domain") == "PPN" else [0] * 6
    return S.mg_params(precision=precision, vc_count=80, vc_tolerance=1e-10, mg_tolerance=1e-6, pre_smooth=2,
                       post_smooth=2, bc_kind=bc, inner_cycles=-8 if precision == S.PREC_MIXED else 1)


@pytest.mark.parametrize("name,gk,prec", CASES, ids=[c[0] for c in CASES])
def test_static_scratch_solve_matches_handle_solve(name, gk, prec):
    import torch
    g = S.grid_desc(**gk)
    prm = _params(prec, gk)
    rhs = random_rhs(g, 5, compatible=gk.get("domain") != "PPN")
    dev = torch.device("cuda", 0)
    rhs_d = torch.from_numpy(rhs).to(dev)
    st = [s // 8 for s in rhs.strides]
    off = 8 * (st[0] + st[1] + st[2])
    ref_d = torch.zeros_like(rhs_d)
    mg = S.Multigrid(g, prm)
    mg.mg_solve_dev(ref_d.data_ptr() + off, rhs_d.data_ptr() + off, st)
    torch.cuda.synchronize()
    ref, ref_hist = ref_d.cpu().numpy(), mg.history.copy()
    mg.close()
    lib, f = _entry()
    for call in range(2):
        out_d = torch.zeros_like(rhs_d)
        hist = np.zeros(512)
        n = C.c_int32()
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        s = f(C.byref(g), C.byref(prm), None, C.c_void_p(out_d.data_ptr() + off),
              C.c_void_p(rhs_d.data_ptr() + off), (C.c_int64 * 3)(*st),
              hist.ctypes.data_as(C.POINTER(C.c_double)), 512, C.byref(n))
        assert s == S.OK, lib.saras_last_error()
        torch.cuda.synchronize()
        if call == 1:  # the first call may load kernels; the second allocates nothing
            assert torch.cuda.mem_get_info()[0] == free_before
        out = out_d.cpu().numpy()
        assert n.value == len(ref_hist) and ref_hist[-1] < 1e-10
        assert np.abs(hist[:n.value] - ref_hist).max() <= RTOL * np.abs(ref_hist).max()
        assert np.abs(out - ref).max() <= RTOL * np.abs(ref).max()


def test_static_scratch_rejects_a_grid_that_does_not_fit():
    import torch
    g = S.grid_desc(n=(128, 128, 128), mesh="UUU", domain="NNN")
    prm = _params(S.PREC_FP64, {})
    lib, f = _entry()
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")  # never touched: the call fails first
    st = (C.c_int64 * 3)(130 * 130, 130, 1)
    n = C.c_int32()
    s = f(C.byref(g), C.byref(prm), None, C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()), st, None, 0,
          C.byref(n))
    assert s == S.BUDGET
    msg = lib.saras_last_error().decode()
    assert "static scratch holds 33554432 bytes" in msg
