"""ctypes binding of oracle/liboracle.so -- TEST INFRASTRUCTURE ONLY.

The oracle is the CPU restatement of SARAS-CC's hot path (oracle/saras_oracle.cpp).
It is loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
to check and time the reference algorithm; the product never imports it.
The ABI structs are the ones declared in include/saras_gb300.h (shared with
the product binding, which defines them for ctypes).
"""
from __future__ import annotations

import ctypes as C
import pathlib
import subprocess
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
sys.path.insert(0, str(HERE.parent / "saras-cc_gb300"))
import saras_gb300 as abi  # noqa: E402  (ctypes struct layouts only)

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        build()
    lib = C.CDLL(str(LIB_PATH))
    vp, i32, i64, dp = C.c_void_p, C.c_int, C.c_int64, C.POINTER(C.c_double)
    lib.oracle_set_threads.argtypes = [i32]
    lib.oracle_max_threads.restype = i32
    lib.oracle_num_levels.argtypes = [C.POINTER(abi.GridDesc), i32]
    lib.oracle_num_levels.restype = i32
    lib.oracle_grid_metrics.argtypes = [C.POINTER(abi.GridDesc), i32, i32, i32, dp, dp, dp,
                                        C.POINTER(i32)]
    lib.oracle_field_metrics.argtypes = [C.POINTER(abi.GridDesc), i32, dp, dp, dp, dp]
    lib.oracle_mg_solve.argtypes = [C.POINTER(abi.GridDesc), C.POINTER(abi.MgParams), vp, vp,
                                    C.POINTER(i64), dp, i32, C.POINTER(i32), C.POINTER(i32), dp]
    lib.oracle_rk3_run.argtypes = [C.POINTER(abi.GridDesc), C.POINTER(abi.Rk3Params), vp, vp, vp, vp,
                                   vp, vp, C.POINTER(i64), i32, C.POINTER(i32), C.POINTER(i32), dp]
    lib.oracle_field_op.argtypes = [C.POINTER(abi.GridDesc), C.POINTER(abi.Rk3Params), i32, i32, C.c_double,
                                    vp, vp, vp, vp, vp, C.POINTER(i64)]
    lib.oracle_rk3_loop.argtypes = [C.POINTER(abi.GridDesc), C.POINTER(abi.Rk3Params), C.POINTER(abi.RunParams),
                                    vp, vp, vp, vp, vp, vp, C.POINTER(i64), dp, C.POINTER(abi.TseriesRow), i32,
                                    C.POINTER(i32), C.POINTER(i32), dp]
    lib.oracle_tseries.argtypes = [C.POINTER(abi.GridDesc), C.POINTER(abi.Rk3Params), C.POINTER(abi.RunParams),
                                   vp, vp, vp, vp, C.POINTER(i64), C.c_double, C.POINTER(abi.TseriesRow), dp]
    _lib = lib
    return lib


def set_threads(n: int):
    load().oracle_set_threads(n)


def max_threads() -> int:
    return load().oracle_max_threads()


def num_levels(grid, levels=0) -> int:
    return load().oracle_num_levels(C.byref(grid), levels)


def grid_metrics(grid, level, axis, levels=0):
    lib = load()
    cap = grid.n[axis] + 2
    x, a, b = (np.zeros(cap) for _ in range(3))
    n = C.c_int()
    dp = C.POINTER(C.c_double)
    s = lib.oracle_grid_metrics(C.byref(grid), levels, level, axis, x.ctypes.data_as(dp),
                                a.ctypes.data_as(dp), b.ctypes.data_as(dp), C.byref(n))
    if s:
        raise RuntimeError(f"oracle_grid_metrics status {s}")
    m = n.value + 2
    return x[:m].copy(), a[:m].copy(), b[:m].copy()


def null_vector(grid, axis):
    """Left null vector of the 1-D all-Neumann finest-level operator along
    `axis` (normalised to max |w| = 1), from the oracle's level-0 metrics:
    the column balance of the stretched second-difference operator of
    poisson_d3.cc:96-246 with Neumann ghosts (ghost = interior) gives the
    flux recurrence w[j+1] (c2 - c1)[j+1] = w[j] (c2 + c1)[j]."""
    n = grid.n[axis]
    _, xixx, xix2 = grid_metrics(grid, 0, axis)
    h = 1.0 / n
    ih2, i2h = 1.0 / (h * h), 0.5 / h
    c2 = xix2[1:n + 1] * ih2
    c1 = xixx[1:n + 1] * i2h
    lo, up = c2 - c1, c2 + c1
    w = np.zeros(n)
    w[0] = 1.0
    for j in range(n - 1):
        w[j + 1] = w[j] * up[j] / lo[j + 1]
    return w / np.abs(w).max()


def project_compatible(grid, f):
    """f minus its component along the separable left null vector of the
    all-Neumann operator, (w.f / w.1): a compatible right-hand side; plain
    mean subtraction on uniform axes."""
    ws = [null_vector(grid, d) if (grid.dims == 3 or d != 1) else np.ones(1) for d in range(3)]
    w = ws[0][:, None, None] * ws[1][None, :, None] * ws[2][None, None, :]
    return f - (w * f).sum() / w.sum()


def field_metrics(grid, axis):
    lib = load()
    m = grid.n[axis] + 2 * grid.pad
    arrs = [np.zeros(m) for _ in range(4)]
    dp = C.POINTER(C.c_double)
    s = lib.oracle_field_metrics(C.byref(grid), axis, *[a.ctypes.data_as(dp) for a in arrs])
    if s:
        raise RuntimeError(f"oracle_field_metrics status {s}")
    return arrs  # x, xi_x, xixx, xix2


class Result:
    pass


def mg_solve(grid, params, out_lhs: np.ndarray, inp_rhs: np.ndarray, hist_cap: int = 512):
    """poisson::mgSolve on numpy padded fields (out_lhs updated in place)."""
    lib = load()
    po, st = abi.field_origin(out_lhs, grid)
    pi, _ = abi.field_origin(inp_rhs, grid)
    hist = np.zeros(hist_cap)
    n, cs, sec = C.c_int(), C.c_int(), C.c_double()
    s = lib.oracle_mg_solve(C.byref(grid), C.byref(params), po, pi, st,
                            hist.ctypes.data_as(C.POINTER(C.c_double)), hist_cap, C.byref(n),
                            C.byref(cs), C.byref(sec))
    r = Result()
    r.status, r.cycles, r.coarse_sweeps, r.seconds = s, n.value, cs.value, sec.value
    r.history = hist[:min(n.value, hist_cap)].copy()
    return r


def rk3_run(grid, params, vx, vy, vz, p, t, pp, nsteps=1):
    lib = load()
    ptrs = []
    st = None
    for f in (vx, vy, vz, p, t, pp):
        if f is None:
            ptrs.append(C.c_void_p(0))
            continue
        ptr, st = abi.field_origin(f, grid)
        ptrs.append(ptr)
    mgc, cni, sec = C.c_int(), C.c_int(), C.c_double()
    s = lib.oracle_rk3_run(C.byref(grid), C.byref(params), *ptrs, st, nsteps, C.byref(mgc),
                           C.byref(cni), C.byref(sec))
    r = Result()
    r.status, r.mg_cycles, r.cn_iters, r.seconds = s, mgc.value, cni.value, sec.value
    return r


def field_op(grid, params, op, f, axis=0, v=(None, None, None), dcoef=1.0):
    """Core of one stencil operator applied to padded field f: op 1 first
    derivative, 2 second derivative along `axis`, 3 the convection term of
    f by velocity v (computeNLin into a zero H)."""
    lib = load()
    out = np.zeros_like(f)
    pf, st = abi.field_origin(f, grid)
    po, _ = abi.field_origin(out, grid)
    pv = [abi.field_origin(a, grid)[0] if a is not None else C.c_void_p(0) for a in v]
    s = lib.oracle_field_op(C.byref(grid), C.byref(params), op, axis, dcoef, pf, *pv, po, st)
    if s:
        raise RuntimeError(f"oracle_field_op status {s}")
    return out


def rk3_loop(grid, params, run, vx, vy, vz, p, t, pp, time=0.0, cap=4096):
    """The solvePDE time loop on numpy padded fields (updated in place)."""
    lib = load()
    ptrs = []
    st = None
    for f in (vx, vy, vz, p, t, pp):
        if f is None:
            ptrs.append(C.c_void_p(0))
            continue
        ptr, st = abi.field_origin(f, grid)
        ptrs.append(ptr)
    rows = (abi.TseriesRow * cap)()
    tm, nr, ns, dt = C.c_double(time), C.c_int(), C.c_int(), C.c_double()
    s = lib.oracle_rk3_loop(C.byref(grid), C.byref(params), C.byref(run), *ptrs, st, C.byref(tm), rows, cap,
                            C.byref(nr), C.byref(ns), C.byref(dt))
    r = Result()
    r.status, r.time, r.n_steps, r.dt = s, tm.value, ns.value, dt.value
    r.rows = [rows[q].as_dict() for q in range(min(nr.value, cap))]
    return r


def tseries(grid, params, run, vx, vy, vz, t, time=0.0):
    """(time-series row, CFL maximum) of the given fields."""
    lib = load()
    ptrs = []
    st = None
    for f in (vx, vy, vz, t):
        if f is None:
            ptrs.append(C.c_void_p(0))
            continue
        ptr, st = abi.field_origin(f, grid)
        ptrs.append(ptr)
    row, cm = abi.TseriesRow(), C.c_double()
    s = lib.oracle_tseries(C.byref(grid), C.byref(params), C.byref(run), *ptrs, st, time, C.byref(row),
                           C.byref(cm))
    if s not in (0, 8):  # 8: the divergence abort
        raise RuntimeError(f"oracle_tseries status {s}")
    return row.as_dict(), cm.value
