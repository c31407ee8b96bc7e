"""ctypes binding of libsaras_gb300.so, the C ABI declared in include/saras_gb300.h.

The binding mirrors the reference's operator interface for the multigrid
Poisson solve and the RK3 time step:

* ``Multigrid(grid, params).mg_solve(out_lhs, inp_rhs)`` follows
  ``void poisson::mgSolve(plainsf &outLHS, const plainsf &inpRHS)``
  (lib/poisson/poisson.cc:109-189): ``inp_rhs`` and ``out_lhs`` are padded
  fields (numpy arrays of shape (Nx+2p, Ny+2p, Nz+2p), k fastest) and
  ``out_lhs`` carries the initial guess in and the solution (core plus one
  ghost layer) out.
* ``RK3(grid, params).time_advance(...)`` follows
  ``lsRK3_d3::timeAdvance(vfield&, sfield&, sfield&)``
  (lib/timestep/lsRK3_d3.cc:190-305).

Every call goes to the CUDA library; there is no CPU path.  Loading fails
loudly when the library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os
import pathlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "lib" / "libsaras_gb300.so"

OK, NOT_CONVERGED, BAD_ARG, OOM, BUDGET, TIMEOUT, CUDA_ERR, NO_DEVICE, DIVERGED, NAN = range(10)
STATUS_NAMES = ["OK", "NOT_CONVERGED", "BAD_ARG", "OOM", "BUDGET", "TIMEOUT", "CUDA_ERR",
                "NO_DEVICE", "DIVERGED", "NAN"]
MESH = {"U": 0, "S": 1, "D": 2}
BC_NEUMANN, BC_DIRICHLET, BC_DIRICHLET_TEST = 0, 1, 2
PREC_FP64_EXACT, PREC_FP64, PREC_MIXED = 0, 1, 2
# time-step stencils: separately rounded in the reference's order, or FAST
STENCIL_EXACT, STENCIL_FAST = 0, 1
FBC_DIRICHLET, FBC_NEUMANN = 0, 1


class GridDesc(C.Structure):
    _fields_ = [("dims", C.c_int32), ("n", C.c_int32 * 3), ("len", C.c_double * 3),
                ("mesh_type", C.c_int32 * 3), ("beta", C.c_double * 3),
                ("periodic", C.c_int32 * 3), ("pad", C.c_int32)]


class MgParams(C.Structure):
    _fields_ = [("vc_count", C.c_int32), ("vc_tolerance", C.c_double), ("solve_flag", C.c_int32),
                ("mg_tolerance", C.c_double), ("sor_param", C.c_double),
                ("pre_smooth", C.c_int32), ("post_smooth", C.c_int32), ("res_type", C.c_int32),
                ("print_residual", C.c_int32), ("bc_kind", C.c_int32 * 6),
                ("test_poisson", C.c_int32), ("precision", C.c_int32), ("levels", C.c_int32),
                ("inner_cycles", C.c_int32)]


class FieldBC(C.Structure):
    _fields_ = [("type", C.c_int32 * 6), ("value", C.c_double * 6)]


class Rk3Params(C.Structure):
    _fields_ = [("nu", C.c_double), ("kappa", C.c_double), ("dt", C.c_double),
                ("cn_tolerance", C.c_double), ("max_iterations", C.c_int32),
                ("g_terms", C.c_double * 3), ("with_scalar", C.c_int32), ("nl_scheme", C.c_int32),
                ("bc_vx", FieldBC), ("bc_vy", FieldBC), ("bc_vz", FieldBC), ("bc_t", FieldBC),
                ("bc_p", FieldBC), ("mg", MgParams), ("pe_limit", C.c_double), ("up_param", C.c_double),
                ("integration", C.c_int32), ("stencil_form", C.c_int32)]


class RunParams(C.Structure):
    _fields_ = [("t_max", C.c_double), ("courant", C.c_double), ("use_cfl", C.c_int32), ("io_count", C.c_int32),
                ("prob_type", C.c_int32), ("max_steps", C.c_int32), ("g_axis", C.c_double * 3)]


class TseriesRow(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("time", "dt", "re", "nu_wall", "nu_vol", "ke", "te", "urms",
                                          "divergence")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def run_params(t_max=1.0, courant=0.2, use_cfl=False, io_count=1, prob_type=5, max_steps=0,
               g_axis=(0.0, 0.0, -1.0)) -> RunParams:
    """Time-loop keys of parameters.yaml ("Final Time", "Courant Number",
    "Use CFL Condition", "I/O Count", "Problem Type", "Gravity Direction")."""
    r = RunParams()
    r.t_max, r.courant, r.use_cfl, r.io_count = t_max, courant, int(bool(use_cfl)), io_count
    r.prob_type, r.max_steps = prob_type, max_steps
    for d in range(3):
        r.g_axis[d] = g_axis[d]
    return r


def grid_desc(n=(16, 16, 16), length=(1.0, 1.0, 1.0), mesh="UUU", beta=(1.0, 1.0, 1.0),
              domain="NNN", dims=3, pad=1) -> GridDesc:
    """Grid descriptor from the parameters.yaml Mesh/Program keys."""
    g = GridDesc()
    g.dims = dims
    nn = list(n)
    if dims == 2 and len(nn) == 2:
        nn = [nn[0], 1, nn[1]]
    if dims == 2:
        nn[1] = 1
    for d in range(3):
        g.n[d] = int(nn[d])
        g.len[d] = float(length[d])
        g.mesh_type[d] = MESH[mesh[d]]
        g.beta[d] = float(beta[d])
        g.periodic[d] = 1 if domain[d] == "P" else 0
    g.pad = pad
    return g


# Multigrid section of the reference's input/parameters.yaml
DEFAULT_MG = dict(vc_count=20, vc_tolerance=1.0e-6, solve_flag=1, mg_tolerance=1.0e-2, sor_param=1.0,
                  pre_smooth=3, post_smooth=6, res_type=0, print_residual=0, test_poisson=0,
                  precision=PREC_FP64_EXACT, levels=0, inner_cycles=1)


def mg_params(**kw) -> MgParams:
    """Multigrid parameters; defaults are the reference's parameters.yaml."""
    p = MgParams()
    for k, v in DEFAULT_MG.items():
        setattr(p, k, v)
    for k, v in kw.items():
        if k == "bc_kind":
            for i in range(6):
                p.bc_kind[i] = int(v[i])
        else:
            setattr(p, k, v)
    return p


def field_bc(types, values) -> FieldBC:
    b = FieldBC()
    for i in range(6):
        b.type[i] = int(types[i])
        b.value[i] = float(values[i])
    return b


def padded_shape(grid: GridDesc) -> tuple:
    """The reference's plainsf shape of a field (core + pad on each side)."""
    p = grid.pad
    ny = 1 if grid.dims == 2 else grid.n[1]
    py = 1 if grid.dims == 2 else p
    return (grid.n[0] + 2 * p, ny + 2 * py, grid.n[2] + 2 * p)


def padded_field(grid: GridDesc, dtype=np.float64) -> np.ndarray:
    """Zero field with the reference's plainsf shape (core + pad on each side)."""
    return np.zeros(padded_shape(grid), dtype=dtype)


def field_origin(a: np.ndarray, grid: GridDesc):
    """(pointer to element (0,0,0), element strides) of a padded field."""
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise ValueError("fields must be C-contiguous float64 arrays")
    p = grid.pad
    py = 1 if grid.dims == 2 else p
    st = [s // 8 for s in a.strides]
    off = p * st[0] + py * st[1] + p * st[2]
    ptr = a.ctypes.data + 8 * off
    return C.c_void_p(ptr), (C.c_int64 * 3)(*st)


_lib = None


def load():
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
    lib = C.CDLL(str(LIB_PATH))
    vp, i32, i64, dp = C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_double)
    lib.saras_mg_default_params.argtypes = [C.POINTER(MgParams)]
    lib.saras_mg_default_params.restype = None
    lib.saras_mg_create.argtypes = [C.POINTER(GridDesc), C.POINTER(MgParams), vp, C.POINTER(vp)]
    lib.saras_mg_create.restype = C.c_int
    for name in ("saras_mg_solve", "saras_mg_solve_dev"):
        f = getattr(lib, name)
        f.argtypes = [vp, vp, vp, C.POINTER(i64), dp, i32, C.POINTER(i32)]
        f.restype = C.c_int
    lib.saras_mg_destroy.argtypes = [vp]
    lib.saras_mg_destroy.restype = C.c_int
    lib.saras_mg_num_levels.argtypes = [vp]
    lib.saras_mg_num_levels.restype = i32
    lib.saras_mg_device_bytes.argtypes = [vp]
    lib.saras_mg_device_bytes.restype = i64
    lib.saras_mg_set_kernel_timing.argtypes = [vp, i32]
    lib.saras_mg_set_kernel_timing.restype = C.c_int
    lib.saras_mg_kernel_stats.argtypes = [vp, i32, C.POINTER(i64), dp, dp]
    lib.saras_mg_kernel_stats.restype = C.c_int
    lib.saras_mg_last_launches.argtypes = [vp]
    lib.saras_mg_last_launches.restype = i64
    lib.saras_mg_last_vcycles.argtypes = [vp]
    lib.saras_mg_last_vcycles.restype = i64
    lib.saras_mg_set_wait_limit.argtypes = [vp, i64]
    lib.saras_mg_set_wait_limit.restype = C.c_int
    lib.saras_measure_fp64_rate.argtypes = [vp, dp, dp]
    lib.saras_measure_fp64_rate.restype = C.c_int
    lib.saras_grid_metrics.argtypes = [C.POINTER(GridDesc), i32, i32, i32, dp, dp, dp, C.POINTER(i32)]
    lib.saras_grid_metrics.restype = C.c_int
    lib.saras_reference_levels.argtypes = [C.POINTER(GridDesc)]
    lib.saras_reference_levels.restype = i32
    lib.saras_neumann_null_vector.argtypes = [C.POINTER(GridDesc), i32, dp]
    lib.saras_neumann_null_vector.restype = C.c_int
    lib.saras_rbc_coefficients.argtypes = [i32, C.c_double, C.c_double, dp, dp, dp]
    lib.saras_rbc_coefficients.restype = C.c_int
    lib.saras_status_string.argtypes = [C.c_int]
    lib.saras_status_string.restype = C.c_char_p
    lib.saras_last_error.argtypes = []
    lib.saras_last_error.restype = C.c_char_p
    _lib = lib
    return lib


_rk3_bound = False


def _bind_rk3(lib):
    global _rk3_bound
    if _rk3_bound:
        return lib
    vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
    lib.saras_rk3_create.argtypes = [C.POINTER(GridDesc), C.POINTER(Rk3Params), vp, C.POINTER(vp)]
    lib.saras_rk3_create.restype = C.c_int
    lib.saras_rk3_upload.argtypes = [vp, vp, vp, vp, vp, vp, vp, C.POINTER(i64)]
    lib.saras_rk3_upload.restype = C.c_int
    lib.saras_rk3_download.argtypes = [vp, vp, vp, vp, vp, vp, vp, C.POINTER(i64)]
    lib.saras_rk3_download.restype = C.c_int
    lib.saras_rk3_step.argtypes = [vp, i32, C.POINTER(i32), C.POINTER(i32)]
    lib.saras_rk3_step.restype = C.c_int
    lib.saras_rk3_destroy.argtypes = [vp]
    lib.saras_rk3_destroy.restype = C.c_int
    lib.saras_rk3_last_launches.argtypes = [vp]
    lib.saras_rk3_last_launches.restype = i64
    lib.saras_rk3_tseries.argtypes = [vp, C.POINTER(RunParams), C.c_double, C.POINTER(TseriesRow)]
    lib.saras_rk3_tseries.restype = C.c_int
    lib.saras_rk3_cfl_dt.argtypes = [vp, C.c_double, C.POINTER(C.c_double)]
    lib.saras_rk3_cfl_dt.restype = C.c_int
    lib.saras_rk3_run.argtypes = [vp, C.POINTER(RunParams), C.POINTER(C.c_double), C.POINTER(TseriesRow), i32,
                                  C.POINTER(i32), C.POINTER(i32)]
    lib.saras_rk3_run.restype = C.c_int
    _rk3_bound = True
    return lib


class SarasError(RuntimeError):
    def __init__(self, status, where):
        lib = load()
        msg = lib.saras_last_error().decode()
        super().__init__(f"{where}: {STATUS_NAMES[status] if status < len(STATUS_NAMES) else status}"
                         f" {msg}")
        self.status = status


def check(status, where, allow=(OK,)):
    if status not in allow:
        raise SarasError(status, where)
    return status


def grid_metrics(grid: GridDesc, level: int, axis: int, levels: int = 0):
    """(x, xixx, xix2) of `axis` at `level`, indices -1..n_l."""
    lib = load()
    cap = grid.n[axis] + 2
    x, a, b = (np.zeros(cap) for _ in range(3))
    n = C.c_int32()
    dp = C.POINTER(C.c_double)
    check(lib.saras_grid_metrics(C.byref(grid), levels, level, axis, x.ctypes.data_as(dp),
                                 a.ctypes.data_as(dp), b.ctypes.data_as(dp), C.byref(n)),
          "saras_grid_metrics")
    m = n.value + 2
    return x[:m].copy(), a[:m].copy(), b[:m].copy()


def null_vector(grid: GridDesc, axis: int) -> np.ndarray:
    lib = load()
    w = np.zeros(grid.n[axis])
    check(lib.saras_neumann_null_vector(C.byref(grid), axis, w.ctypes.data_as(C.POINTER(C.c_double))),
          "saras_neumann_null_vector")
    return w


def measure_fp64_rate(stream: int | None = None):
    """(FP64 fused multiply-adds per second, separately rounded FP64 adds and
    multiplies per second) of the current device."""
    lib = load()
    a, b = C.c_double(), C.c_double()
    check(lib.saras_measure_fp64_rate(C.c_void_p(stream or 0), C.byref(a), C.byref(b)), "saras_measure_fp64_rate")
    return a.value, b.value


def project_compatible(grid: GridDesc, f: np.ndarray) -> np.ndarray:
    """Removes from a core RHS its component outside the range of the
    all-Neumann operator: f - (w.f / w.1) with w the separable left null
    vector.  On uniform axes this is mean subtraction."""
    ws = [null_vector(grid, d) if (grid.dims == 3 or d != 1) else np.ones(1) for d in range(3)]
    w = ws[0][:, None, None] * ws[1][None, :, None] * ws[2][None, None, :]
    return f - (w * f).sum() / w.sum()


class Multigrid:
    """Device-resident multigrid hierarchy: the reference's multigrid_d3 /
    multigrid_d2 object (lib/poisson/poisson.h:148-205)."""

    def __init__(self, grid: GridDesc, params: MgParams, stream: int | None = None):
        self.lib = load()
        self.grid = grid
        self.params = params
        h = C.c_void_p()
        check(self.lib.saras_mg_create(C.byref(grid), C.byref(params), C.c_void_p(stream or 0),
                                       C.byref(h)), "saras_mg_create")
        self.h = h
        self.history = []
        self.cycles = 0

    @property
    def levels(self) -> int:
        return self.lib.saras_mg_num_levels(self.h)

    def mg_solve(self, out_lhs: np.ndarray, inp_rhs: np.ndarray, hist_cap: int = 512) -> int:
        """mgSolve with host fields; returns OK or NOT_CONVERGED."""
        po, st = field_origin(out_lhs, self.grid)
        pi, _ = field_origin(inp_rhs, self.grid)
        hist = np.zeros(hist_cap)
        n = C.c_int32()
        s = self.lib.saras_mg_solve(self.h, po, pi, st, hist.ctypes.data_as(C.POINTER(C.c_double)),
                                    hist_cap, C.byref(n))
        check(s, "saras_mg_solve", allow=(OK, NOT_CONVERGED))
        self.cycles = n.value
        self.history = hist[:min(n.value, hist_cap)].copy()
        return s

    def mg_solve_dev(self, out_ptr: int, inp_ptr: int, strides, hist_cap: int = 512) -> int:
        """mgSolve with device pointers to element (0,0,0)."""
        st = (C.c_int64 * 3)(*strides)
        hist = np.zeros(hist_cap)
        n = C.c_int32()
        s = self.lib.saras_mg_solve_dev(self.h, C.c_void_p(out_ptr), C.c_void_p(inp_ptr), st,
                                        hist.ctypes.data_as(C.POINTER(C.c_double)), hist_cap,
                                        C.byref(n))
        check(s, "saras_mg_solve_dev", allow=(OK, NOT_CONVERGED))
        self.cycles = n.value
        self.history = hist[:min(n.value, hist_cap)].copy()
        return s

    def set_kernel_timing(self, on: bool):
        check(self.lib.saras_mg_set_kernel_timing(self.h, 1 if on else 0), "set_kernel_timing")

    def kernel_stats(self, kclass: int):
        n = C.c_int64()
        ms = C.c_double()
        b = C.c_double()
        check(self.lib.saras_mg_kernel_stats(self.h, kclass, C.byref(n), C.byref(ms), C.byref(b)),
              "kernel_stats")
        return n.value, ms.value, b.value

    def last_launches(self) -> int:
        return self.lib.saras_mg_last_launches(self.h)

    def set_wait_limit(self, polls: int):
        """Bound of the TMA sweeps' mbarrier waits in polls (0: default)."""
        check(self.lib.saras_mg_set_wait_limit(self.h, polls), "set_wait_limit")

    def last_vcycles(self) -> int:
        """V-cycles of the last solve (MIXED: FP32 V-cycles of all outer
        iterations)."""
        return self.lib.saras_mg_last_vcycles(self.h)

    def device_bytes(self) -> int:
        return self.lib.saras_mg_device_bytes(self.h)

    def close(self):
        if self.h:
            self.lib.saras_mg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def rbc_coefficients(rbc_type: int, ra: float, pr: float):
    lib = load()
    nu, ka, fb = C.c_double(), C.c_double(), C.c_double()
    check(lib.saras_rbc_coefficients(rbc_type, ra, pr, C.byref(nu), C.byref(ka), C.byref(fb)),
          "saras_rbc_coefficients")
    return nu.value, ka.value, fb.value


class RK3:
    """Device-resident lsRK3 integrator (lib/timestep/lsRK3_d3.cc)."""

    def __init__(self, grid: GridDesc, params: Rk3Params, stream: int | None = None):
        self.lib = _bind_rk3(load())
        self.grid = grid
        self.params = params
        h = C.c_void_p()
        check(self.lib.saras_rk3_create(C.byref(grid), C.byref(params), C.c_void_p(stream or 0),
                                        C.byref(h)), "saras_rk3_create")
        self.h = h

    def _ptrs(self, fields):
        out = []
        st = None
        for f in fields:
            if f is None:
                out.append(C.c_void_p(0))
                continue
            p = self.grid.pad
            py = 1 if self.grid.dims == 2 else p
            s = [x // 8 for x in f.strides]
            out.append(C.c_void_p(f.ctypes.data + 8 * (p * s[0] + py * s[1] + p * s[2])))
            st = (C.c_int64 * 3)(*s)
        return out, st

    def upload(self, vx, vy, vz, p, t, pp):
        ptrs, st = self._ptrs([vx, vy, vz, p, t, pp])
        check(self.lib.saras_rk3_upload(self.h, *ptrs, st), "saras_rk3_upload")

    def download(self, vx, vy, vz, p, t, pp):
        ptrs, st = self._ptrs([vx, vy, vz, p, t, pp])
        check(self.lib.saras_rk3_download(self.h, *ptrs, st), "saras_rk3_download")

    def step(self, nsteps: int = 1):
        mgc, cni = C.c_int32(), C.c_int32()
        check(self.lib.saras_rk3_step(self.h, nsteps, C.byref(mgc), C.byref(cni)), "saras_rk3_step")
        return mgc.value, cni.value

    def last_launches(self) -> int:
        return self.lib.saras_rk3_last_launches(self.h)

    def tseries(self, run: RunParams, time: float = 0.0) -> dict:
        """Time-series row of the current fields (tseries::writeTSData)."""
        row = TseriesRow()
        check(self.lib.saras_rk3_tseries(self.h, C.byref(run), time, C.byref(row)), "saras_rk3_tseries",
              allow=(OK, DIVERGED))
        return row.as_dict()

    def cfl_dt(self, courant: float) -> float:
        dt = C.c_double()
        check(self.lib.saras_rk3_cfl_dt(self.h, courant, C.byref(dt)), "saras_rk3_cfl_dt")
        return dt.value

    def run(self, run: RunParams, time: float = 0.0, cap: int = 4096):
        """The solvePDE time loop from `time`: (status, end time, steps, rows)."""
        rows = (TseriesRow * cap)()
        tm, nr, ns = C.c_double(time), C.c_int32(), C.c_int32()
        s = self.lib.saras_rk3_run(self.h, C.byref(run), C.byref(tm), rows, cap, C.byref(nr), C.byref(ns))
        check(s, "saras_rk3_run", allow=(OK, DIVERGED))
        return s, tm.value, ns.value, [rows[q].as_dict() for q in range(min(nr.value, cap))]

    def close(self):
        if self.h:
            self.lib.saras_rk3_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ServeParams(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_int64), ("max_cases", C.c_int32), ("max_cycles", C.c_int32),
                ("tolerance", C.c_double), ("mg_tolerance", C.c_double), ("sor_param", C.c_double),
                ("pre_smooth", C.c_int32), ("post_smooth", C.c_int32),
                ("cells_per_item", C.c_int32), ("threads", C.c_int32), ("blocks_per_sm", C.c_int32),
                ("pad_", C.c_int32)]


class ServeStats(C.Structure):
    _fields_ = [("bytes_allocated", C.c_int64), ("batched_cycles", C.c_int64), ("launches", C.c_int64),
                ("admitted", C.c_int64), ("retired", C.c_int64), ("active", C.c_int32),
                ("pending", C.c_int32), ("pooled", C.c_int32), ("max_active", C.c_int32),
                ("t_batch_s", C.c_double), ("t_admit_s", C.c_double), ("t_retire_s", C.c_double),
                ("t_steps_s", C.c_double)]


_serve_bound = False


def _bind_serve(lib):
    global _serve_bound
    if _serve_bound:
        return lib
    vp, i32, i64, dp = C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_double)
    lib.saras_serve_default_params.argtypes = [C.POINTER(ServeParams)]
    lib.saras_serve_default_params.restype = None
    lib.saras_serve_create.argtypes = [C.POINTER(ServeParams), C.POINTER(vp)]
    lib.saras_serve_create.restype = C.c_int
    lib.saras_serve_submit.argtypes = [vp, i64, C.POINTER(GridDesc), vp, vp]
    lib.saras_serve_submit.restype = C.c_int
    lib.saras_serve_submit_step.argtypes = [vp, i64, C.POINTER(GridDesc), C.POINTER(Rk3Params), vp, vp, vp, vp,
                                            vp, vp]
    lib.saras_serve_submit_step.restype = C.c_int
    lib.saras_serve_step.argtypes = [vp, C.POINTER(i32), C.POINTER(i32)]
    lib.saras_serve_step.restype = C.c_int
    lib.saras_serve_poll.argtypes = [vp, C.POINTER(i64), dp, C.POINTER(i32), C.POINTER(i32), dp, i32,
                                     C.POINTER(i32)]
    lib.saras_serve_poll.restype = C.c_int
    lib.saras_serve_autotune.argtypes = [vp, C.POINTER(GridDesc), i32, i32, C.POINTER(ServeParams)]
    lib.saras_serve_autotune.restype = C.c_int
    lib.saras_serve_get_stats.argtypes = [vp, C.POINTER(ServeStats)]
    lib.saras_serve_get_stats.restype = C.c_int
    lib.saras_serve_destroy.argtypes = [vp]
    lib.saras_serve_destroy.restype = C.c_int
    _serve_bound = True
    return lib


def serve_params(**kw) -> ServeParams:
    lib = _bind_serve(load())
    p = ServeParams()
    lib.saras_serve_default_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class Serve:
    """Continuous-batching engine of independent Poisson requests (MIXED
    form, all admitted requests advanced by one graph launch per step) and
    time-step requests, whose pressure solves join the same batch.
    Request buffers are padded host fields (``padded_field(grid)``) that
    must stay alive until the request is returned by ``poll``."""

    def __init__(self, params: ServeParams | None = None):
        self.lib = _bind_serve(load())
        self.params = params or serve_params()
        h = C.c_void_p()
        check(self.lib.saras_serve_create(C.byref(self.params), C.byref(h)), "saras_serve_create")
        self.h = h
        self._keep = {}

    def submit(self, rid: int, grid: GridDesc, rhs: np.ndarray, lhs: np.ndarray):
        shape = padded_shape(grid)
        for a in (rhs, lhs):
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.shape != shape:
                raise ValueError("request fields must be C-contiguous float64 padded boxes of the grid")
        check(self.lib.saras_serve_submit(self.h, rid, C.byref(grid), C.c_void_p(rhs.ctypes.data),
                                          C.c_void_p(lhs.ctypes.data)), "saras_serve_submit")
        self._keep[rid] = (grid, rhs, lhs)

    def submit_step(self, rid: int, grid: GridDesc, params: Rk3Params, fields: dict):
        """One time step of `fields` (vx, vy, vz, p, t, pp padded boxes,
        updated in place when the request is polled)."""
        shape = padded_shape(grid)
        ptrs = []
        for k in ("vx", "vy", "vz", "p", "t", "pp"):
            a = fields.get(k)
            if a is None:
                ptrs.append(C.c_void_p(0))
                continue
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.shape != shape:
                raise ValueError("request fields must be C-contiguous float64 padded boxes of the grid")
            ptrs.append(C.c_void_p(a.ctypes.data))
        check(self.lib.saras_serve_submit_step(self.h, rid, C.byref(grid), C.byref(params), *ptrs),
              "saras_serve_submit_step")
        self._keep[rid] = (grid, params, fields)

    def step(self):
        a, p = C.c_int32(), C.c_int32()
        check(self.lib.saras_serve_step(self.h, C.byref(a), C.byref(p)), "saras_serve_step")
        return a.value, p.value

    def poll(self, cap: int = 4096):
        ids = np.zeros(cap, np.int64)
        res = np.zeros(cap)
        cyc = np.zeros(cap, np.int32)
        st = np.zeros(cap, np.int32)
        lat = np.zeros(cap)
        n = C.c_int32()
        i32p = C.POINTER(C.c_int32)
        dp = C.POINTER(C.c_double)
        check(self.lib.saras_serve_poll(self.h, ids.ctypes.data_as(C.POINTER(C.c_int64)), res.ctypes.data_as(dp),
                                        cyc.ctypes.data_as(i32p), st.ctypes.data_as(i32p),
                                        lat.ctypes.data_as(dp), cap, C.byref(n)), "saras_serve_poll")
        out = []
        for q in range(n.value):
            rid = int(ids[q])
            self._keep.pop(rid, None)
            out.append(dict(id=rid, residual=float(res[q]), cycles=int(cyc[q]), status=int(st[q]),
                            latency_s=float(lat[q])))
        return out

    def run(self, max_steps: int = 1_000_000):
        """Steps until nothing is active or pending; returns every finished request."""
        done = []
        for _ in range(max_steps):
            a, p = self.step()
            done += self.poll()
            if a == 0 and p == 0:
                break
        return done

    def autotune(self, grids, cycles: int = 3) -> ServeParams:
        arr = (GridDesc * len(grids))(*grids)
        chosen = ServeParams()
        check(self.lib.saras_serve_autotune(self.h, arr, len(grids), cycles, C.byref(chosen)),
              "saras_serve_autotune")
        return chosen

    def stats(self) -> dict:
        s = ServeStats()
        check(self.lib.saras_serve_get_stats(self.h, C.byref(s)), "saras_serve_get_stats")
        return {k: getattr(s, k) for k, _ in ServeStats._fields_}

    def close(self):
        if self.h:
            self.lib.saras_serve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def exported_symbols():
    """Names declared by include/saras_gb300.h (checked by the tests)."""
    import re
    hdr = (HERE.parent / "include" / "saras_gb300.h").read_text()
    return sorted(set(re.findall(r"\b(saras_[a-z0-9_]+)\s*\(", hdr)))


if os.environ.get("SARAS_GB300_EAGER_LOAD"):
    load()
