"""GPU time loop (saras_rk3_run / saras_rk3_tseries / saras_rk3_cfl_dt) against
the oracle's restatement of scalar_d3::solvePDE, vfield::computeTStp and
tseries::writeTSData (src/solvers/scalar/scalar_d3.cc:184-262,
lib/field/vfield.cc:691-719, lib/io/tseries.cc:209-488).

Bars: the CFL time step, the divergence maximum, the step count, the time
and every field bit for bit (maxima are order-independent; the fields come
from the bit-exact steps); the energy, Nusselt and Reynolds sums to 1e-12
relative -- the reference sums sequentially, the GPU in a fixed tree order.
"""
import numpy as np
import pytest

import pyoracle as O
import saras_gb300 as S
from test_gpu_rk3 import assert_fields_equal, initial_fields, rbc_params

pytestmark = pytest.mark.gpu

GRIDS = [
    (dict(n=(16, 16, 32), mesh="UUD", beta=(1, 1, 1.5), domain="PPN"), 0.05),
    (dict(n=(16, 16, 16), mesh="DDD", beta=(1.1, 1.2, 1.3), domain="NNN"), 0.05),
    (dict(n=(32, 1, 32), mesh="UUD", beta=(1, 1, 1.3), domain="PNN", dims=2), 0.05),
]
IDS = ["rbc_ppn_uud", "box_nnn_ddd", "planar_pnn"]


def close_rows(a, b, keys=("ke", "te", "nu_wall", "re", "urms")):
    assert a["divergence"] == b["divergence"]
    assert a["time"] == b["time"] and a["dt"] == b["dt"]
    for k in keys:
        assert abs(a[k] - b[k]) <= 1e-12 * max(abs(b[k]), 1e-300), (k, a[k], b[k])
    assert abs(a["nu_vol"] - b["nu_vol"]) <= 1e-12 * max(1.0, abs(b["nu_vol"])), (a["nu_vol"], b["nu_vol"])


@pytest.mark.parametrize("gk,amp", GRIDS, ids=IDS)
@pytest.mark.parametrize("pad", [1, 2])
@pytest.mark.parametrize("sc", [1, 0])
def test_tseries_row_and_cfl(gk, amp, pad, sc):
    g = S.grid_desc(pad=pad, **gk)
    prm = rbc_params(g, with_scalar=sc)
    f = initial_fields(g, 7, amp)
    rk = S.RK3(g, prm)
    rk.upload(f["vx"], f["vy"], f["vz"], f["p"], f["t"], f["pp"])
    for run in (S.run_params(), S.run_params(prob_type=9), S.run_params(g_axis=(-1.0, 0.0, 0.0))):
        row = rk.tseries(run, time=0.25)
        ref, cfl = O.tseries(g, prm, run, f["vx"], f["vy"], f["vz"], f["t"] if sc else None, time=0.25)
        close_rows(row, ref, ("ke", "te", "nu_wall", "re", "urms") if sc else ("ke", "urms"))
        assert rk.cfl_dt(0.4) == 0.4 / cfl
    rk.close()


@pytest.mark.parametrize("gk,amp", GRIDS, ids=IDS)
@pytest.mark.parametrize("pad,integration,nl", [(1, 2, 1), (2, 2, 3), (2, 1, 2)])
def test_time_loop_matches_oracle(gk, amp, pad, integration, nl):
    """CFL-limited steps (the Courant number puts dt below the "Time-Step"
    cap after the first step), a row every second step, until Final Time."""
    g = S.grid_desc(pad=pad, **gk)
    prm = rbc_params(g, integration=integration, nl_scheme=nl, pe_limit=0.5)
    prm.dt = 4e-3
    run = S.run_params(t_max=0.012, courant=0.008, use_cfl=True, io_count=2)
    f0 = initial_fields(g, 4, amp)
    gpu = {k: v.copy() for k, v in f0.items()}
    orc = {k: v.copy() for k, v in f0.items()}
    rk = S.RK3(g, prm)
    rk.upload(gpu["vx"], gpu["vy"], gpu["vz"], gpu["p"], gpu["t"], gpu["pp"])
    st, t_end, steps, rows = rk.run(run, time=0.0)
    rk.download(gpu["vx"], gpu["vy"], gpu["vz"], gpu["p"], gpu["t"], gpu["pp"])
    rk.close()
    ref = O.rk3_loop(g, prm, run, orc["vx"], orc["vy"], orc["vz"], orc["p"], orc["t"], orc["pp"])
    assert st == ref.status == 0
    assert steps == ref.n_steps and t_end == ref.time and len(rows) == len(ref.rows)
    assert steps >= 3 and len({r["dt"] for r in rows}) > 1  # the CFL step changed dt
    for a, b in zip(rows, ref.rows):
        close_rows(a, b)
    assert_fields_equal(g, gpu, orc)


def test_time_loop_without_cfl_equals_steps():
    gk, amp = GRIDS[1]
    g = S.grid_desc(**gk)
    prm = rbc_params(g)
    f0 = initial_fields(g, 4, amp)
    a = {k: v.copy() for k, v in f0.items()}
    b = {k: v.copy() for k, v in f0.items()}
    rk = S.RK3(g, prm)
    rk.upload(a["vx"], a["vy"], a["vz"], a["p"], a["t"], a["pp"])
    st, t_end, steps, rows = rk.run(S.run_params(t_max=3 * prm.dt, io_count=1), time=0.0)
    rk.download(a["vx"], a["vy"], a["vz"], a["p"], a["t"], a["pp"])
    rk.close()
    assert st == S.OK and steps == 3 and len(rows) == 4
    rk = S.RK3(g, prm)
    rk.upload(b["vx"], b["vy"], b["vz"], b["p"], b["t"], b["pp"])
    rk.step(3)
    rk.download(b["vx"], b["vy"], b["vz"], b["p"], b["t"], b["pp"])
    rk.close()
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_time_loop_bad_arguments():
    g = S.grid_desc(n=(8, 8, 8), domain="NNN")
    rk = S.RK3(g, rbc_params(g))
    with pytest.raises(S.SarasError):
        rk.run(S.run_params(io_count=0))
    with pytest.raises(S.SarasError):
        rk.run(S.run_params(use_cfl=True, courant=0.0))
    rk.close()
