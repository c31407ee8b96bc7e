"""The FAST time-step stencils (saras_rk3_params.stencil_form = 1): the same
right-hand sides and Crank-Nicolson sweeps as the separately rounded form
(which test_gpu_rk3.py holds bit for bit to the oracle's restatement of
lsRK3_d3/eulerCN_d3::timeAdvance), with folded coefficients and fused
multiply-adds.  Bar: after three steps with the FP64_EXACT pressure solve,
the same V-cycle and Jacobi counts as the exact form and every field within
1e-10 of it, relative to the field's largest magnitude; and the same against
the oracle directly on one case.
"""
import numpy as np
import pytest

import pyoracle as O
import saras_gb300 as S
from test_gpu_rk3 import initial_fields, rbc_params

pytestmark = pytest.mark.gpu

TOL = 1e-10
FIELDS = ("vx", "vy", "vz", "p", "t", "pp")

CASES = [
    # dScheme 1, central non-linear term, RK3, RBC box with periodic sides
    (dict(n=(16, 16, 32), mesh="UUD", beta=(1, 1, 1.5), domain="PPN"), 0.0, {}),
    # dScheme 2 (pad 2) with the hybrid upwind term on a stretched wall box
    (dict(n=(16, 16, 16), mesh="DDD", beta=(1.1, 1.2, 1.3), domain="NNN", pad=2), 0.05,
     dict(nl_scheme=2, pe_limit=0.5)),
    # dScheme 1, hybrid upwind (first order above the Peclet limit)
    (dict(n=(16, 16, 16), mesh="DDD", beta=(1.1, 1.2, 1.3), domain="NNN"), 0.05,
     dict(nl_scheme=2, pe_limit=0.5)),
    # Morinishi's skew-symmetric term, dScheme 1 and 2
    (dict(n=(16, 16, 32), mesh="UUD", beta=(1, 1, 1.3), domain="PPN"), 0.05, dict(nl_scheme=3)),
    (dict(n=(16, 16, 32), mesh="UUD", beta=(1, 1, 1.3), domain="PPN", pad=2), 0.05, dict(nl_scheme=3)),
    # Euler / Crank-Nicolson, planar
    (dict(n=(32, 1, 32), mesh="UUD", beta=(1, 1, 1.3), domain="PNN", dims=2), 0.0, dict(integration=1)),
    # no scalar (a random start on a wall box: with u = 0 and no buoyancy
    # nothing moves)
    (dict(n=(16, 16, 16), mesh="DDD", beta=(1.1, 1.2, 1.3), domain="NNN"), 0.05, dict(with_scalar=0)),
]
IDS = ["ppn_ds1", "nnn_ds2_upwind", "nnn_ds1_upwind", "ppn_morinishi", "ppn_ds2_morinishi", "planar_euler",
       "hydro"]


def _run(gk, amp, form, steps=3, **pk):
    g = S.grid_desc(**gk)
    prm = rbc_params(g, **pk)
    prm.stencil_form = form
    f = initial_fields(g, 4, amp)
    rk = S.RK3(g, prm)
    rk.upload(f["vx"], f["vy"], f["vz"], f["p"], f["t"], f["pp"])
    counts = rk.step(steps)
    rk.download(f["vx"], f["vy"], f["vz"], f["p"], f["t"], f["pp"])
    rk.close()
    return g, f, counts


def _close(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() / scale


@pytest.mark.parametrize("gk,amp,pk", CASES, ids=IDS)
def test_fast_stencils_match_exact(gk, amp, pk):
    g, exact, ce = _run(gk, amp, S.STENCIL_EXACT, **pk)
    _, fast, cf = _run(gk, amp, S.STENCIL_FAST, **pk)
    assert cf == ce, (cf, ce)
    planar = g.dims == 2
    for k in FIELDS:
        if planar and k == "vy":
            continue
        if "with_scalar" in pk and k == "t":
            continue
        a, b = (fast[k][:, 1, :], exact[k][:, 1, :]) if planar else (fast[k], exact[k])
        err = _close(a, b)
        assert err <= TOL, (k, err)
    # the forms differ: the FAST values are not the separately rounded ones
    assert any(not np.array_equal(fast[k], exact[k]) for k in ("vx", "vz", "p"))


def test_fast_stencils_against_the_oracle():
    gk = dict(n=(16, 16, 32), mesh="UUD", beta=(1, 1, 1.5), domain="PPN")
    g, fast, cf = _run(gk, 0.0, S.STENCIL_FAST)
    prm = rbc_params(g)
    orc = initial_fields(g, 4, 0.0)
    r = O.rk3_run(g, prm, orc["vx"], orc["vy"], orc["vz"], orc["p"], orc["t"], orc["pp"], 3)
    assert r.status == 0 and cf == (r.mg_cycles, r.cn_iters)
    for k in FIELDS:
        assert _close(fast[k], orc[k]) <= TOL, k


def test_stencil_form_is_checked():
    g = S.grid_desc(n=(16, 16, 16), mesh="UUU", domain="PPN")
    prm = rbc_params(g)
    prm.stencil_form = 2
    with pytest.raises(S.SarasError):
        S.RK3(g, prm)
