"""Time-step requests in the serving engine (saras_serve_submit_step): one
lsRK3 or eulerCN timeAdvance whose pressure solves run in the engine's
batch next to Poisson requests.

Bars: a step request's fields are bit-for-bit the same alone, in a mix with
Poisson and other step requests, and the same as saras_rk3_step on a handle
whose multigrid is the MIXED form with the engine's smoothing and coarsest
tolerance and the request's own Residual Tolerance and V-Cycle Count; the
Poisson requests of the mix keep their alone results.
"""
import numpy as np
import pytest

import saras_gb300 as S
from helpers import random_rhs
from test_gpu_rk3 import initial_fields, rbc_params

pytestmark = pytest.mark.gpu

# the engine's form, smoothing and coarsest tolerance; step requests stop
# their pressure solves at their own Residual Tolerance / V-Cycle Count
ENGINE = dict(tolerance=1e-9, max_cycles=400, mg_tolerance=1e-9, pre_smooth=3, post_smooth=6, max_cases=16)
STEP_TOL, STEP_CAP = 1e-6, 20
STEPS = [
    dict(gk=dict(n=(16, 16, 16), mesh="DDD", beta=(1.1, 1.2, 1.3), domain="NNN"), amp=0.05, pk={}),
    dict(gk=dict(n=(16, 16, 32), mesh="UUD", beta=(1, 1, 1.3), domain="PPN", pad=2), amp=0.05,
         pk=dict(nl_scheme=3)),
    dict(gk=dict(n=(32, 1, 32), mesh="UUD", beta=(1, 1, 1.3), domain="PNN", dims=2), amp=0.05,
         pk=dict(integration=1, nl_scheme=2, pe_limit=0.5)),
]
POISSON = [dict(n=(32, 32, 32), mesh="UUD", beta=(1, 1, 1.2), domain="NNN"),
           dict(n=(64, 1, 64), mesh="UUD", beta=(1, 1, 1.4), domain="NNN", dims=2)]


def _step_request(q):
    c = STEPS[q]
    g = S.grid_desc(**c["gk"])
    prm = rbc_params(g, vc_tol=STEP_TOL, **c["pk"])
    prm.mg.vc_count = STEP_CAP
    return g, prm, initial_fields(g, 20 + q, c["amp"])


def _alone_handle(q):
    """saras_rk3_step with the engine's multigrid parameters."""
    g, prm, f = _step_request(q)
    prm.mg = S.mg_params(precision=S.PREC_MIXED, vc_count=STEP_CAP, vc_tolerance=STEP_TOL, mg_tolerance=1e-9,
                         pre_smooth=3, post_smooth=6)
    rk = S.RK3(g, prm)
    rk.upload(f["vx"], f["vy"], f["vz"], f["p"], f["t"], f["pp"])
    rk.step(1)
    rk.download(f["vx"], f["vy"], f["vz"], f["p"], f["t"], f["pp"])
    rk.close()
    return f


def _serve(step_ids, poisson_ids):
    eng = S.Serve(S.serve_params(**ENGINE))
    fields, pois = {}, {}
    for q in step_ids:
        g, prm, f = _step_request(q)
        eng.submit_step(100 + q, g, prm, f)
        fields[q] = f
    for q in poisson_ids:
        g = S.grid_desc(**POISSON[q])
        rhs, lhs = random_rhs(g, 40 + q), S.padded_field(g)
        eng.submit(q, g, rhs, lhs)
        pois[q] = lhs
    done = {d["id"]: d for d in eng.run()}
    st = eng.stats()
    eng.close()
    return fields, pois, done, st


@pytest.fixture(scope="module")
def alone():
    return {q: _serve([q], [])[0][q] for q in range(len(STEPS))}


def test_step_request_equals_rk3_step(alone):
    for q in range(len(STEPS)):
        ref = _alone_handle(q)
        for k in ref:
            assert np.array_equal(alone[q][k], ref[k]), (q, k)


def test_steps_same_in_the_mix(alone):
    pois_alone = _serve([], [0, 1])[1]
    fields, pois, done, st = _serve([0, 1, 2], [0, 1])
    assert st["max_active"] == 5
    for q in range(len(STEPS)):
        # a pressure solve stopped at its V-Cycle Count is no failure (mgSolve
        # returns after vcCount cycles, poisson.cc:182-188)
        assert done[100 + q]["status"] == S.OK, done[100 + q]
        assert done[100 + q]["cycles"] >= 1
        for k in fields[q]:
            assert np.array_equal(fields[q][k], alone[q][k]), (q, k)
    for q in (0, 1):
        assert done[q]["status"] == S.OK
        assert np.array_equal(pois[q], pois_alone[q])


def test_step_request_changes_fields():
    g, prm, f0 = _step_request(0)
    f = {k: v.copy() for k, v in f0.items()}
    eng = S.Serve(S.serve_params(**ENGINE))
    eng.submit_step(7, g, prm, f)
    done = eng.run()
    eng.close()
    assert done[0]["id"] == 7 and np.isfinite(f["vx"]).all()
    assert not np.array_equal(f["vx"], f0["vx"]) and not np.array_equal(f["p"], f0["p"])


def test_step_request_over_budget():
    g, prm, f = _step_request(0)
    eng = S.Serve(S.serve_params(hbm_budget_bytes=1 << 20, **ENGINE))
    eng.submit_step(9, g, prm, f)
    done = eng.run()
    eng.close()
    assert done[0]["status"] == S.BUDGET


def test_step_request_bad_solve_keys():
    g, prm, f = _step_request(0)
    prm.mg.vc_count = 0
    eng = S.Serve(S.serve_params(**ENGINE))
    with pytest.raises(S.SarasError):
        eng.submit_step(3, g, prm, f)
    eng.close()


def test_pooled_integrator_gives_same_results(alone):
    """A second request of the same shape reuses the first one's integrator
    (re-pointed at its stretching and parameters): results unchanged."""
    eng = S.Serve(S.serve_params(**ENGINE))
    g0, prm0, f0 = _step_request(0)
    g1 = S.grid_desc(**dict(STEPS[0]["gk"], beta=(1.3, 1.1, 1.2)))
    prm1 = rbc_params(g1, vc_tol=STEP_TOL)
    prm1.mg.vc_count = STEP_CAP
    f1 = initial_fields(g1, 5, 0.05)
    eng.submit_step(1, g1, prm1, f1)
    assert eng.run()[0]["id"] == 1
    assert eng.stats()["pooled"] == 1
    eng.submit_step(2, g0, prm0, f0)
    assert eng.run()[0]["id"] == 2
    eng.close()
    for k in f0:
        assert np.array_equal(f0[k], alone[0][k]), k


def test_failing_step_request_leaves_the_mix():
    """A time-step request whose temperature holds a NaN fails in its first
    Crank-Nicolson sweep, on the engine's step worker: it is polled with
    status NAN, and a Poisson request served beside it keeps its alone
    result."""
    pois_alone = _serve([], [0])[1]
    g, prm, f = _step_request(0)
    f["t"][3, 3, 3] = np.nan
    eng = S.Serve(S.serve_params(**ENGINE))
    eng.submit_step(100, g, prm, f)
    gp = S.grid_desc(**POISSON[0])
    rhs, lhs = random_rhs(gp, 40), S.padded_field(gp)
    eng.submit(0, gp, rhs, lhs)
    done = {d["id"]: d for d in eng.run()}
    st = eng.stats()
    eng.close()
    assert done[100]["status"] == S.NAN
    assert done[0]["status"] == S.OK and np.array_equal(lhs, pois_alone[0])
    assert st["active"] == 0 and st["retired"] == 2
