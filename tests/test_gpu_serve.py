"""Serving engine (continuous batching of independent Poisson requests) on
the GPU, through the C ABI.

Bars: a request's solution, residual and outer-iteration count are bit-for-
bit the same alone, in any mix, under any schedule the autotuner may pick,
and the same as the single-problem MIXED solve (saras_mg_solve) with the
engine's parameters.  Against the FP64 oracle the converged solution agrees
to 1e-9 relative (constant null-space component removed).
"""
import numpy as np
import pytest

import pyoracle as O
import saras_gb300 as S
from helpers import core, demean, random_rhs

pytestmark = pytest.mark.gpu

TOL = 1e-8
# cells of equal extent in every direction before stretching (the reference
# V-cycle diverges on strongly anisotropic cells), 3/6 smoothing (the
# reference defaults) and a 1e-9 coarsest tolerance
CASES = [
    dict(n=(32, 32, 32), mesh="UUD", beta=(1, 1, 1.2), domain="NNN"),
    dict(n=(64, 1, 64), mesh="UUD", beta=(1, 1, 1.4), domain="NNN", dims=2),
    dict(n=(48, 32, 16), length=(1.0, 2 / 3, 1 / 3), mesh="UUD", beta=(1, 1, 1.05), domain="NNN"),
    dict(n=(32, 32, 32), mesh="UUU", domain="NNN"),
    dict(n=(16, 16, 32), length=(0.5, 0.5, 1.0), mesh="UUD", beta=(1, 1, 1.5), domain="NNN"),
]
MG = dict(mg_tolerance=1e-9, pre_smooth=3, post_smooth=6)


def _params(**kw):
    base = dict(tolerance=TOL, max_cycles=400, max_cases=16, **MG)
    base.update(kw)
    return S.serve_params(**base)


def _request(gk, seed):
    g = S.grid_desc(**gk)
    return g, random_rhs(g, seed), S.padded_field(g)


def _serve(reqs, params=None, tune=None):
    eng = S.Serve(params or _params())
    if tune:
        eng.autotune([S.grid_desc(**gk) for gk in tune], cycles=1)
    for rid, (g, rhs, lhs) in reqs.items():
        eng.submit(rid, g, rhs, lhs)
    done = {d["id"]: d for d in eng.run()}
    stats = eng.stats()
    eng.close()
    return done, stats


def _alone(gk, seed):
    g, rhs, lhs = _request(gk, seed)
    done, _ = _serve({0: (g, rhs, lhs)})
    return lhs, done[0]


@pytest.fixture(scope="module")
def alone():
    return [_alone(gk, 10 + q) for q, gk in enumerate(CASES)]


def test_each_request_converges(alone):
    for (lhs, d), gk in zip(alone, CASES):
        assert d["status"] == S.OK, (gk, d)
        assert d["residual"] < TOL and d["cycles"] > 1
        assert np.isfinite(lhs).all()


def test_same_alone_and_in_the_mix(alone):
    reqs = {q: _request(gk, 10 + q) for q, gk in enumerate(CASES)}
    done, stats = _serve(reqs)
    assert stats["max_active"] == len(CASES)  # all on the device together
    for q in range(len(CASES)):
        lhs_a, d_a = alone[q]
        assert done[q]["status"] == S.OK
        assert done[q]["cycles"] == d_a["cycles"]
        assert done[q]["residual"] == d_a["residual"]
        assert np.array_equal(reqs[q][2], lhs_a)


def test_same_as_single_problem_mixed_solve(alone):
    for q, gk in enumerate(CASES):
        g, rhs, _ = _request(gk, 10 + q)
        lhs = S.padded_field(g)
        mg = S.Multigrid(g, S.mg_params(precision=S.PREC_MIXED, vc_count=400, vc_tolerance=TOL, **MG))
        assert mg.mg_solve(lhs, rhs) == S.OK
        cycles = mg.cycles
        mg.close()
        lhs_a, d_a = alone[q]
        assert cycles == d_a["cycles"], gk
        assert np.array_equal(lhs, lhs_a), gk


def test_matches_fp64_oracle():
    """Served to 1e-10, the solutions agree with the oracle's converged FP64
    solve to 1e-9 relative (constant null-space component removed)."""
    reqs = {q: _request(CASES[q], 10 + q) for q in (0, 1, 4)}
    done, _ = _serve(reqs, params=_params(tolerance=1e-10))
    for q, (g, rhs, lhs) in reqs.items():
        assert done[q]["status"] == S.OK
        orc = S.padded_field(g)
        r = O.mg_solve(g, S.mg_params(vc_count=400, vc_tolerance=1e-12, **MG), orc, rhs)
        assert r.history[-1] < 1e-12
        a, b = demean(core(lhs, g)), demean(core(orc, g))
        assert np.abs(a - b).max() <= 1e-9 * np.abs(b).max(), CASES[q]


def test_continuous_admission_with_two_slots(alone):
    """Requests arrive while others are on the device; slots free up as
    requests retire; results are unchanged."""
    eng = S.Serve(_params(max_cases=2))
    reqs = {q: _request(gk, 10 + q) for q, gk in enumerate(CASES)}
    order = list(range(len(CASES)))
    for q in order[:2]:
        eng.submit(q, *reqs[q])
    done = {}
    nxt = 2
    steps = 0
    while True:
        a, p = eng.step()
        steps += 1
        assert a <= 2
        if steps % 3 == 0 and nxt < len(order):  # a late arrival
            eng.submit(order[nxt], *reqs[order[nxt]])
            nxt += 1
        for d in eng.poll():
            done[d["id"]] = d
        if a == 0 and p == 0 and nxt == len(order):
            break
        assert steps < 5000
    st = eng.stats()
    eng.close()
    assert st["max_active"] == 2 and st["retired"] == len(CASES)
    for q in order:
        assert done[q]["status"] == S.OK and done[q]["latency_s"] > 0
        assert np.array_equal(reqs[q][2], alone[q][0])
        assert done[q]["cycles"] == alone[q][1]["cycles"]


def test_hbm_budget_admission(alone):
    g0 = S.grid_desc(**CASES[0])
    mg = S.Multigrid(g0, S.mg_params(precision=S.PREC_MIXED))
    one = mg.device_bytes()
    mg.close()
    # room for about one 32^3 hierarchy: requests queue behind the budget
    eng = S.Serve(_params(hbm_budget_bytes=int(one * 1.6)))
    reqs = {q: _request(CASES[0], 10) for q in range(3)}
    big = S.grid_desc(n=(128, 128, 128), mesh="UUU", domain="NNN")
    big_rhs, big_lhs = random_rhs(big, 3), S.padded_field(big)
    for q, r in reqs.items():
        eng.submit(q, *r)
    eng.submit(99, big, big_rhs, big_lhs)
    done = {d["id"]: d for d in eng.run()}
    st = eng.stats()
    eng.close()
    assert st["max_active"] == 1
    assert st["bytes_allocated"] <= int(one * 1.6)
    assert done[99]["status"] == S.BUDGET
    for q in range(3):
        assert done[q]["status"] == S.OK
        assert np.array_equal(reqs[q][2], alone[0][0])


def test_autotuned_schedule_gives_same_results(alone):
    reqs = {q: _request(gk, 10 + q) for q, gk in enumerate(CASES)}
    done, _ = _serve(reqs, tune=CASES[:3])
    for q in range(len(CASES)):
        assert done[q]["cycles"] == alone[q][1]["cycles"]
        assert np.array_equal(reqs[q][2], alone[q][0])
    # a hand-picked schedule far from the default
    reqs = {q: _request(gk, 10 + q) for q, gk in enumerate(CASES)}
    done, _ = _serve(reqs, params=_params(cells_per_item=64, threads=64, blocks_per_sm=1))
    for q in range(len(CASES)):
        assert np.array_equal(reqs[q][2], alone[q][0])


def test_nan_request_does_not_disturb_the_mix(alone):
    reqs = {q: _request(gk, 10 + q) for q, gk in enumerate(CASES[:2])}
    g, rhs, lhs = _request(CASES[2], 7)
    rhs[5, 5, 5] = np.nan
    reqs[50] = (g, rhs, lhs)
    done, _ = _serve(reqs)
    assert done[50]["status"] == S.NAN and done[50]["cycles"] == 1
    for q in range(2):
        assert done[q]["status"] == S.OK
        assert np.array_equal(reqs[q][2], alone[q][0])


def test_bad_arguments():
    with pytest.raises(S.SarasError):
        S.Serve(_params(max_cases=0))
    eng = S.Serve(_params())
    shallow = S.grid_desc(n=(2, 2, 2), mesh="UUU", domain="NNN")
    with pytest.raises(S.SarasError):
        eng.submit(1, shallow, S.padded_field(shallow), S.padded_field(shallow))
    g, rhs, lhs = _request(CASES[0], 1)
    eng.submit(2, g, rhs, lhs)
    with pytest.raises(S.SarasError):  # autotune wants an idle engine
        eng.autotune([g])
    eng.close()


def test_cycle_cap_reports_not_converged(alone):
    """A request that reaches the engine's outer-iteration cap above its
    tolerance returns NOT_CONVERGED with its residual; the others in the
    same batch finish as they would alone."""
    reqs = {q: _request(gk, 10 + q) for q, gk in enumerate(CASES[:2])}
    done, _ = _serve(reqs, params=_params(max_cycles=1))
    for q in range(2):
        assert done[q]["status"] == S.NOT_CONVERGED and done[q]["cycles"] == 1
        assert done[q]["residual"] > TOL
    # with room for every outer iteration the same requests converge, bit for
    # bit as alone
    reqs = {q: _request(gk, 10 + q) for q, gk in enumerate(CASES[:2])}
    done, _ = _serve(reqs)
    for q in range(2):
        assert done[q]["status"] == S.OK
        assert np.array_equal(reqs[q][2], alone[q][0])
