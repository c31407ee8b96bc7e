"""The TMA-staged FP32 colour sweep (large 3-D levels of the MIXED form).

Bars: bit-identical to the batched item kernels of the serving engine, which
sweep cell by cell with the same arithmetic (so the MIXED solve of a level
large enough for the TMA path equals the served solve bit for bit,
periodic axes included, and so does a solve whose finest level takes the
fused red-black iteration, which recomputes the first colour on halo rows
and planes instead of reading it back from HBM), and the converged MIXED
solution agrees with the oracle's FP64 solve to 1e-9 relative (constant
component removed) once both reach 1e-11.
"""
import numpy as np
import pytest

import pyoracle as O
import saras_gb300 as S
from helpers import core, demean, random_rhs

pytestmark = pytest.mark.gpu

MG = dict(mg_tolerance=1e-9, pre_smooth=3, post_smooth=6)
# the last three grids' finest levels (4M cells, rows of 256 or 128 cells,
# cells of equal extent on all axes: red-black point smoothing converges
# slowly on anisotropic cells)
# take the fused red-black iteration for pairs of smoothing iterations: with
# 3 / 6 sweeps one pair plus a colour-sweep iteration before the descent and
# three pairs after it; with 2 / 2 pairs only
GRIDS = [
    ("128c_uud", dict(n=(128, 128, 128), mesh="UUD", beta=(1, 1, 1.2), domain="NNN"), MG),
    ("128x128x64_ppn", dict(n=(128, 128, 64), length=(1.0, 1.0, 0.5), mesh="UUD", beta=(1, 1, 1.1),
                            domain="PPN"), MG),
    ("fused_128x128x256_uud", dict(n=(128, 128, 256), length=(1.0, 1.0, 2.0), mesh="UUD", beta=(1, 1, 1.2),
                                   domain="NNN"), MG),
    ("fused_256x128x128_ppn", dict(n=(256, 128, 128), length=(2.0, 1.0, 1.0), mesh="UUU", domain="PPN"), MG),
    ("fused_128x128x256_uud_2x2", dict(n=(128, 128, 256), length=(1.0, 1.0, 2.0), mesh="UUD", beta=(1, 1, 1.2),
                                       domain="NNN"), dict(mg_tolerance=1e-9, pre_smooth=2, post_smooth=2)),
    # every axis periodic: the fused iteration's wraps in x, y and z (rows
    # read across the row's ends) and the single-block bottom on a periodic box
    ("fused_128x128x256_ppp", dict(n=(128, 128, 256), length=(1.0, 1.0, 2.0), mesh="UUU", domain="PPP"), MG),
    # even smoothing counts: the finest level is stored row-split (each row's
    # red cells, then its black cells) for the fused iteration
    ("rowsplit_128x128x256_ppp_2x2", dict(n=(128, 128, 256), length=(1.0, 1.0, 2.0), mesh="UUU", domain="PPP"),
     dict(mg_tolerance=1e-9, pre_smooth=2, post_smooth=2)),
    # rows of 512 cells: the fused iteration and the residual-restriction
    # load and store rows as two 256-cell halves (4-D tensor maps) on 4-row
    # tiles; the plain layout whatever the smoothing counts
    ("fused_64x128x512_uud", dict(n=(64, 128, 512), length=(0.125, 0.25, 1.0), mesh="UUD", beta=(1, 1, 1.2),
                                  domain="NNN"), MG),
    ("fused_64x128x512_ppp_2x2", dict(n=(64, 128, 512), length=(0.125, 0.25, 1.0), mesh="UUU", domain="PPP"),
     dict(mg_tolerance=1e-9, pre_smooth=2, post_smooth=2)),
]
DDD = dict(n=(128, 128, 256), length=(1.0, 1.0, 2.0), mesh="DDD", beta=(1.05, 1.05, 1.1), domain="NNN")


@pytest.mark.parametrize("name,gk,mgk", GRIDS, ids=[g[0] for g in GRIDS])
def test_tma_sweep_matches_cellwise_kernels(name, gk, mgk):
    g = S.grid_desc(**gk)
    rhs = random_rhs(g, 21)
    single = S.padded_field(g)
    mg = S.Multigrid(g, S.mg_params(precision=S.PREC_MIXED, vc_count=100, vc_tolerance=1e-8, **mgk))
    assert mg.mg_solve(single, rhs) == S.OK
    cycles = mg.cycles
    mg.close()
    eng = S.Serve(S.serve_params(tolerance=1e-8, max_cycles=100, max_cases=4, **mgk))
    served = S.padded_field(g)
    eng.submit(1, g, rhs, served)
    done = eng.run()
    eng.close()
    assert done[0]["status"] == S.OK and done[0]["cycles"] == cycles
    assert np.array_equal(served, single)


# the fused iteration's wall mirrors are checked against the oracle with
# Dirichlet (odd) and Neumann (even) walls
ORACLE_CASES = [
    ("128c_uud", GRIDS[0][1], MG),
    ("fused_128x128x256_uud", GRIDS[2][1], MG),
    ("fused_ddd_dirichlet_z", DDD, dict(MG, bc_kind=[0, 0, 0, 0, 1, 1])),
    ("fused_ddd_dirichlet_xy", DDD, dict(MG, bc_kind=[1, 1, 1, 1, 0, 0])),
    # 128^3 reaches 8^3 above a 4^3 coarsest level: the single-block bottom
    # (smoothing, restriction, coarsest solve, prolongation) with Dirichlet
    # walls on every face
    ("bottom_128c_dirichlet", dict(n=(128, 128, 128), mesh="UUD", beta=(1, 1, 1.2), domain="NNN"),
     dict(MG, bc_kind=[1, 1, 1, 1, 1, 1])),
    # the row-split finest level with Dirichlet z walls
    ("rowsplit_dirichlet_z_2x2", GRIDS[4][1], dict(mg_tolerance=1e-9, pre_smooth=2, post_smooth=2,
                                                   bc_kind=[0, 0, 0, 0, 1, 1])),
]


@pytest.mark.parametrize("name,gk,mgk", ORACLE_CASES, ids=[c[0] for c in ORACLE_CASES])
def test_tma_mixed_solve_matches_oracle(name, gk, mgk):
    g = S.grid_desc(**gk)
    rhs = random_rhs(g, 22)
    mix = S.padded_field(g)
    mg = S.Multigrid(g, S.mg_params(precision=S.PREC_MIXED, vc_count=100, vc_tolerance=1e-11, **mgk))
    assert mg.mg_solve(mix, rhs) == S.OK and mg.history[-1] < 1e-11
    mg.close()
    orc = S.padded_field(g)
    # the converged solution does not depend on the smoothing counts: the
    # oracle smooths 3 / 6 to reach 1e-12 within its cycle cap
    r = O.mg_solve(g, S.mg_params(vc_count=100, vc_tolerance=1e-12, **dict(mgk, pre_smooth=3, post_smooth=6)),
                   orc, rhs)
    assert r.history[-1] < 1e-12
    a, b = demean(core(mix, g)), demean(core(orc, g))
    assert np.abs(a - b).max() <= 1e-9 * np.abs(b).max()


@pytest.mark.parametrize("gk", [
    # colour sweeps through the TMA ring (2M cells)
    dict(n=(128, 128, 128), mesh="UUD", beta=(1, 1, 1.2), domain="NNN"),
    # the fused iteration on the row-split layout (4M cells, 2/2 smoothing)
    dict(n=(128, 128, 256), length=(1.0, 1.0, 2.0), mesh="UUD", beta=(1, 1, 1.2), domain="NNN"),
], ids=["tma_colour_128c", "fused_128x128x256"])
def test_bounded_wait_runs_out_and_handle_recovers(gk):
    """A bound of one poll on the TMA sweeps' mbarrier waits makes a wait run
    out in the first V-cycle of a normal MIXED solve: the kernel records the
    error, waits (with the default bound) for the copies it issued and
    returns, and the solve reports TIMEOUT.  With the default bound restored,
    the next solve on the same handle is bit for bit the solve of a fresh
    handle."""
    g = S.grid_desc(**gk)
    rhs = random_rhs(g, 41)
    prm = S.mg_params(precision=S.PREC_MIXED, vc_count=100, vc_tolerance=1e-10, mg_tolerance=1e-6, pre_smooth=2,
                      post_smooth=2, inner_cycles=-16)
    mg = S.Multigrid(g, prm)
    mg.set_wait_limit(1)
    lhs = S.padded_field(g)
    with pytest.raises(S.SarasError) as e:
        mg.mg_solve(lhs, rhs)
    assert e.value.status == S.TIMEOUT
    mg.set_wait_limit(0)
    again = S.padded_field(g)
    assert mg.mg_solve(again, rhs) == S.OK
    hist = mg.history.copy()
    mg.close()
    fresh = S.Multigrid(g, prm)
    ref = S.padded_field(g)
    assert fresh.mg_solve(ref, rhs) == S.OK
    assert np.array_equal(again, ref) and np.array_equal(hist, fresh.history)
    fresh.close()


def test_handles_with_different_rings_interleave():
    """Handles whose large levels use TMA rings of different sizes (rows of
    256 and of 128 cells) solve interleaved: a plan made for one handle
    leaves the other's launches valid, and each solve repeats its bits."""
    ga = S.grid_desc(n=(128, 128, 256), length=(1.0, 1.0, 2.0), mesh="UUD", beta=(1, 1, 1.2), domain="NNN")
    gb = S.grid_desc(n=(128, 128, 128), mesh="UUD", beta=(1, 1, 1.2), domain="NNN")
    prm = S.mg_params(precision=S.PREC_MIXED, vc_count=100, vc_tolerance=1e-8, mg_tolerance=1e-6, pre_smooth=2,
                      post_smooth=2, inner_cycles=-16)
    ra, rb = random_rhs(ga, 51), random_rhs(gb, 52)
    a = S.Multigrid(ga, prm)
    first = S.padded_field(ga)
    assert a.mg_solve(first, ra) == S.OK
    b = S.Multigrid(gb, prm)
    ub = S.padded_field(gb)
    assert b.mg_solve(ub, rb) == S.OK
    again = S.padded_field(ga)
    assert a.mg_solve(again, ra) == S.OK
    assert np.array_equal(first, again)
    a.close()
    b.close()
