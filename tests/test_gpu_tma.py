"""The TMA-staged FP32 colour sweep (large 3-D levels of the MIXED form).

Bars: bit-identical to the batched item kernels of the serving engine, which
sweep cell by cell with the same arithmetic (so the MIXED solve of a level
large enough for the TMA path equals the served solve bit for bit,
periodic axes included), and the converged MIXED solution agrees with the
oracle's FP64 solve to 1e-9 relative (constant component removed) once both
reach 1e-11.
"""
import numpy as np
import pytest

import pyoracle as O
import saras_gb300 as S
from helpers import core, demean, random_rhs

pytestmark = pytest.mark.gpu

MG = dict(mg_tolerance=1e-9, pre_smooth=3, post_smooth=6)
GRIDS = [
    ("128c_uud", dict(n=(128, 128, 128), mesh="UUD", beta=(1, 1, 1.2), domain="NNN")),
    ("128x128x64_ppn", dict(n=(128, 128, 64), length=(1.0, 1.0, 0.5), mesh="UUD", beta=(1, 1, 1.1),
                            domain="PPN")),
]


@pytest.mark.parametrize("name,gk", GRIDS, ids=[g[0] for g in GRIDS])
def test_tma_sweep_matches_cellwise_kernels(name, gk):
    g = S.grid_desc(**gk)
    rhs = random_rhs(g, 21)
    single = S.padded_field(g)
    mg = S.Multigrid(g, S.mg_params(precision=S.PREC_MIXED, vc_count=100, vc_tolerance=1e-8, **MG))
    assert mg.mg_solve(single, rhs) == S.OK
    cycles = mg.cycles
    mg.close()
    eng = S.Serve(S.serve_params(tolerance=1e-8, max_cycles=100, max_cases=4, **MG))
    served = S.padded_field(g)
    eng.submit(1, g, rhs, served)
    done = eng.run()
    eng.close()
    assert done[0]["status"] == S.OK and done[0]["cycles"] == cycles
    assert np.array_equal(served, single)


def test_tma_mixed_solve_matches_oracle():
    g = S.grid_desc(**GRIDS[0][1])
    rhs = random_rhs(g, 22)
    mix = S.padded_field(g)
    mg = S.Multigrid(g, S.mg_params(precision=S.PREC_MIXED, vc_count=100, vc_tolerance=1e-11, **MG))
    assert mg.mg_solve(mix, rhs) == S.OK and mg.history[-1] < 1e-11
    mg.close()
    orc = S.padded_field(g)
    r = O.mg_solve(g, S.mg_params(vc_count=100, vc_tolerance=1e-12, **MG), orc, rhs)
    assert r.history[-1] < 1e-12
    a, b = demean(core(mix, g)), demean(core(orc, g))
    assert np.abs(a - b).max() <= 1e-9 * np.abs(b).max()
