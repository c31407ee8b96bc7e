"""The planar Taylor-Green vortex on the GPU: lsRK3_d2 and eulerCN_d2 with the
FP64_EXACT pressure solve on a grid periodic in x and z.  Bar: the fields,
the V-cycle and Jacobi counts equal the oracle's bit for bit (the oracle's
deviation from the exact decay falls at second order,
test_oracle_taylor_green.py), and the velocity is within 2e-5 of the exact
decay at 64 cells a side after 20 steps.
"""
import numpy as np
import pytest

import pyoracle as O
import saras_gb300 as S
from test_oracle_taylor_green import STEPS, deviations, setup

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,integration,nl_scheme", [(64, 2, 1), (32, 2, 3), (32, 1, 1)],
                         ids=["rk3_64", "rk3_morinishi_32", "euler_cn_32"])
def test_taylor_green_bitwise(n, integration, nl_scheme):
    g, prm, f0 = setup(n, integration, nl_scheme)
    gpu = {k: v.copy() for k, v in f0.items()}
    orc = {k: v.copy() for k, v in f0.items()}
    rk = S.RK3(g, prm)
    rk.upload(gpu["vx"], gpu["vy"], gpu["vz"], gpu["p"], gpu["t"], gpu["pp"])
    counts = rk.step(STEPS)
    rk.download(gpu["vx"], gpu["vy"], gpu["vz"], gpu["p"], gpu["t"], gpu["pp"])
    rk.close()
    r = O.rk3_run(g, prm, orc["vx"], orc["vy"], orc["vz"], orc["p"], orc["t"], orc["pp"], STEPS)
    assert r.status == 0
    assert counts == (r.mg_cycles, r.cn_iters), (counts, r.mg_cycles, r.cn_iters)
    core = (slice(1, -1), slice(1, 2), slice(1, -1))
    for k in ("vx", "vz", "p", "pp"):
        assert np.array_equal(gpu[k][core], orc[k][core]), (k, np.abs(gpu[k] - orc[k])[core].max())
    # the periodic ghosts of the x-z plane too
    for k in ("vx", "vz", "p", "pp"):
        assert np.array_equal(gpu[k][:, 1, :], orc[k][:, 1, :]), ("ghosts", k)
    eu, ew, _ = deviations(gpu, g)
    if n == 64:
        assert eu < 2e-5 and ew < 2e-5
