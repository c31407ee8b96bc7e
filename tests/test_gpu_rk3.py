"""GPU time-step parity: saras_rk3_step (through the C ABI) against the
oracle's restatement of lsRK3_d3/lsRK3_d2::timeAdvance (lib/timestep/
lsRK3_d3.cc:190-305) and eulerCN_d3/_d2::timeAdvance (eulerCN_d3.cc:88-268)
with the FP64_EXACT pressure solve.  Bar: every field (velocity, pressure,
temperature, pressure correction, ghost layers included) bit-for-bit after
three time steps; for the planar case the j = 0 plane, the only plane the 2D
reference computes.  With dScheme 2 (two ghost layers) the pressure
correction is compared over its core and first ghost layer (what mgSolve
writes) and the pressure without the second ghost layer of wall axes (never
read by a stencil; the reference adds the correction's unwritten outer layer
to it).  With the MIXED pressure solve the fields agree with the oracle to
1e-5 relative.
"""
import numpy as np
import pytest

import pyoracle as O
import saras_gb300 as S

pytestmark = pytest.mark.gpu


def rbc_params(g, ra=1e5, pr=1.0, dt=2e-3, mg_precision=S.PREC_FP64_EXACT, with_scalar=1, vc_tol=1e-6,
               nl_scheme=1, integration=2, pe_limit=2.0, up_param=0.8):
    nu, ka, fb = S.rbc_coefficients(2, ra, pr)
    p = S.Rk3Params()
    p.nu, p.kappa, p.dt = nu, ka, dt
    p.cn_tolerance = 1e-12
    p.max_iterations = 0
    for d, gv in enumerate((0.0, 0.0, -fb)):
        p.g_terms[d] = gv if with_scalar else 0.0
    p.with_scalar = with_scalar
    p.nl_scheme = nl_scheme
    p.integration = integration
    p.pe_limit, p.up_param = pe_limit, up_param
    dirich0 = S.field_bc([S.FBC_DIRICHLET] * 6, [0.0] * 6)
    p.bc_vx = dirich0
    p.bc_vy = dirich0
    p.bc_vz = dirich0
    p.bc_t = S.field_bc([S.FBC_NEUMANN] * 4 + [S.FBC_DIRICHLET] * 2, [0, 0, 0, 0, 1.0, 0.0])
    p.bc_p = S.field_bc([S.FBC_NEUMANN] * 6, [0.0] * 6)
    # the reference's Multigrid defaults (input/parameters.yaml): the pressure
    # RHS of a collocated step is not exactly compatible with the singular
    # operator, so the coarsest solve must stop at its loose tolerance
    p.mg = S.mg_params(vc_count=20, vc_tolerance=vc_tol, pre_smooth=3, post_smooth=6, mg_tolerance=1e-2,
                       precision=mg_precision)
    return p


def initial_fields(g, seed, vel_amp=0.0):
    """Rayleigh-Benard start (scalar_d3 set-up): u = 0, P = 1, T = conductive
    profile plus seeded noise of amplitude 1e-3.  A random velocity is only
    used on all-wall boxes, where its divergence stays compatible enough for
    the pressure solve."""
    rng = np.random.default_rng(seed)
    f = {k: S.padded_field(g) for k in ("vx", "vy", "vz", "p", "t", "pp")}
    if vel_amp:
        for k in ("vx", "vy", "vz"):
            f[k][...] = rng.uniform(-vel_amp, vel_amp, f[k].shape)
    z = np.linspace(0, 1, f["t"].shape[2])
    f["t"][...] = (1.0 - z)[None, None, :] + rng.uniform(-5e-4, 5e-4, f["t"].shape)
    f["p"][...] = 1.0
    return f


def run_pair(gk, steps=3, vel_amp=0.0, **pk):
    g = S.grid_desc(**gk)
    prm = rbc_params(g, **pk)
    f0 = initial_fields(g, 4, vel_amp)
    gpu = {k: v.copy() for k, v in f0.items()}
    orc = {k: v.copy() for k, v in f0.items()}
    rk = S.RK3(g, prm)
    rk.upload(gpu["vx"], gpu["vy"], gpu["vz"], gpu["p"], gpu["t"], gpu["pp"])
    mgc, cni = rk.step(steps)
    rk.download(gpu["vx"], gpu["vy"], gpu["vz"], gpu["p"], gpu["t"], gpu["pp"])
    rk.close()
    r = O.rk3_run(g, prm, orc["vx"], orc["vy"], orc["vz"], orc["p"], orc["t"], orc["pp"], steps)
    assert r.status == 0
    return g, gpu, orc, (mgc, cni), (r.mg_cycles, r.cn_iters)


@pytest.mark.parametrize("gk,amp", [
    (dict(n=(16, 16, 32), mesh="UUD", beta=(1, 1, 1.5), domain="PPN"), 0.0),
    (dict(n=(16, 16, 16), mesh="DDD", beta=(1.1, 1.2, 1.3), domain="NNN"), 0.05),
], ids=["rbc_ppn_uud", "box_nnn_ddd"])
def test_rk3_bitwise(gk, amp):
    g, gpu, orc, gc, oc = run_pair(gk, vel_amp=amp)
    assert gc == oc, (gc, oc)
    for k in ("vx", "vy", "vz", "p", "t", "pp"):
        assert np.array_equal(gpu[k], orc[k]), (k, np.abs(gpu[k] - orc[k]).max())


def test_rk3_hydro_bitwise():
    gk = dict(n=(16, 16, 16), mesh="UUD", beta=(1, 1, 1.2), domain="PNN")
    g, gpu, orc, gc, oc = run_pair(gk, with_scalar=0)
    for k in ("vx", "vy", "vz", "p", "pp"):
        assert np.array_equal(gpu[k], orc[k]), k


def test_rk3_planar_bitwise():
    gk = dict(n=(32, 1, 32), mesh="UUD", beta=(1, 1, 1.3), domain="PNN", dims=2)
    g, gpu, orc, gc, oc = run_pair(gk)
    for k in ("vx", "vz", "p", "t", "pp"):
        assert np.array_equal(gpu[k][:, 1, :], orc[k][:, 1, :]), k


def test_rk3_mixed_pressure_solve():
    """Same step with the MIXED pressure solve: the pressure solve plateaus
    (incompatible RHS) after the same cycles, so fields agree to 1e-5."""
    gk = dict(n=(16, 16, 32), mesh="UUD", beta=(1, 1, 1.5), domain="PPN")
    g = S.grid_desc(**gk)
    prm_m = rbc_params(g, mg_precision=S.PREC_MIXED)
    prm_o = rbc_params(g)
    f0 = initial_fields(g, 4)
    gpu = {k: v.copy() for k, v in f0.items()}
    orc = {k: v.copy() for k, v in f0.items()}
    rk = S.RK3(g, prm_m)
    rk.upload(gpu["vx"], gpu["vy"], gpu["vz"], gpu["p"], gpu["t"], gpu["pp"])
    rk.step(2)
    rk.download(gpu["vx"], gpu["vy"], gpu["vz"], gpu["p"], gpu["t"], gpu["pp"])
    O.rk3_run(g, prm_o, orc["vx"], orc["vy"], orc["vz"], orc["p"], orc["t"], orc["pp"], 2)
    for k in ("vx", "vy", "vz", "t"):
        a, b = gpu[k][1:-1, 1:-1, 1:-1], orc[k][1:-1, 1:-1, 1:-1]
        assert np.abs(a - b).max() <= 1e-5 * np.abs(b).max(), k


@pytest.mark.parametrize("gk,amp", [
    (dict(n=(16, 16, 32), mesh="UUD", beta=(1, 1, 1.5), domain="PPN"), 0.0),
    (dict(n=(16, 16, 16), mesh="DDD", beta=(1.1, 1.2, 1.3), domain="NNN"), 0.05),
    (dict(n=(32, 1, 32), mesh="UUD", beta=(1, 1, 1.3), domain="PNN", dims=2), 0.05),
], ids=["rbc_ppn_uud", "box_nnn_ddd", "planar_pnn"])
def test_rk3_morinishi_bitwise(gk, amp):
    """Non-Linear Term 3 (Morinishi's skew-symmetric form, second-order
    branch of vfield/sfield::morinishiNLin) against the oracle, bit for bit."""
    g, gpu, orc, gc, oc = run_pair(gk, vel_amp=amp, nl_scheme=3)
    assert gc == oc, (gc, oc)
    planar = gk.get("dims") == 2
    for k in (("vx", "vz", "p", "t", "pp") if planar else ("vx", "vy", "vz", "p", "t", "pp")):
        a, b = (gpu[k][:, 1, :], orc[k][:, 1, :]) if planar else (gpu[k], orc[k])
        assert np.array_equal(a, b), (k, np.abs(a - b).max())
    # the scheme changes the step: the convection term differs from nlScheme 1
    g1, gpu1, _, _, _ = run_pair(gk, vel_amp=amp, nl_scheme=1)
    assert not np.array_equal(gpu1["vx"], gpu["vx"])


def _mask(g, key, shape):
    """Cells compared for field `key`: everything, except for dScheme 2 the
    pressure's second ghost layer on wall axes and the pressure
    correction's second ghost layer."""
    m = np.ones(shape, bool)
    if g.pad < 2 or key not in ("p", "pp"):
        return m
    for a in range(3):
        if g.dims == 2 and a == 1:
            continue
        if key == "pp" or not g.periodic[a]:
            idx = [slice(None)] * 3
            idx[a] = [0, shape[a] - 1]
            m[tuple(idx)] = False
    return m


def assert_fields_equal(g, gpu, orc, with_scalar=1):
    planar = g.dims == 2
    keys = ["vx", "vz", "p", "pp"] + (["t"] if with_scalar else [])
    if not planar:
        keys.append("vy")
    for k in keys:
        a, b = gpu[k], orc[k]
        m = _mask(g, k, a.shape)
        if planar:
            a, b, m = a[:, 1, :], b[:, 1, :], m[:, 1, :]
        assert np.array_equal(a[m], b[m]), (k, np.abs(a[m] - b[m]).max())


SCHEME_GRIDS = [
    (dict(n=(16, 16, 32), mesh="UUD", beta=(1, 1, 1.5), domain="PPN"), 0.0),
    (dict(n=(16, 16, 16), mesh="DDD", beta=(1.1, 1.2, 1.3), domain="NNN"), 0.05),
    (dict(n=(32, 1, 32), mesh="UUD", beta=(1, 1, 1.3), domain="PNN", dims=2), 0.05),
]
SCHEME_IDS = ["rbc_ppn_uud", "box_nnn_ddd", "planar_pnn"]


@pytest.mark.parametrize("gk,amp", SCHEME_GRIDS, ids=SCHEME_IDS)
@pytest.mark.parametrize("nl", [1, 2, 3])
def test_dscheme2_bitwise(gk, amp, nl):
    """Differentiation Scheme 2 (pad 2, fourth-order interior stencils) with
    each non-linear scheme, RK3.  The PPN grid has Nz != Ny, which exercises
    Morinishi's last-z-point test against the y extent."""
    g, gpu, orc, gc, oc = run_pair(dict(gk, pad=2), vel_amp=amp, nl_scheme=nl, pe_limit=0.5)
    assert gc == oc, (gc, oc)
    assert_fields_equal(g, gpu, orc)


@pytest.mark.parametrize("pad", [1, 2])
def test_upwind_bitwise(pad):
    """Hybrid upwinding (nlScheme 2) with a Peclet limit that splits the
    cells between the central and the biased stencils."""
    gk = dict(n=(16, 16, 16), mesh="DDD", beta=(1.1, 1.2, 1.3), domain="NNN", pad=pad)
    g, gpu, orc, gc, oc = run_pair(gk, vel_amp=0.05, nl_scheme=2, pe_limit=0.5, up_param=0.3)
    assert gc == oc
    assert_fields_equal(g, gpu, orc)
    # the biased stencils change the step
    g2, gpu2, _, _, _ = run_pair(gk, vel_amp=0.05, nl_scheme=2, pe_limit=1e9, up_param=0.3)
    assert not np.array_equal(gpu2["vx"], gpu["vx"])


@pytest.mark.parametrize("gk,amp", SCHEME_GRIDS, ids=SCHEME_IDS)
@pytest.mark.parametrize("pad,nl", [(1, 1), (1, 3), (2, 3), (2, 2)])
def test_euler_cn_bitwise(gk, amp, pad, nl):
    """Integration Scheme 1 (eulerCN) against the oracle, bit for bit."""
    g, gpu, orc, gc, oc = run_pair(dict(gk, pad=pad), vel_amp=amp, nl_scheme=nl, integration=1, pe_limit=0.5)
    assert gc == oc, (gc, oc)
    assert_fields_equal(g, gpu, orc)


def test_euler_cn_hydro_bitwise():
    gk = dict(n=(16, 16, 16), mesh="UUD", beta=(1, 1, 1.2), domain="PNN", pad=2)
    g, gpu, orc, gc, oc = run_pair(gk, with_scalar=0, integration=1, nl_scheme=3)
    assert_fields_equal(g, gpu, orc, with_scalar=0)
