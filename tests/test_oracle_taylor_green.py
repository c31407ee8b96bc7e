"""A known answer for the whole time step of the oracle: the planar
Taylor-Green vortex.

The reference's initial condition 1 (lib/initial/taylorGreen.cc:57-71, the
PLANAR branch) sets u = sin(kx) cos(kz), w = -cos(kx) sin(kz), k = 2 pi / L.
On a domain periodic in x and z this is an exact solution of the
incompressible Navier-Stokes equations: the convection term
(k/2) (sin 2kx, sin 2kz) is balanced by the gradient of
p = (cos 2kx + cos 2kz) / 4, so the velocity decays as exp(-2 nu k^2 t) and
the pressure as exp(-4 nu k^2 t).  Every part of lsRK3_d2 / eulerCN_d2::
timeAdvance takes part: the non-linear term, the Crank-Nicolson diffusion
sweeps, the pressure-correction multigrid solve, the divergence and the
pressure gradient.

Bars, at t = 0.02 with nu = 1e-2 from P = 0 (20 steps of dt = 1e-3; 80 of
2.5e-4 for eulerCN, first order in time, whose time error would otherwise
show in the pressure at 64 cells):
* dScheme 1, with each non-linear form and both integrators: the deviation
  of the velocity, and of the pressure up to a constant, falls by a factor
  between 3.5 and 4.5 per halving of h from 16 to 64 cells a side (second
  order);
* the hybrid upwind form agrees with the central form to rounding where the
  cell Peclet number u h / nu is below the limit (64 cells: 1.56 < 2), and is
  far worse above it (16 cells: 6.25), where its deviation falls at first
  order (16 to 32 cells, both above the limit);
* the 3-D step of a y-independent field repeats the planar step;
* with both periodic axes tanh-stretched the velocity still converges at
  second order;
* dScheme 2: the reference uses its second-order forms on the first and last
  core cell of an axis whatever the axis's periodicity (derivative.cc:83-87
  and 108-113: xfr and xlr name the first and last rank).  On a periodic axis
  the divergence then no longer sums to zero, so the pressure equation's
  right-hand side is not compatible with the singular periodic operator and
  every solve stops at the V-cycle count.  The deviation still falls by more
  than 4 per halving.
"""
import math

import numpy as np
import pytest

import pyoracle as O
import saras_gb300 as S
from test_oracle_stencils import params

NU, DT, STEPS = 1e-2, 1e-3, 20
K = 2 * math.pi
VC_COUNT = 60


def setup(n, integration=2, nl_scheme=1, pad=1, planar=True, sub=1, mesh="UUU", beta=1.0):
    """Grid, parameters and the Taylor-Green start.  `sub` divides the time
    step (the caller multiplies the step count); `mesh` and `beta` stretch
    the x and z axes."""
    b = (beta, 1.0, beta)
    if planar:
        g = S.grid_desc(n=(n, 1, n), mesh=mesh, beta=b, domain="PNP", dims=2, pad=pad)
    else:
        g = S.grid_desc(n=(n, 4, n), mesh=mesh, beta=b, domain="PPP", pad=pad)
    prm = params(nl_scheme=nl_scheme, integration=integration)
    prm.nu, prm.dt = NU, DT / sub
    per = S.field_bc([S.FBC_NEUMANN] * 6, [0.0] * 6)
    prm.bc_vx = prm.bc_vy = prm.bc_vz = prm.bc_p = prm.bc_t = per
    prm.mg = S.mg_params(vc_count=VC_COUNT, vc_tolerance=1e-10, pre_smooth=3, post_smooth=6, mg_tolerance=1e-12)
    f = {k: S.padded_field(g) for k in ("vx", "vy", "vz", "p", "t", "pp")}
    x, z = centres(g)
    f["vx"][...] = np.sin(K * x) * np.cos(K * z)
    f["vz"][...] = -np.cos(K * x) * np.sin(K * z)
    return g, prm, f


def centres(g):
    """Cell-centre coordinates along x and z, ghosts included."""
    return O.field_metrics(g, 0)[0][:, None, None], O.field_metrics(g, 2)[0][None, None, :]


def deviations(f, g, planar=True):
    """Deviations of u, w and p (p up to its mean) from the exact solution at
    t = STEPS * DT over the core."""
    pad = g.pad
    x, z = centres(g)
    t = STEPS * DT
    du = math.exp(-2 * NU * K * K * t)
    dp = math.exp(-4 * NU * K * K * t)
    ys = slice(1, 2) if planar else slice(pad, -pad)
    core = (slice(pad, -pad), ys, slice(pad, -pad))
    eu = np.abs(f["vx"] - np.sin(K * x) * np.cos(K * z) * du)[core].max()
    ew = np.abs(f["vz"] + np.cos(K * x) * np.sin(K * z) * du)[core].max()
    pd = (f["p"] - 0.25 * (np.cos(2 * K * x) + np.cos(2 * K * z)) * dp)[core]
    ep = np.abs(pd - pd.mean()).max()
    return eu, ew, ep


def taylor_green(n, integration=2, nl_scheme=1, pad=1, planar=True, sub=1, mesh="UUU", beta=1.0):
    """Runs the oracle from the Taylor-Green start to t = STEPS * DT; returns
    the deviations of u, w and p, the fields and the V-cycle count."""
    g, prm, f = setup(n, integration, nl_scheme, pad, planar, sub, mesh, beta)
    r = O.rk3_run(g, prm, f["vx"], f["vy"], f["vz"], f["p"], f["t"], f["pp"], STEPS * sub)
    assert r.status == 0
    eu, ew, ep = deviations(f, g, planar)
    return eu, ew, ep, f, r.mg_cycles


def ratios(errs):
    return [a / b for a, b in zip(errs, errs[1:])]


@pytest.mark.parametrize("integration,nl_scheme", [(2, 1), (2, 3), (1, 1)], ids=["rk3", "rk3_morinishi", "euler_cn"])
def test_taylor_green_second_order(integration, nl_scheme):
    sub = 4 if integration == 1 else 1
    runs = [taylor_green(n, integration, nl_scheme, sub=sub) for n in (16, 32, 64)]
    for q, name in enumerate(("u", "w", "p")):
        errs = [r[q] for r in runs]
        for ratio in ratios(errs):
            assert 3.5 < ratio < 4.5, (name, errs)
    # the velocity after 20 steps is within 2e-5 of the exact decay at 64^2
    assert runs[-1][0] < 2e-5 and runs[-1][1] < 2e-5
    # the x-z symmetry of the vortex survives the step
    assert abs(runs[-1][0] - runs[-1][1]) <= 1e-12
    # each pressure solve converges (about six V-cycles)
    assert all(r[4] < 10 * 3 * STEPS * sub for r in runs)


def test_taylor_green_hybrid_upwind_follows_peclet_limit():
    """Cell Peclet number 1 * h / nu against the limit 2 of params()."""
    ec, _, _, fc, _ = taylor_green(64, nl_scheme=1)
    eu, _, _, fu, _ = taylor_green(64, nl_scheme=2)
    scale = np.abs(fc["vx"]).max()
    assert np.abs(fu["vx"] - fc["vx"]).max() <= 1e-12 * scale
    assert abs(eu - ec) <= 1e-10
    c16 = taylor_green(16, nl_scheme=1)[0]
    u16 = taylor_green(16, nl_scheme=2)[0]
    assert u16 > 5 * c16
    # above the limit at 16 and 32 cells (Peclet 6.25 and 3.1) the upwind
    # term is first order: the deviation halves with h
    u32 = taylor_green(32, nl_scheme=2)[0]
    assert 1.8 < u16 / u32 < 2.5, (u16, u32)


def test_taylor_green_stretched_periodic_axes():
    """Both periodic axes tanh-stretched (double-sided, beta 1.2), as the
    512^3 configuration's are: the velocity's deviation still falls at
    second order.  The stretched divergence is not orthogonal to the
    operator's left null vector, so the pressure solves stop at the V-cycle
    count there."""
    runs = [taylor_green(n, mesh="DUD", beta=1.2) for n in (16, 32, 64)]
    for q in (0, 1):
        errs = [r[q] for r in runs]
        for a, b in zip(errs, errs[1:]):
            assert 3.5 < a / b < 4.5, errs
    assert runs[-1][0] < 2e-3


def test_taylor_green_3d_repeats_planar():
    for n in (16, 32):
        a = taylor_green(n)
        b = taylor_green(n, planar=False)
        for q in range(3):
            assert abs(a[q] - b[q]) <= 1e-9 * a[q], (n, q, a[q], b[q])


def test_taylor_green_dscheme2_periodic_end_cells():
    # the end-cell forms: the first derivative of a periodic line does not
    # sum to zero with dScheme 2, it does with dScheme 1
    for pad, nonzero in ((1, False), (2, True)):
        g = S.grid_desc(n=(16, 4, 16), domain="PPP", pad=pad)
        f = S.padded_field(g)
        x = (np.arange(f.shape[0]) - pad + 0.5) / 16
        f[...] = (np.sin(K * x) + 0.3 * np.cos(2 * K * x))[:, None, None]
        d = O.field_op(g, params(), 1, f, axis=0)
        s = abs(d[pad:-pad, pad, pad].sum())
        assert (s > 1e-3) if nonzero else (s < 1e-12), (pad, s)
    runs = [taylor_green(n, pad=2) for n in (16, 32)]
    # every solve of the 60 stops at the V-cycle count
    assert all(r[4] == VC_COUNT * 3 * STEPS for r in runs)
    for q in range(3):
        assert runs[0][q] / runs[1][q] > 4.0, (q, runs[0][q], runs[1][q])
