"""A known answer for the time step between walls: decay of a sine mode
under no-slip and fixed-temperature walls, with buoyancy.

On a box periodic in x and y with walls at z = 0 and z = 1, the fields
u = sin(pi z) and T = sin(pi z), with v = w = 0, u = 0 and T = 0 on the
walls, and gravity along -z, solve the Boussinesq equations exactly: u and T
depend on z alone, so convection vanishes; u decays as exp(-nu pi^2 t) and T
as exp(-kappa pi^2 t); the buoyancy Fb T of the w equation is balanced by
the hydrostatic pressure p = -Fb cos(pi z) / pi exp(-kappa pi^2 t), so w
stays zero.  The test runs the Dirichlet ghost writers (dirichlet.cc), the
Crank-Nicolson sweeps against walls, the buoyancy term
(buoyantForce.cc:64-69) and the pressure correction with Neumann pressure
walls, which the all-periodic tests do not reach.

Bars, at t = 0.02 (20 RK3 steps of dt = 1e-3; 80 eulerCN steps of 2.5e-4),
nu = 1e-2, kappa = 2e-2, Fb = 1:
* uniform mesh: the deviations of u and T fall by a factor between 3.5 and
  4.5 per halving of h from 16 to 64 cells (second order), the pressure's
  (up to a constant) by more than 3, and max |w| stays below 1e-8;
* dScheme 2 on the uniform mesh: second order too (its first and last core
  cells take the second-order forms), with about half dScheme 1's
  deviation; max |w| stays below 1e-6;
* a moving top wall (u = 1 there, the lid of the reference's lid-driven
  cavity): u = z + sin(pi z) exp(-nu pi^2 t) is exact, and so is the linear
  Couette profile on the grid, so the deviation equals the fixed wall's to
  rounding, and the top ghost is 2 - u at the last core cell;
* a prescribed heat flux (Neumann temperature walls with value dT/dz = -1,
  neumann.cc): T = 1 - z is a steady state, kept to rounding on a uniform
  mesh with either pad, with the ghosts on the same line;
* tanh-stretched mesh (double-sided, beta 1.3): the reference places the
  ghost coordinates and metrics by copying from the other end of the axis
  (grid.cc:467-477), so the left ghost sits at -z_1 and carries the right
  end's xi_zz.  With the mirrored Dirichlet ghost the second difference at
  the first cell beside a wall then has an O(1) truncation error (the
  xi-stencil assumes the ghost on the smooth tanh map, O(dxi^2) away from
  -z_1).  The error is local: the deviation of u and T still falls by more
  than 2 per halving and is below 3e-4 at 64 cells.
"""
import math

import numpy as np
import pytest

import pyoracle as O
import saras_gb300 as S
from test_oracle_stencils import params

NU, KAPPA, FB, DT, STEPS = 1e-2, 2e-2, 1.0, 1e-3, 20


def wall_decay(nz, mesh="UUU", integration=2, sub=1, pad=1):
    g = S.grid_desc(n=(4, 4, nz), mesh=mesh, beta=(1, 1, 1.3), domain="PPN", pad=pad)
    p = params(integration=integration)
    p.nu, p.kappa, p.dt = NU, KAPPA, DT / sub
    p.with_scalar = 1
    for d, gv in enumerate((0.0, 0.0, -FB)):
        p.g_terms[d] = gv
    p.bc_vx = p.bc_vy = p.bc_vz = S.field_bc([S.FBC_DIRICHLET] * 6, [0.0] * 6)
    p.bc_t = S.field_bc([S.FBC_NEUMANN] * 4 + [S.FBC_DIRICHLET] * 2, [0.0] * 6)
    p.bc_p = S.field_bc([S.FBC_NEUMANN] * 6, [0.0] * 6)
    p.mg = S.mg_params(vc_count=30, vc_tolerance=1e-10, pre_smooth=3, post_smooth=6, mg_tolerance=1e-10)
    f = {k: S.padded_field(g) for k in ("vx", "vy", "vz", "p", "t", "pp")}
    z = O.field_metrics(g, 2)[0][None, None, :]
    f["vx"][...] = np.sin(math.pi * z)
    f["t"][...] = np.sin(math.pi * z)
    r = O.rk3_run(g, p, f["vx"], f["vy"], f["vz"], f["p"], f["t"], f["pp"], STEPS * sub)
    assert r.status == 0
    t = STEPS * DT
    core = (slice(pad, -pad),) * 3
    eu = np.abs(f["vx"] - np.sin(math.pi * z) * math.exp(-NU * math.pi ** 2 * t))[core].max()
    et = np.abs(f["t"] - np.sin(math.pi * z) * math.exp(-KAPPA * math.pi ** 2 * t))[core].max()
    ew = np.abs(f["vz"])[core].max()
    pd = (f["p"] + FB * np.cos(math.pi * z) / math.pi * math.exp(-KAPPA * math.pi ** 2 * t))[core]
    ep = np.abs(pd - pd.mean()).max()
    return eu, et, ew, ep


@pytest.mark.parametrize("integration", [2, 1], ids=["rk3", "euler_cn"])
def test_wall_decay_second_order(integration):
    sub = 4 if integration == 1 else 1
    runs = [wall_decay(nz, integration=integration, sub=sub) for nz in (16, 32, 64)]
    for q, name in ((0, "u"), (1, "T")):
        errs = [r[q] for r in runs]
        for a, b in zip(errs, errs[1:]):
            assert 3.5 < a / b < 4.5, (name, errs)
    pe = [r[3] for r in runs]
    assert pe[0] / pe[1] > 3 and pe[1] / pe[2] > 3, pe
    assert max(r[2] for r in runs) < 1e-8


def test_wall_decay_stretched():
    runs = [wall_decay(nz, mesh="UUD") for nz in (16, 32, 64)]
    for q in (0, 1):
        errs = [r[q] for r in runs]
        assert errs[0] / errs[1] > 2 and errs[1] / errs[2] > 2, errs
        assert errs[2] < 3e-4
    # the first cell beside a wall: O(1) truncation of the second
    # difference of sin(pi z), against O(h^2) inside
    g = S.grid_desc(n=(4, 4, 32), mesh="UUD", beta=(1, 1, 1.3), domain="PPN")
    z = O.field_metrics(g, 2)[0]
    assert z[0] == pytest.approx(-z[1], rel=1e-12)
    prm = params()
    prm.bc_vx = prm.bc_vy = prm.bc_vz = S.field_bc([S.FBC_DIRICHLET] * 6, [0.0] * 6)
    f = S.padded_field(g)
    f[...] = np.sin(math.pi * z)[None, None, :]
    d2 = O.field_op(g, prm, 2, f, axis=2)[2, 2, 1:-1]
    err = np.abs(d2 + math.pi ** 2 * np.sin(math.pi * z[1:-1]))
    assert err[0] > 1.0 and err[-1] > 1.0
    assert err[2:-2].max() < 0.1


def test_wall_decay_dscheme2():
    runs = [wall_decay(nz, pad=2) for nz in (16, 32, 64)]
    for q in (0, 1):
        errs = [r[q] for r in runs]
        for a, b in zip(errs, errs[1:]):
            assert 3.5 < a / b < 4.5, errs
    assert runs[1][0] < 0.6 * wall_decay(32)[0]
    assert max(r[2] for r in runs) < 1e-6


def couette(nz, lid, pad=1):
    """u = lid * z + sin(pi z) under walls at rest below and moving at `lid`
    above, no scalar; returns the deviation from the exact decay and u."""
    g = S.grid_desc(n=(4, 4, nz), domain="PPN", pad=pad)
    p = params()
    p.nu, p.dt = NU, DT
    p.bc_vx = S.field_bc([S.FBC_DIRICHLET] * 6, [0.0] * 5 + [lid])
    p.bc_vy = p.bc_vz = S.field_bc([S.FBC_DIRICHLET] * 6, [0.0] * 6)
    p.bc_p = S.field_bc([S.FBC_NEUMANN] * 6, [0.0] * 6)
    p.mg = S.mg_params(vc_count=30, vc_tolerance=1e-10, pre_smooth=3, post_smooth=6, mg_tolerance=1e-10)
    f = {k: S.padded_field(g) for k in ("vx", "vy", "vz", "p", "t", "pp")}
    z = O.field_metrics(g, 2)[0][None, None, :]
    f["vx"][...] = lid * z + np.sin(math.pi * z)
    r = O.rk3_run(g, p, f["vx"], f["vy"], f["vz"], f["p"], f["t"], f["pp"], STEPS)
    assert r.status == 0
    exact = lid * z + np.sin(math.pi * z) * math.exp(-NU * math.pi ** 2 * STEPS * DT)
    core = (slice(pad, -pad),) * 3
    return np.abs(f["vx"] - exact)[core].max(), f["vx"]


@pytest.mark.parametrize("pad", [1, 2])
def test_moving_wall(pad):
    errs = []
    for nz in (16, 32):
        e1, u = couette(nz, 1.0, pad)
        e0, _ = couette(nz, 0.0, pad)
        assert abs(e1 - e0) < 1e-12, (e1, e0)
        errs.append(e1)
        if pad == 1:
            assert np.abs(u[:, :, -1] + u[:, :, -2] - 2.0).max() < 1e-14
            assert np.abs(u[:, :, 0] + u[:, :, 1]).max() < 1e-14
    assert 3.5 < errs[0] / errs[1] < 4.5, errs


@pytest.mark.parametrize("pad", [1, 2])
def test_heat_flux_walls_keep_linear_profile(pad):
    n = 16
    g = S.grid_desc(n=(4, 4, n), domain="PPN", pad=pad)
    p = params()
    p.nu, p.kappa, p.dt = NU, KAPPA, DT
    p.with_scalar = 1
    p.bc_vx = p.bc_vy = p.bc_vz = S.field_bc([S.FBC_DIRICHLET] * 6, [0.0] * 6)
    p.bc_t = S.field_bc([S.FBC_NEUMANN] * 6, [0.0] * 4 + [-1.0, -1.0])
    p.bc_p = S.field_bc([S.FBC_NEUMANN] * 6, [0.0] * 6)
    p.mg = S.mg_params(vc_count=30, vc_tolerance=1e-10, pre_smooth=3, post_smooth=6, mg_tolerance=1e-10)
    f = {k: S.padded_field(g) for k in ("vx", "vy", "vz", "p", "t", "pp")}
    z = O.field_metrics(g, 2)[0][None, None, :]
    f["t"][...] = 1.0 - z
    r = O.rk3_run(g, p, f["vx"], f["vy"], f["vz"], f["p"], f["t"], f["pp"], 10)
    assert r.status == 0
    core = (slice(pad, -pad),) * 3
    assert np.abs(f["t"] - (1.0 - z))[core].max() < 1e-13
    if pad == 1:
        # the ghosts continue the line: 1 + h/2 below, -h/2 above
        assert np.abs(f["t"][:, :, 0] - (1.0 + 0.5 / n)).max() < 1e-13
        assert np.abs(f["t"][:, :, -1] + 0.5 / n).max() < 1e-13
    # a flux of the wrong sign on one wall moves the profile
    p.bc_t = S.field_bc([S.FBC_NEUMANN] * 6, [0.0] * 4 + [-1.0, 1.0])
    f["t"][...] = 1.0 - z
    O.rk3_run(g, p, f["vx"], f["vy"], f["vz"], f["p"], f["t"], f["pp"], 10)
    assert np.abs(f["t"] - (1.0 - z))[core].max() > 1e-4
