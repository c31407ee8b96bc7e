"""CPU tests that pin the oracle's time-step stencils and integrators.

Blitz++, which defines the reference's central12n/22n/14n/24n stencils, is
not vendored, and the reference stores no outputs of its time step, so these
properties pin the restatement instead:

* polynomial exactness of the first and second derivatives on uniform and
  stretched grids (calcDerivative1/2, derivative.cc:104-318): second-order
  central forms are exact up to degree 2 (3 for the second difference on a
  uniform axis), the fourth-order forms of dScheme 2 up to degree 4 (5) in
  the interior, with the reference's second-order forms on the first and
  last core cell;
* the convection term (computeNLin, vfield.cc:205-690, sfield.cc:160-495)
  with a constant velocity: standard and Morinishi forms give U dF/dx
  exactly for polynomials of the stencil's degree, the hybrid upwind form
  falls back to the central form below the Peclet limit and its biased
  stencils are exact for linear (first-order) and quadratic (second-order)
  fields above it;
* Morinishi's last-z-point test against the y extent (vfield.cc:337,427);
* the integrators' weights: a z-dependent shear flow on an all-periodic
  uniform grid has no convection and no pressure, so one step multiplies it
  by the amplification factor of the scheme for the discrete Laplacian's
  eigenvalue: prod_k (1 + alpha_k dt nu lam) / (1 - beta_k dt nu lam) for
  lsRK3 and (1 + dt nu lam / 2) / (1 - dt nu lam / 2) for eulerCN.
"""
import math

import numpy as np
import pytest

import pyoracle as O
import saras_gb300 as S


def params(nl_scheme=1, integration=2, pe_limit=2.0, up_param=0.8):
    p = S.Rk3Params()
    p.nu, p.kappa, p.dt = 1e-2, 1e-2, 1e-3
    p.cn_tolerance = 1e-14
    p.nl_scheme = nl_scheme
    p.integration = integration
    p.pe_limit, p.up_param = pe_limit, up_param
    p.with_scalar = 0
    p.mg = S.mg_params(vc_count=20, vc_tolerance=1e-10, pre_smooth=3, post_smooth=6, mg_tolerance=1e-10)
    return p


def xi_of(g, axis):
    """Computational coordinate of the cell centres over -pad..n+pad-1."""
    p = 1 if (g.dims == 2 and axis == 1) else g.pad
    n = g.n[axis]
    return (np.arange(-p, n + p) + 0.5) / n


def along(g, axis, vals):
    """Padded field that varies along `axis` only."""
    f = S.padded_field(g)
    shape = [1, 1, 1]
    shape[axis] = len(vals)
    f[...] = np.asarray(vals).reshape(shape)
    return f


def core_line(a, g, axis):
    p = g.pad
    py = 1 if g.dims == 2 else p
    c = a[p:p + g.n[0], py:py + (1 if g.dims == 2 else g.n[1]), p:p + g.n[2]]
    idx = [0, 0, 0]
    idx[axis] = slice(None)
    return c[tuple(idx)]


GRIDS = [
    dict(n=(16, 12, 20), mesh="DSD", beta=(1.2, 1.1, 1.3), length=(1.0, 0.7, 2.0), domain="NNN"),
    dict(n=(24, 1, 16), mesh="UUD", beta=(1, 1, 1.4), domain="PNN", dims=2),
]


@pytest.mark.parametrize("gk", GRIDS, ids=["3d_stretched", "planar"])
@pytest.mark.parametrize("pad", [1, 2])
def test_derivatives_polynomial_exact(gk, pad):
    g = S.grid_desc(pad=pad, **gk)
    prm = params()
    axes = (0, 2) if g.dims == 2 else (0, 1, 2)
    for axis in axes:
        xi = xi_of(g, axis)
        _, xi_x, xixx, xix2 = O.field_metrics(g, axis)
        p = 1 if (g.dims == 2 and axis == 1) else g.pad
        core = slice(p, p + g.n[axis])
        n = g.n[axis]
        for deg in range(1, 6):
            f = along(g, axis, xi ** deg)
            d1 = core_line(O.field_op(g, prm, 1, f, axis), g, axis)
            d2 = core_line(O.field_op(g, prm, 2, f, axis), g, axis)
            e1 = deg * xi[core] ** (deg - 1) * xi_x[core]
            e2 = deg * (deg - 1) * xi[core] ** max(deg - 2, 0) * xix2[core] + deg * xi[core] ** (deg - 1) * xixx[core]
            s1, s2 = np.abs(e1).max() + 1.0, np.abs(e2).max() + 1.0
            inner = slice(1, n - 1) if pad == 2 else slice(0, n)
            exact1 = 4 if pad == 2 else 2
            # xixx * (first difference) limits a stretched axis to exact1
            exact2 = exact1 if np.abs(xixx).max() > 0 else (5 if pad == 2 else 3)
            if deg <= exact1:
                assert np.abs(d1[inner] - e1[inner]).max() <= 1e-9 * s1, (axis, deg)
            else:
                assert np.abs(d1[inner] - e1[inner]).max() > 1e-9 * s1, (axis, deg)
            if deg <= exact2:
                assert np.abs(d2[inner] - e2[inner]).max() <= 1e-8 * s2, (axis, deg)
            if pad == 2:
                ends = [0, n - 1]
                # the reference's second-order forms on the first and last cell
                if deg <= 2:
                    assert np.abs(d1[ends] - e1[ends]).max() <= 1e-9 * s1
                if deg <= (2 if np.abs(xixx).max() > 0 else 3):
                    assert np.abs(d2[ends] - e2[ends]).max() <= 1e-8 * s2
                if deg == 3:
                    assert np.abs(d1[ends] - e1[ends]).max() > 1e-9 * s1


def _const_velocity(g, u):
    return tuple(None if (g.dims == 2 and d == 1) else np.full(S.padded_field(g).shape, u[d]) for d in range(3))


@pytest.mark.parametrize("pad", [1, 2])
@pytest.mark.parametrize("nl", [1, 3])
def test_convection_exact_for_constant_velocity(pad, nl):
    gk = dict(n=(16, 16, 16), mesh="DUD", beta=(1.2, 1, 1.3), domain="NNN")
    g = S.grid_desc(pad=pad, **gk)
    u = (0.3, -0.2, 0.5)
    v = _const_velocity(g, u)
    prm = params(nl_scheme=nl)
    deg = 4 if pad == 2 else 2
    for axis in range(3):
        xi = xi_of(g, axis)
        _, xi_x, _, _ = O.field_metrics(g, axis)
        p = g.pad
        core = slice(p, p + g.n[axis])
        f = along(g, axis, xi ** deg)
        h = core_line(O.field_op(g, prm, 3, f, v=v), g, axis)
        e = -u[axis] * deg * xi[core] ** (deg - 1) * xi_x[core]
        inner = slice(1, g.n[axis] - 1) if pad == 2 else slice(None)
        assert np.abs(h[inner] - e[inner]).max() <= 1e-9 * (np.abs(e).max() + 1.0), (axis, nl)


def test_morinishi_last_z_point_follows_y_extent():
    """dScheme 2, Nz != Ny: the second-order form is taken at k = Ny - 1 and
    the fourth-order form at k = Nz - 1, which reads the second ghost layer."""
    g = S.grid_desc(n=(8, 8, 16), domain="NNN", pad=2)
    prm = params(nl_scheme=3)
    v = _const_velocity(g, (0.0, 0.0, 0.7))
    xi = xi_of(g, 2)
    f = along(g, 2, xi ** 3)
    h = core_line(O.field_op(g, prm, 3, f, v=v), g, 2)
    _, xi_x, _, _ = O.field_metrics(g, 2)
    e = -0.7 * 3 * xi[2:18] ** 2 * xi_x[2:18]
    err = np.abs(h - e)
    assert err[7] > 1e-6 and err[0] > 1e-6        # second order at k = 0 and k = Ny - 1
    assert err[15] < 1e-9 and err[1:7].max() < 1e-9  # fourth order at k = Nz - 1
    f2 = f.copy()
    f2[:, :, -1] += 1.0                             # the second ghost layer above the top
    h2 = core_line(O.field_op(g, prm, 3, f2, v=v), g, 2)
    assert h2[15] != h[15] and np.array_equal(h2[:15], h[:15])


@pytest.mark.parametrize("pad", [1, 2])
def test_upwind_central_below_peclet_limit(pad):
    g = S.grid_desc(n=(16, 16, 16), mesh="UUD", beta=(1, 1, 1.2), domain="NNN", pad=pad)
    rng = np.random.default_rng(3)
    f = rng.uniform(-1, 1, S.padded_field(g).shape)
    v = tuple(rng.uniform(-0.1, 0.1, f.shape) for _ in range(3))
    # Pe = |u| dh / dcoef < 2 everywhere: central differences of the order
    # dScheme gives (nlScheme 1 for dScheme 1; the fourth-order central form
    # with second-order end cells for dScheme 2)
    up = O.field_op(g, params(nl_scheme=2), 3, f, v=v, dcoef=1.0)
    if pad == 1:
        ref = O.field_op(g, params(nl_scheme=1), 3, f, v=v, dcoef=1.0)
        assert np.allclose(up, ref, rtol=1e-13, atol=1e-13)
    else:
        st = O.field_op(g, params(nl_scheme=1), 3, f, v=v, dcoef=1.0)
        assert np.allclose(up, st, rtol=1e-11, atol=1e-11)


@pytest.mark.parametrize("pad,deg", [(1, 1), (2, 2)])
@pytest.mark.parametrize("sign", [1.0, -1.0])
def test_upwind_biased_stencils_exact(pad, deg, sign):
    g = S.grid_desc(n=(16, 16, 16), domain="NNN", pad=pad)
    u = sign * 0.5
    prm = params(nl_scheme=2, up_param=0.3)
    for axis in range(3):
        uu = [0.0, 0.0, 0.0]
        uu[axis] = u
        v = _const_velocity(g, uu)
        xi = xi_of(g, axis)
        _, xi_x, _, _ = O.field_metrics(g, axis)
        core = slice(g.pad, g.pad + 16)
        f = along(g, axis, xi ** deg)
        h = core_line(O.field_op(g, prm, 3, f, v=v, dcoef=1e-9), g, axis)   # Pe >> limit
        e = -u * deg * xi[core] ** (deg - 1) * xi_x[core]
        assert np.abs(h - e).max() <= 1e-9
        # one degree more is not reproduced by the biased stencil
        f3 = along(g, axis, xi ** (deg + 1))
        h3 = core_line(O.field_op(g, prm, 3, f3, v=v, dcoef=1e-9), g, axis)
        e3 = -u * (deg + 1) * xi[core] ** deg * xi_x[core]
        assert np.abs(h3 - e3)[2:-2].max() > 1e-6


@pytest.mark.parametrize("integration", [1, 2])
def test_integrator_amplification_of_shear_mode(integration):
    n = 16
    g = S.grid_desc(n=(8, 8, n), domain="PPP", pad=1)
    prm = params(integration=integration)
    prm.dt = 5e-2
    prm.nu = 2e-3
    per = S.field_bc([S.FBC_NEUMANN] * 6, [0.0] * 6)
    prm.bc_vx = prm.bc_vy = prm.bc_vz = prm.bc_p = prm.bc_t = per
    zc = (np.arange(-1, n + 1) + 0.5) / n
    vx = along(g, 2, np.sin(2 * math.pi * zc))
    f = {k: S.padded_field(g) for k in ("vy", "vz", "p", "t", "pp")}
    r = O.rk3_run(g, prm, vx, f["vy"], f["vz"], f["p"], f["t"], f["pp"], 1)
    assert r.status == 0
    h = 1.0 / n
    lam = -4.0 / h ** 2 * math.sin(math.pi * h) ** 2
    dt, nu = prm.dt, prm.nu
    if integration == 1:
        amp = (1 + 0.5 * dt * nu * lam) / (1 - 0.5 * dt * nu * lam)
    else:
        amp = 1.0
        for a in (4 / 15, 1 / 15, 1 / 6):
            amp *= (1 + a * dt * nu * lam) / (1 - a * dt * nu * lam)
    got = vx[1:-1, 1:-1, 1:-1]
    want = amp * np.sin(2 * math.pi * zc[1:-1])[None, None, :]
    assert np.abs(got - want).max() < 1e-11
    assert np.abs(f["vz"]).max() == 0.0 and np.abs(f["pp"]).max() < 1e-12


def _rbc(g, with_scalar=1):
    """Rayleigh-Benard set-up: no-slip walls, hot bottom and cold top, the
    reference's Multigrid defaults for the pressure solve."""
    p = params()
    p.with_scalar = with_scalar
    p.nu, p.kappa = 3e-3, 3e-3
    p.cn_tolerance = 1e-12
    for d, gv in enumerate((0.0, 0.0, -1.0)):
        p.g_terms[d] = gv if with_scalar else 0.0
    p.bc_vx = p.bc_vy = p.bc_vz = S.field_bc([S.FBC_DIRICHLET] * 6, [0.0] * 6)
    p.bc_t = S.field_bc([S.FBC_NEUMANN] * 4 + [S.FBC_DIRICHLET] * 2, [0, 0, 0, 0, 1.0, 0.0])
    p.bc_p = S.field_bc([S.FBC_NEUMANN] * 6, [0.0] * 6)
    p.mg = S.mg_params(vc_count=20, vc_tolerance=1e-6, pre_smooth=3, post_smooth=6, mg_tolerance=1e-2)
    return p


@pytest.mark.parametrize("gk", [dict(n=(8, 8, 16), mesh="UUD", beta=(1, 1, 1.3), domain="PPN"),
                                dict(n=(16, 1, 16), mesh="UUD", beta=(1, 1, 1.2), domain="PNN", dims=2)],
                         ids=["3d", "planar"])
def test_tseries_conductive_state(gk):
    """tseries::writeTSData on the conductive Rayleigh-Benard state T = 1 - z,
    u = 0, on a grid symmetric about mid-height: Nu (wall) = Nu (volume) = 1
    and zero kinetic and thermal energy (theta = T + z - 1 = 0)."""
    g = S.grid_desc(**gk)
    p = _rbc(g)
    x, _, _, _ = O.field_metrics(g, 2)
    t = along(g, 2, 1.0 - x)
    z = [S.padded_field(g) for _ in range(3)]
    row, cfl = O.tseries(g, p, S.run_params(), z[0], z[1], z[2], t)
    assert abs(row["nu_wall"] - 1.0) < 1e-12 and row["nu_vol"] == 1.0
    assert row["ke"] == 0.0 and abs(row["te"]) < 1e-28 and row["divergence"] == 0.0 and cfl == 0.0


def test_tseries_uniform_flow_energy_and_cfl():
    # uniform cells: the volumes dXi/xi_x add up to the box exactly
    g = S.grid_desc(n=(8, 8, 16), length=(2.0, 1.0, 1.0), domain="NNN")
    p = _rbc(g, with_scalar=0)
    vx = np.full(S.padded_field(g).shape, 0.3)
    vz = np.full(vx.shape, -0.4)
    row, cfl = O.tseries(g, p, S.run_params(), vx, np.zeros_like(vx), vz, None)
    assert abs(row["ke"] - 0.5 * (0.09 + 0.16)) < 1e-14 and abs(row["urms"] - 0.5) < 1e-14
    assert row["divergence"] < 1e-12
    assert cfl == pytest.approx(0.3 / (2.0 / 8) + 0.4 / (1.0 / 16), rel=1e-15)


def test_time_loop_fixed_dt_equals_steps():
    """Without CFL the loop is nsteps calls of timeAdvance: t_max = 4 dt runs
    four steps and leaves the same fields as four steps."""
    g = S.grid_desc(n=(8, 8, 8), mesh="UUD", beta=(1, 1, 1.2), domain="NNN")
    p = _rbc(g)
    p.dt = 1e-3
    rng = np.random.default_rng(5)
    f = {k: S.padded_field(g) for k in ("vx", "vy", "vz", "p", "t", "pp")}
    for k in ("vx", "vy", "vz"):
        f[k][...] = rng.uniform(-0.05, 0.05, f[k].shape)
    f["t"][...] = rng.uniform(0, 1, f["t"].shape)
    a = {k: v.copy() for k, v in f.items()}
    r = O.rk3_loop(g, p, S.run_params(t_max=4e-3, io_count=2), a["vx"], a["vy"], a["vz"], a["p"], a["t"], a["pp"])
    assert r.status == 0 and r.n_steps == 4 and len(r.rows) == 3
    assert [row["time"] for row in r.rows] == [0.0, 2e-3, 2e-3 + 2e-3]
    b = {k: v.copy() for k, v in f.items()}
    O.rk3_run(g, p, b["vx"], b["vy"], b["vz"], b["p"], b["t"], b["pp"], 4)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
