"""CPU tests of the oracle (the restatement of the reference's hot path) and of
the product's host-side grid geometry.

The reference ships no golden vectors; the oracle is pinned against
(1) the reference's own known answer, tests/mgTest: TEST_POISSON with RHS 1
and analytic r^2/6 Dirichlet walls on a 'DDD' grid, whose deviation from the
analytic solution must fall at second order (poisson.cc:132-176),
(2) the 2D manufactured solution cos(2 pi x) cos(2 pi z) -> -f/(8 pi^2),
(3) the tanh-grid formulas of grid::createTanHypGrid evaluated independently
in numpy (grid.cc:442-463), (4) the V-cycle depths setVCDepth gives
(grid.cc:678-742), (5) committed fixtures of small solves
(tests/golden/, made by tests/golden/make_golden.py), and (6) 3-D
manufactured solutions on the benchmark meshes (z tanh-stretched with
Neumann walls; stretched on every axis with Dirichlet z walls), recovered at
second order.
"""
import json
import math
import pathlib

import numpy as np
import pytest

import pyoracle as O
import saras_gb300 as S

GOLDEN = pathlib.Path(__file__).parent / "golden"


@pytest.mark.parametrize("n,domain,dims,levels", [
    ((256, 256, 256), "NNN", 3, 7),
    ((256, 1, 256), "NNN", 2, 7),
    ((512, 512, 512), "PPN", 3, 9),
    ((256, 256, 256), "PPN", 3, 8),
    ((96, 96, 96), "NNN", 3, 5),
    ((192, 192, 96), "NNN", 3, 5),
    ((96, 96, 48), "NNN", 3, 4),
])
def test_vcycle_depth(n, domain, dims, levels):
    g = S.grid_desc(n=n, domain=domain, dims=dims)
    assert O.num_levels(g) == levels


def _tanh_ref(mtype, beta, L, xi):
    thb = math.tanh(beta)
    btl = beta * L
    if mtype == "D":
        x = L * (1.0 - math.tanh(beta * (1.0 - 2.0 * xi)) / thb) / 2.0
        ndx = x / L
        fx = thb / (btl * (1.0 - ((1.0 - 2.0 * ndx) * thb) ** 2))
        fxx = -4.0 * thb ** 3 * (1.0 - 2.0 * ndx) / (L * btl * (1.0 - (thb * (1.0 - 2.0 * ndx)) ** 2) ** 2)
    else:
        x = L * (1.0 - math.tanh(beta * (1.0 - xi)) / thb)
        ndx = x / L
        fx = thb / (btl * (1.0 - ((1.0 - ndx) * thb) ** 2))
        fxx = -2.0 * thb ** 3 * (1.0 - ndx) / (L * btl * (1.0 - (thb * (1.0 - ndx)) ** 2) ** 2)
    return x, fx, fxx, fx * fx


@pytest.mark.parametrize("mtype", ["S", "D"])
def test_tanh_metrics_match_formula(mtype):
    g = S.grid_desc(n=(32, 16, 64), mesh="UU" + mtype, beta=(1, 1, 1.3), length=(1, 1, 2.0), domain="NNN")
    x, xixx, xix2 = O.grid_metrics(g, 0, 2)
    for i in range(64):
        xi = (2 * i + 1) / 64 / 2
        xr, fx, fxx, fx2 = _tanh_ref(mtype, 1.3, 2.0, xi)
        assert abs(x[i + 1] - xr) < 1e-13
        assert abs(xixx[i + 1] - fxx) <= 1e-12 * abs(fxx) + 1e-14
        assert abs(xix2[i + 1] - fx2) <= 1e-12 * fx2
    # coarse level: cell centre at the mean of its children's xi
    xc, _, c2 = O.grid_metrics(g, 2, 2)
    lv1 = [0.5 * ((2 * (2 * i) + 1) / 128 + (2 * (2 * i + 1) + 1) / 128) for i in range(32)]
    lv2 = [0.5 * (lv1[2 * i] + lv1[2 * i + 1]) for i in range(16)]
    for i in range(16):
        xr, fx, fxx, fx2 = _tanh_ref(mtype, 1.3, 2.0, lv2[i])
        assert abs(xc[i + 1] - xr) < 1e-13
        assert abs(c2[i + 1] - fx2) <= 1e-12 * fx2


def test_product_metrics_equal_oracle_bitwise():
    for gk in [dict(n=(32, 16, 64), mesh="SUD", beta=(1.1, 1, 1.3), domain="NNN"),
               dict(n=(64, 64, 64), mesh="DDD", beta=(1.2, 1.2, 1.2), domain="PPN"),
               dict(n=(48, 1, 96), mesh="DUS", beta=(1.5, 1, 1.2), domain="NNN", dims=2),
               dict(n=(16, 16, 16), mesh="DDD", beta=(1.0, 1.0, 1.0), domain="NNN", pad=2)]:
        g = S.grid_desc(**gk)
        levels = O.num_levels(g)
        lib = S.load()
        assert lib.saras_reference_levels(g) == levels
        for lvl in range(levels):
            for ax in (0, 1, 2):
                if g.dims == 2 and ax == 1:
                    continue
                a = O.grid_metrics(g, lvl, ax)
                b = S.grid_metrics(g, lvl, ax)
                for p, q in zip(a, b):
                    assert np.array_equal(p, q), (gk, lvl, ax)


def test_null_vector_annihilates_operator():
    g = S.grid_desc(n=(8, 8, 48), mesh="UUD", beta=(1, 1, 1.4), domain="NNN")
    w = S.null_vector(g, 2)
    _, xixx, xix2 = O.grid_metrics(g, 0, 2)
    n = 48
    h = 1.0 / n
    A = np.zeros((n, n))
    for i in range(n):
        c2, c1 = xix2[i + 1] / h ** 2, xixx[i + 1] * 0.5 / h
        lo, up = c2 - c1, c2 + c1
        A[i, i] -= 2 * c2
        if i > 0:
            A[i, i - 1] += lo
        else:
            A[i, i] += lo
        if i < n - 1:
            A[i, i + 1] += up
        else:
            A[i, i] += up
    assert np.abs(w @ A).max() < 1e-9 * np.abs(A).max()
    assert np.abs(A @ np.ones(n)).max() < 1e-9 * np.abs(A).max()


def test_mgtest_second_order():
    """Deviation from the analytic r^2/6 falls at second order from 24 to 96
    cells a side, 96^3 being tests/mgTest's own grid (1.0e-5 there)."""
    errs = []
    for n in (24, 48, 96):
        g = S.grid_desc(n=(n, n, n), mesh="DDD", beta=(1, 1, 1), domain="NNN")
        prm = S.mg_params(vc_count=20, vc_tolerance=1e-6, pre_smooth=5, post_smooth=5, mg_tolerance=1e-6,
                          test_poisson=1, bc_kind=[2] * 6)
        rhs = S.padded_field(g)
        rhs[1:-1, 1:-1, 1:-1] = 1.0
        lhs = S.padded_field(g)
        r = O.mg_solve(g, prm, lhs, rhs)
        assert r.cycles == 20 and r.history[-1] < 1e-10
        xs = [O.grid_metrics(g, 0, d)[0][1:-1] for d in range(3)]
        pa = ((xs[0][:, None, None] - 0.5) ** 2 + (xs[1][None, :, None] - 0.5) ** 2
              + (xs[2][None, None, :] - 0.5) ** 2) / 6
        errs.append(np.abs(pa - lhs[1:-1, 1:-1, 1:-1]).max())
    for a, b in zip(errs, errs[1:]):
        assert 3.5 < a / b < 4.5, errs
    assert errs[-1] < 1.1e-5


def test_mgtest_planar():
    """tests/mgTest in a PLANAR build (poisson.cc:139-147): RHS 1, analytic
    ((x-1/2)^2 + (z-1/2)^2)/4 on the TEST_POISSON Dirichlet walls.  The
    deviation falls at second order on the tanh mesh; on a uniform mesh,
    where the five-point stencil is exact for the quadratic, it is h^2/16:
    the mirrored wall ghost's error alone."""
    for mesh in ("DUD", "UUU"):
        errs = []
        for n in (32, 64, 128):
            g = S.grid_desc(n=(n, 1, n), mesh=mesh, beta=(1, 1, 1), domain="NNN", dims=2)
            prm = S.mg_params(vc_count=20, vc_tolerance=1e-6, pre_smooth=5, post_smooth=5, mg_tolerance=1e-6,
                              test_poisson=1, bc_kind=[2] * 6)
            rhs = S.padded_field(g)
            rhs[1:-1, 1, 1:-1] = 1.0
            lhs = S.padded_field(g)
            r = O.mg_solve(g, prm, lhs, rhs)
            assert r.status == 0 and r.history[-1] < 1e-10
            x = O.grid_metrics(g, 0, 0)[0][1:-1]
            z = O.grid_metrics(g, 0, 2)[0][1:-1]
            pa = ((x[:, None] - 0.5) ** 2 + (z[None, :] - 0.5) ** 2) / 4
            errs.append(np.abs(pa - lhs[1:-1, 1, 1:-1]).max())
            if mesh == "UUU":
                assert abs(errs[-1] - 1.0 / (16 * n * n)) < 1e-8 / (n * n), (n, errs[-1])
        for a, b in zip(errs, errs[1:]):
            assert 3.9 < a / b < 4.1, (mesh, errs)


def test_2d_cos_manufactured_second_order():
    errs = []
    for n in (64, 128):
        g = S.grid_desc(n=(n, 1, n), domain="NNN", dims=2)
        x = O.grid_metrics(g, 0, 0)[0][1:-1]
        z = O.grid_metrics(g, 0, 2)[0][1:-1]
        f = np.cos(2 * np.pi * x)[:, None] * np.cos(2 * np.pi * z)[None, :]
        rhs = S.padded_field(g)
        rhs[1:-1, 1, 1:-1] = f
        lhs = S.padded_field(g)
        prm = S.mg_params(vc_count=200, vc_tolerance=1e-10, pre_smooth=2, post_smooth=2, mg_tolerance=1e-12)
        r = O.mg_solve(g, prm, lhs, rhs)
        assert r.status == 0 and r.history[-1] < 1e-10 and r.cycles < 20
        u = lhs[1:-1, 1, 1:-1]
        ex = -f / (8 * np.pi ** 2)
        errs.append(np.abs((u - u.mean()) - (ex - ex.mean())).max())
    assert 3.5 < errs[0] / errs[1] < 4.5, errs


def _manufactured_3d(n, mesh, beta, domain, bc_kind, exact, lap):
    """Solves A u = lap(exact) at the cell centres of a 3-D grid; returns the
    deviation from `exact` over the core (the constant removed where the
    operator is singular)."""
    g = S.grid_desc(n=(n, n, n), mesh=mesh, beta=beta, domain=domain)
    xs = [O.field_metrics(g, d)[0] for d in range(3)]
    x, y, z = xs[0][:, None, None], xs[1][None, :, None], xs[2][None, None, :]
    ex = exact(x, y, z)
    core = (slice(1, -1),) * 3
    rhs = S.padded_field(g)
    singular = all(k == 0 for k in bc_kind)
    f = lap(x, y, z)[core]
    # an all-Neumann operator wants a compatible right-hand side (its
    # component along the discrete left null vector removed)
    rhs[core] = O.project_compatible(g, f) if singular else f
    lhs = S.padded_field(g)
    prm = S.mg_params(vc_count=200, vc_tolerance=1e-10, pre_smooth=3, post_smooth=6, mg_tolerance=1e-12,
                      bc_kind=bc_kind)
    r = O.mg_solve(g, prm, lhs, rhs)
    assert r.status == 0 and r.cycles < 40
    d = (lhs - ex)[core]
    return np.abs(d - d.mean()).max() if singular else np.abs(d).max()


def test_benchmark_mesh_manufactured_second_order():
    """The operator of the 256^3 benchmark's mesh (z tanh-stretched, beta 1.3,
    Neumann walls) converges to the Laplacian: cos(pi x) cos(pi y) cos(pi z)
    is recovered with a deviation falling by 4 per halving of h."""
    pi = math.pi
    errs = [_manufactured_3d(n, "UUD", (1, 1, 1.3), "NNN", [0] * 6,
                             lambda x, y, z: np.cos(pi * x) * np.cos(pi * y) * np.cos(pi * z),
                             lambda x, y, z: -3 * pi ** 2 * np.cos(pi * x) * np.cos(pi * y) * np.cos(pi * z))
            for n in (16, 32, 64)]
    for a, b in zip(errs, errs[1:]):
        assert 3.7 < a / b < 4.3, errs


def test_dirichlet_stretched_mesh_manufactured_second_order():
    """The 512^3 configuration's mesh (tanh-stretched on every axis, beta 1.2,
    periodic x and y, homogeneous Dirichlet walls in z through the boundary
    selector): cos(2 pi x) cos(2 pi y) sin(pi z) at second order."""
    pi = math.pi
    errs = [_manufactured_3d(n, "DDD", (1.2, 1.2, 1.2), "PPN", [0, 0, 0, 0, 1, 1],
                             lambda x, y, z: np.cos(2 * pi * x) * np.cos(2 * pi * y) * np.sin(pi * z),
                             lambda x, y, z: -9 * pi ** 2 * np.cos(2 * pi * x) * np.cos(2 * pi * y) * np.sin(pi * z))
            for n in (16, 32, 64)]
    for a, b in zip(errs, errs[1:]):
        assert 3.5 < a / b < 4.3, errs


def test_oracle_thread_count_invariant():
    g = S.grid_desc(n=(16, 16, 32), mesh="UUD", beta=(1, 1, 1.3), domain="NNN")
    from helpers import random_rhs
    rhs = random_rhs(g, 2)
    out = []
    for t in (1, 4):
        O.set_threads(t)
        lhs = S.padded_field(g)
        r = O.mg_solve(g, S.mg_params(vc_count=3, vc_tolerance=1e-30, pre_smooth=2, post_smooth=2), lhs, rhs)
        out.append((lhs, r.history))
    O.set_threads(1)
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_golden_fixtures():
    """Small oracle solves and RK3 steps against committed fixtures."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    ref = json.loads((GOLDEN / "golden.json").read_text())
    now = mk.compute()
    assert ref.keys() == now.keys()
    for k in ref:
        a, b = np.array(ref[k]), np.array(now[k])
        # fixtures are recorded on x86-64; libm's tanh/pow may differ in the
        # last bit on other hosts
        np.testing.assert_allclose(b, a, rtol=1e-9, atol=1e-14, err_msg=k)


@pytest.mark.parametrize("n,dims", [((2, 2, 2), 3), ((3, 5, 7), 3), ((2, 1, 2), 2), ((4, 4, 4), 3),
                                    ((6, 6, 6), 3), ((64, 8, 16), 3), ((8, 1, 8), 2), ((96, 96, 48), 3)])
def test_depth_rule_and_rejected_sizes(n, dims):
    """setVCDepth (grid.cc:678-742) on small, odd and ragged sizes: the
    product's host-side depth equals the oracle's, and the sizes the
    reference cannot build a hierarchy for are rejected by both (-1)."""
    g = S.grid_desc(n=n, domain="NNN", dims=dims)
    lib = S.load()
    assert lib.saras_reference_levels(g) == O.num_levels(g)


@pytest.mark.parametrize("gk", [
    dict(n=(256, 256, 256), mesh="UUD", beta=(1, 1, 1.3), domain="NNN"),
    dict(n=(32, 16, 64), mesh="SDU", beta=(1.2, 1.4, 1.0), domain="NNN"),
    dict(n=(64, 1, 32), mesh="DUS", beta=(1.1, 1.0, 1.3), domain="NNN", dims=2),
])
def test_oracle_null_vector_equals_product(gk):
    """The oracle's left null vector and compatible projection (numpy, from
    the oracle's metrics) are bit-identical to the product's host
    restatement, so the CPU baseline solves exactly the GPU's right-hand side
    without loading the product library."""
    g = S.grid_desc(**gk)
    for d in (0, 2) if g.dims == 2 else (0, 1, 2):
        assert np.array_equal(O.null_vector(g, d), S.null_vector(g, d)), d
    ny = 1 if g.dims == 2 else g.n[1]
    f = np.random.default_rng(4).uniform(-1, 1, (g.n[0], ny, g.n[2]))
    assert np.array_equal(O.project_compatible(g, f), S.project_compatible(g, f))


def test_product_grid_equals_oracle_on_random_grids():
    """Seeded sweep over shapes (powers of two times 1, 3, 5 or 7, and a few
    ragged sizes), mesh types, stretching factors, periodicity and pad: the
    product's host-side level count and per-level metrics equal the
    oracle's bit for bit."""
    rng = np.random.default_rng(11)
    lib = S.load()
    checked = 0
    for _ in range(40):
        dims = 2 if rng.random() < 0.3 else 3
        n = [int(rng.choice([1, 3, 5, 7])) << int(rng.integers(1, 6)) for _ in range(3)]
        if rng.random() < 0.15:
            n[int(rng.integers(0, 3))] = int(rng.integers(5, 40))
        if dims == 2:
            n[1] = 1
        mesh = "".join(rng.choice(list("USD"), 3))
        beta = tuple(float(b) for b in rng.uniform(0.8, 1.6, 3))
        domain = "".join(rng.choice(list("PN"), 3))
        pad = int(rng.choice([1, 2]))
        g = S.grid_desc(n=tuple(n), mesh=mesh, beta=beta, domain=domain, dims=dims, pad=pad)
        levels = O.num_levels(g)
        assert lib.saras_reference_levels(g) == levels, (n, dims)
        if levels < 1:
            continue
        for lvl in range(levels):
            for ax in (0, 1, 2):
                if dims == 2 and ax == 1:
                    continue
                for p, q in zip(O.grid_metrics(g, lvl, ax), S.grid_metrics(g, lvl, ax)):
                    assert np.array_equal(p, q), (n, mesh, beta, domain, dims, pad, lvl, ax)
        checked += 1
    assert checked >= 30
