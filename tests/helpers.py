"""Shared input builders for the tests (seeded synthetic fields)."""
import numpy as np

import saras_gb300 as S


def core(a, g):
    if g.dims == 2:
        return a[1:-1, 1, 1:-1]
    p = g.pad
    return a[p:-p, p:-p, p:-p]


def random_rhs(g, seed, compatible=True):
    rng = np.random.default_rng(seed)
    rhs = S.padded_field(g)
    ny = 1 if g.dims == 2 else g.n[1]
    f = rng.uniform(-1.0, 1.0, (g.n[0], ny, g.n[2]))
    if compatible:
        f = S.project_compatible(g, f)
    p = g.pad
    py = 1 if g.dims == 2 else p
    rhs[p:p + g.n[0], py:py + ny, p:p + g.n[2]] = f
    return rhs


def random_guess(g, seed, amp=1e-3):
    rng = np.random.default_rng(seed)
    a = S.padded_field(g)
    ny = 1 if g.dims == 2 else g.n[1]
    p = g.pad
    py = 1 if g.dims == 2 else p
    a[p:p + g.n[0], py:py + ny, p:p + g.n[2]] = rng.uniform(-amp, amp, (g.n[0], ny, g.n[2]))
    return a


def demean(x):
    return x - x.mean()
