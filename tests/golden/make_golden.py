"""Generates tests/golden/golden.json: small oracle results (residual
histories and checksums of multigrid solves) used as regression fixtures.

The reference itself cannot be built here, so these fixtures pin the oracle
against its own earlier output; the reference-anchored pins are the
manufactured-solution and grid-formula tests in tests/test_oracle.py.

Run:  python tests/golden/make_golden.py   (rewrites golden.json)
"""
import json
import pathlib
import sys

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "saras-cc_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))

import pyoracle as O  # noqa: E402
import saras_gb300 as S  # noqa: E402


def _rhs(g, seed):
    rng = np.random.default_rng(seed)
    ny = 1 if g.dims == 2 else g.n[1]
    f = rng.uniform(-1, 1, (g.n[0], ny, g.n[2]))
    f = f - f.mean()
    rhs = S.padded_field(g)
    rhs[1:-1, 1:-1, 1:-1] = f
    return rhs


def _summ(a):
    return [float(a.sum()), float((a * a).sum()), float(a.flat[len(a.flat) // 3]), float(a.max())]


def compute():
    O.set_threads(1)
    out = {}
    cases = {
        "mg3d_uud_nnn": (dict(n=(8, 8, 16), mesh="UUD", beta=(1, 1, 1.3), domain="NNN"), {}),
        "mg3d_ddd_ppn": (dict(n=(8, 8, 8), mesh="DDD", beta=(1.2, 1.2, 1.2), domain="PPN"),
                         dict(bc_kind=[0, 0, 0, 0, 1, 1])),
        "mg2d_nn": (dict(n=(16, 1, 16), domain="NNN", dims=2), {}),
    }
    for name, (gk, mk) in cases.items():
        g = S.grid_desc(**gk)
        rhs = _rhs(g, 11)
        lhs = S.padded_field(g)
        prm = S.mg_params(vc_count=4, vc_tolerance=1e-30, pre_smooth=2, post_smooth=2, mg_tolerance=1e-12, **mk)
        r = O.mg_solve(g, prm, lhs, rhs)
        out[name + "_hist"] = [float(x) for x in r.history]
        out[name + "_sol"] = _summ(lhs)
    return out


if __name__ == "__main__":
    res = compute()
    (pathlib.Path(__file__).parent / "golden.json").write_text(json.dumps(res, indent=1))
    print("wrote", len(res), "fixtures")
