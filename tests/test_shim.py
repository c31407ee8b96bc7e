"""The C++ drop-in (saras-cc_gb300/shim/saras_shim.h) compiles against the
library, reads the reference's parameters.yaml keys and, on a GPU, solves
through multigrid_d3::mgSolve."""
import pathlib
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
SHIM = ROOT / "saras-cc_gb300" / "shim"
LIB = ROOT / "saras-cc_gb300" / "lib"


def _build(tmp_path):
    exe = tmp_path / "mgsolve_example"
    subprocess.run(["g++", "-O2", "-std=c++17", str(SHIM / "mgsolve_example.cpp"), "-I", str(SHIM),
                    "-L", str(LIB), "-lsaras_gb300", f"-Wl,-rpath,{LIB}", "-o", str(exe)], check=True)
    return exe


def test_shim_compiles_and_parses(tmp_path):
    exe = _build(tmp_path)
    out = subprocess.run([str(exe), str(ROOT / "tests" / "golden" / "mg_params.yaml"), "--parse-only"],
                         capture_output=True, text=True, check=True).stdout
    assert "grid 32x32x32 mesh UUU domain NNN levels 4 vcCount 60 tol 1.0e-10 pre/post 2/2" in out


REJECTED = [
    ('"X Size": 32', '"X Size": 1', "ERROR: Insufficient number of points along X axis. Aborting"),
    ('"Y Size": 32', '"Y Size": 1', "ERROR: Insufficient number of points along Y axis. Aborting"),
    ('"Z Size": 32', '"Z Size": 1', "ERROR: Insufficient number of points along Z axis. Aborting"),
    ('"Domain Type": "NNN"', '"Domain Type": "NN"', "ERROR: Domain type string is not correct. Aborting"),
    ('"Mesh Type": "UUU"', '"Mesh Type": "UUUU"', "ERROR: Mesh type string is not correct. Aborting"),
    ('"Solve Tolerance": 1.0e-10', '"Solve Tolerance": 1.0e-10\n    "Time-Step": 0.1\n    "Final Time": 0.01',
     "ERROR: Time step is larger than the maximum duration assigned for simulation. Aborting"),
    ('"Residual Type": 0', '"Residual Type": 3',
     "ERROR: The specified value for printing error at end of V-Cycles is not defined. Aborting"),
    # grid::grid (grid.cc:69-77)
    ('"Differentiation Scheme": 1', '"Differentiation Scheme": 3',
     "Undefined finite differencing scheme in YAML file. ABORTING"),
]


def test_shim_rejects_what_the_reference_rejects(tmp_path):
    """parser::checkData (parser.cc:299-411): each input the reference
    aborts on is rejected with its message (exit status 3 from the example,
    which catches the exception), before any device work."""
    exe = _build(tmp_path)
    base = (ROOT / "tests" / "golden" / "mg_params.yaml").read_text()
    for old, new, msg in REJECTED:
        assert old in base, old
        y = tmp_path / "bad.yaml"
        y.write_text(base.replace(old, new, 1))
        r = subprocess.run([str(exe), str(y), "--parse-only"], capture_output=True, text=True)
        assert r.returncode == 3 and msg in r.stdout, (new, r.returncode, r.stdout, r.stderr)
    # a time step within the final time passes
    y = tmp_path / "ok.yaml"
    y.write_text(base.replace('"Solve Tolerance": 1.0e-10', '"Solve Tolerance": 1.0e-10\n    "Time-Step": 0.01\n'
                              '    "Final Time": 1.0', 1))
    r = subprocess.run([str(exe), str(y), "--parse-only"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout


def test_shim_grid_anisotropy(tmp_path):
    """grid::checkAnisotropy (grid.cc:756-804) runs when an axis is
    stretched: it reports the largest ratio of two cell widths (centres -1..N
    along each axis), with a WARNING above 7."""
    import sys
    sys.path.insert(0, str(ROOT / "oracle"))
    import numpy as np
    import pyoracle as O
    import saras_gb300 as S
    exe = _build(tmp_path)
    base = (ROOT / "tests" / "golden" / "mg_params.yaml").read_text()
    r = subprocess.run([str(exe), str(ROOT / "tests" / "golden" / "mg_params.yaml"), "--parse-only"],
                       capture_output=True, text=True, check=True)
    assert "anisotropy" not in r.stdout  # uniform: no check, as in the reference
    for beta, warn in ((1.3, False), (3.0, True)):
        y = tmp_path / "stretched.yaml"
        y.write_text(base.replace('"Mesh Type": "UUU"', '"Mesh Type": "UUD"').replace('"Z Beta": 1.0',
                                                                                     f'"Z Beta": {beta}'))
        out = subprocess.run([str(exe), str(y), "--parse-only"], capture_output=True, text=True,
                             check=True).stdout
        if warn:
            assert "WARNING: Grid anisotropy exceeds limits. Finite-difference calculations will be inaccurate" in out
            continue
        g = S.grid_desc(n=(32, 32, 32), mesh="UUD", beta=(1, 1, beta), domain="NNN")
        w = [np.abs(np.diff(O.field_metrics(g, d)[0])) for d in range(3)]
        ar = max(w[a].max() / w[b].min() for a in range(3) for b in range(3) if a != b)
        got = float(out.split("Maximum grid anisotropy is")[1].split()[0])
        assert abs(got - ar) <= 1e-5 * ar, (got, ar)


@pytest.mark.gpu
def test_shim_mgsolve(tmp_path):
    exe = _build(tmp_path)
    out = subprocess.run([str(exe), str(ROOT / "tests" / "golden" / "mg_params.yaml")],
                         capture_output=True, text=True, check=True).stdout
    line = [l for l in out.splitlines() if l.startswith("mgSolve")][0]
    err = float(line.split()[-1])
    assert err < 2e-4, out  # second-order discretisation error at 32^3
