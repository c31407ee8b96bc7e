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


@pytest.mark.gpu
def test_shim_mgsolve(tmp_path):
    exe = _build(tmp_path)
    out = subprocess.run([str(exe), str(ROOT / "tests" / "golden" / "mg_params.yaml")],
                         capture_output=True, text=True, check=True).stdout
    line = [l for l in out.splitlines() if l.startswith("mgSolve")][0]
    err = float(line.split()[-1])
    assert err < 2e-4, out  # second-order discretisation error at 32^3
