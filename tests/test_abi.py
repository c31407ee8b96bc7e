"""The C-ABI library loads on a machine without a GPU and exports every
entry point include/saras_gb300.h declares; entry points that need no device
answer on the CPU, and device entry points fail with a status, not a crash."""
import ctypes as C

import saras_gb300 as S


def test_library_exports_header_symbols():
    lib = S.load()
    names = S.exported_symbols()
    assert "saras_mg_solve" in names and "saras_rk3_step" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings():
    lib = S.load()
    assert lib.saras_status_string(S.NOT_CONVERGED) == b"NOT_CONVERGED"
    assert lib.saras_status_string(S.BAD_ARG) == b"BAD_ARG"


def test_default_params_match_parameters_yaml():
    lib = S.load()
    p = S.MgParams()
    lib.saras_mg_default_params(C.byref(p))
    q = S.mg_params()
    for f, _ in S.MgParams._fields_:
        a, b = getattr(p, f), getattr(q, f)
        if f == "bc_kind":
            assert list(a) == list(b)
        else:
            assert a == b, f


def test_rbc_coefficients():
    nu, ka, fb = S.rbc_coefficients(2, 1e7, 1.0)
    assert abs(nu - (1.0 / 1e7) ** 0.5) < 1e-18 and abs(ka - (1.0 / 1e7) ** 0.5) < 1e-18 and fb == 1.0
    nu, ka, fb = S.rbc_coefficients(1, 1e4, 0.71)
    assert nu == 0.71 and ka == 1.0 and fb == 1e4 * 0.71


def test_struct_layout():
    # sizes the C compiler gives the header structs on LP64 targets
    assert C.sizeof(S.GridDesc) == 96
    assert C.sizeof(S.FieldBC) == 24 + 48


def test_struct_layout_matches_c_compiler(tmp_path):
    """Every header struct has the size and field offsets the C compiler
    gives it (the ctypes mirrors are what the Python side passes)."""
    import shutil
    import subprocess
    if not shutil.which("gcc"):
        import pytest
        pytest.skip("no C compiler")
    structs = {"saras_grid_desc": S.GridDesc, "saras_mg_params": S.MgParams, "saras_field_bc": S.FieldBC,
               "saras_rk3_params": S.Rk3Params, "saras_serve_params": S.ServeParams,
               "saras_serve_stats": S.ServeStats, "saras_run_params": S.RunParams,
               "saras_tseries_row": S.TseriesRow}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "saras_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    inc = S.HERE.parent / "include"
    subprocess.run(["gcc", "-I", str(inc), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {(a, b): int(c) for a, b, c in (l.split() for l in out if l)}
    for cname, py in structs.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)
