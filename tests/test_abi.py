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
