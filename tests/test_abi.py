"""The C-ABI library: builds for sm_103a, loads, and exports exactly the
entry points include/lbmpsm.h declares.  Without a GPU, creating a lattice
must fail with a CUDA error (no CPU fallback)."""
import os
import re

import pytest

import lbmpsm

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "lbmpsm.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(lbmpsm_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_the_binding_symbols():
    assert set(declared_functions()) == set(lbmpsm.SYMBOLS)


def test_library_exports_every_declared_symbol():
    lib = lbmpsm.load()
    missing = [s for s in declared_functions() if not hasattr(lib, s)]
    assert not missing, missing


def test_error_text_for_bad_arguments_without_touching_the_gpu():
    import ctypes as C
    lib = lbmpsm.load()
    p = lbmpsm.FixParams()
    p.dimension = 3
    p.prd = (C.c_double * 3)(8.0, 8.0, 8.0)
    p.periodic = (C.c_int * 3)(1, 1, 1)
    p.nevery, p.Nlc, p.lc, p.rho, p.nu, p.Re, p.tau = 1, 9, 8.0, 1.0, 0.1, 1.0, 0.5  # tau <= 0.5
    h = C.c_void_p()
    assert lib.lbmpsm_create(C.byref(p), None, C.byref(h)) == lbmpsm.ERR_ARG
    assert b"Illegal fix lbm-psm command" in lib.lbmpsm_last_error(None)
    p.tau, p.Re = 0.7, 1e6  # Mach > 0.3
    assert lib.lbmpsm_create(C.byref(p), None, C.byref(h)) == lbmpsm.ERR_MACH
    p.Re = 1.0
    p.prd = (C.c_double * 3)(8.5, 8.0, 8.0)  # not a multiple of dx
    assert lib.lbmpsm_create(C.byref(p), None, C.byref(h)) == lbmpsm.ERR_GRID


def test_no_cpu_fallback(has_gpu):
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(lbmpsm.LbmPsmError) as e:
        lbmpsm.Lattice(prd=(8, 8, 8), Nlc=9, lc=8.0, nu=0.2 / 3, Re=1.0)
    assert e.value.code in (lbmpsm.ERR_CUDA, lbmpsm.ERR_NOMEM)


def test_group_and_sensitivity_argument_checks_without_touching_the_gpu():
    import ctypes as C
    lib = lbmpsm.load()
    g = C.c_void_p()
    assert lib.lbmpsm_group_create(None, 0, C.byref(g)) == lbmpsm.ERR_ARG
    assert b"at least one lattice" in lib.lbmpsm_last_error(None)
    arr = (C.c_void_p * 2)(None, None)
    assert lib.lbmpsm_group_create(arr, 2, C.byref(g)) == lbmpsm.ERR_ARG
    assert lib.lbmpsm_group_run_fixed(None, 1) == lbmpsm.ERR_ARG
    assert lib.lbmpsm_group_collide_launches(None) == -1
    assert lib.lbmpsm_host_direct(None) == -1
    assert lib.lbmpsm_group_tune_ms(None, None) == lbmpsm.ERR_ARG
    assert lib.lbmpsm_adjoint_drag(None, 0, None, None, None, None, None, 10, 1, 10, None, 5,
                                   1e-4, None, None, None, None, None) == lbmpsm.ERR_ARG
    assert lib.lbmpsm_tangent_drag(None, 0, None, None, None, None, None, 10, 1, 10, None, 1e-4,
                                   0.0, None, None, None, None) == lbmpsm.ERR_ARG
