"""The C-ABI library builds for sm_103a, loads without a GPU, and exports every
function include/blademaster_gb300.h declares with the header's struct sizes.
No compute call is made here."""

import ctypes

from blademaster_gb300 import _native


def test_library_exports_every_declared_symbol():
    lib = _native.lib()
    declared = _native.exported_symbols()
    assert len(declared) >= 30
    missing = [name for name in declared if not hasattr(lib, name)]
    assert not missing, missing


def test_struct_layouts_match_the_header():
    lib = _native.lib()
    assert lib.bm_params_size() == ctypes.sizeof(_native.Params)
    assert lib.bm_buffers_size() == ctypes.sizeof(_native.Buffers)
    assert lib.bm_step_args_size() == ctypes.sizeof(_native.StepArgs)
    assert b"sm_103a" in lib.bm_version()


def test_invalid_arguments_fail_with_a_message():
    lib = _native.lib()
    p = _native.Params()
    b = _native.Buffers()
    handle = ctypes.c_void_p()
    rc = lib.bm_solver_create(ctypes.byref(p), ctypes.byref(b), ctypes.byref(handle))
    assert rc == 1 and b"invalid sizes" in lib.bm_last_error()
    assert lib.bm_blade_query(None, -1, None, 0.0, None, None, None, None) == 1


def test_solver_refuses_a_cpu_device():
    import pytest
    from blademaster_gb300.solver import Solver, Config

    with pytest.raises(ValueError, match="CUDA device required"):
        Solver(Config(), device="cpu")
