"""The C-ABI library builds, loads and exports every symbol its header
declares; argument validation runs on the host (no GPU needed)."""

import ctypes
import os
import re

import pytest

from openusct_gb300 import _lib, build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "usct_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(usct_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def test_header_declares_the_expected_entry_points():
    syms = declared_symbols()
    for s in ["usct_plan_create", "usct_forward_fmc", "usct_misfit_and_gradient",
              "usct_forward_fmc_dev", "usct_misfit_and_gradient_dev",
              "usct_gn_hessian_vector_dev", "usct_batch_backward", "usct_plain_bytes"]:
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_table_covers_the_header():
    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_plan_argument_validation_on_host(lib):
    p = ctypes.c_void_p()
    dims = (ctypes.c_int * 4)(8, 8, 8, 8)
    one = (ctypes.c_int * 2)(0, 1)
    cell = (ctypes.c_int64 * 1)(0)
    w = (ctypes.c_double * 1)(1.0)
    rc = lib.usct_plan_create(ctypes.byref(p), 4, dims, 1e-3, 1e-7, 10, 1, one, cell, w, 1, one,
                              cell, w, 0, 0, 0, 0, 0)
    assert rc == _lib.USCT_ERR_ARG
    assert b"ndim" in lib.usct_last_error()
    rc = lib.usct_plan_create(ctypes.byref(p), 3, dims, 1e-3, 1e-7, 10, 1, one, cell, w, 1, one,
                              cell, w, 3, 0, 0, 0, 0)
    assert rc == _lib.USCT_ERR_ARG and b"power of two" in lib.usct_last_error()
    assert lib.usct_version() >= 10000


def test_header_constants_match_the_bindings():
    text = open(HEADER).read()
    consts = dict(re.findall(r"#define (USCT_[A-Z_]+) \(?([0-9]+)", text))
    assert int(consts["USCT_SMOOTH_MAX_RADIUS"]) == _lib.SMOOTH_MAX_RADIUS
    assert int(consts["USCT_DOT_WS_DOUBLES"]) == _lib.DOT_WS_DOUBLES


def test_update_kernels_validate_arguments_on_host(lib):
    dims = (ctypes.c_int * 3)(4, 5, 6)
    taps = (ctypes.c_double * 70)(*([0.1] * 70))
    a, b, c = ctypes.c_void_p(4096), ctypes.c_void_p(8192), ctypes.c_void_p(12288)
    rc = lib.usct_smooth_dev(a, b, c, 3, dims, taps, _lib.SMOOTH_MAX_RADIUS + 1, None)
    assert rc == _lib.USCT_ERR_ARG and b"radius" in lib.usct_last_error()
    rc = lib.usct_smooth_dev(a, a, c, 3, dims, taps, 4, None)
    assert rc == _lib.USCT_ERR_ARG and b"distinct" in lib.usct_last_error()
    rc = lib.usct_smooth_dev(a, b, b, 3, dims, taps, 4, None)
    assert rc == _lib.USCT_ERR_ARG and b"distinct" in lib.usct_last_error()
    rc = lib.usct_smooth_dev(a, b, c, 4, dims, taps, 4, None)
    assert rc == _lib.USCT_ERR_ARG and b"ndim" in lib.usct_last_error()
    rc = lib.usct_model_trial_dev(a, 1.0, b, c, None, None, a, 10, None)
    assert rc == _lib.USCT_ERR_ARG and b"lo and hi" in lib.usct_last_error()
    assert lib.usct_vec_dot_dev(None, None, 10, a, None) == _lib.USCT_ERR_ARG


def test_cpp_example_compiles_and_links(tmp_path):
    """The plain C++ example (usct_example.cpp, the counterpart of the
    reference's example_main.cpp) builds against the header and library."""
    exe = build.build_example(str(tmp_path / "usct_example"))
    assert os.path.exists(exe) and os.access(exe, os.X_OK)
