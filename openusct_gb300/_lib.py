"""ctypes binding of ``libusct_gb300.so`` (the C ABI in ``include/usct_gb300.h``).

The library is loaded from the package directory only.  If it is missing the
import of any compute entry point fails loudly: there is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import os
import threading

from .build import LIB

_lock = threading.Lock()
_lib = None

USCT_OK = 0
USCT_ERR_ARG = 1
USCT_ERR_CUDA = 2
USCT_ERR_NOMEM = 3
USCT_ERR_STATE = 4

MODE_FORWARD = 0
MODE_GRADIENT = 1
MODE_BORN = 2

SMOOTH_MAX_RADIUS = 64      # USCT_SMOOTH_MAX_RADIUS
DOT_WS_DOUBLES = 609        # USCT_DOT_WS_DOUBLES

INFO = {"batch": 0, "nbatch": 1, "ckpt_k": 2, "nseg": 3, "tile_x": 4, "tile_y": 5,
        "zchunk": 6, "level_floats": 7, "launches": 8, "variant": 9, "tblock": 10}
SET = {"variant": 0, "stages": 1, "stages_adj": 2, "graphs": 3, "wait_test": 4, "tblock": 5,
       "tblock_stages": 6, "tblock_zchunk": 7}

_vp = ctypes.c_void_p
_i = ctypes.c_int
_d = ctypes.c_double
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_int64)
_dp = ctypes.POINTER(ctypes.c_double)

# name -> (restype, argtypes); every symbol of include/usct_gb300.h
SIGNATURES = {
    "usct_last_error": (ctypes.c_char_p, []),
    "usct_version": (_i, []),
    "usct_plan_create": (_i, [ctypes.POINTER(_vp), _i, _ip, _d, _d, _i, _i, _ip, _lp, _dp, _i, _ip,
                              _lp, _dp, _i, _i, _i, _i, _i]),
    "usct_plan_destroy": (None, [_vp]),
    "usct_plan_info": (_i, [_vp, _i, _lp]),
    "usct_plan_set": (_i, [_vp, _i, ctypes.c_int64]),
    "usct_plan_check": (_i, [_vp, _vp]),
    "usct_model_bytes": (ctypes.c_size_t, [_vp]),
    "usct_batch_bytes": (ctypes.c_size_t, [_vp, _i]),
    "usct_model_prepare": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "usct_batch_forward": (_i, [_vp, _vp, _vp, _i, _i, _vp, _vp]),
    "usct_batch_misfit": (_i, [_vp, _vp, _i, _vp, _vp, _vp]),
    "usct_batch_misfit_mt": (_i, [_vp, _vp, _i, _vp, _i, _vp, _vp]),
    "usct_batch_misfit_tw": (_i, [_vp, _vp, _i, _vp, _vp, _i, _vp, _vp]),
    "usct_batch_adjoint_source": (_i, [_vp, _vp, _i, _vp, _vp]),
    "usct_batch_backward": (_i, [_vp, _vp, _vp, _i, _vp]),
    "usct_model_gradient": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "usct_forward_fmc_dev": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "usct_misfit_and_gradient_dev": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "usct_misfit_and_gradient_mt_dev": (_i, [_vp, _vp, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp,
                                             _vp]),
    "usct_misfit_and_gradient_tw_dev": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _i, _vp, _vp, _vp,
                                             _vp, _vp]),
    "usct_gn_hessian_vector_dev": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "usct_smooth_dev": (_i, [_vp, _vp, _vp, _i, _ip, _dp, _i, _vp]),
    "usct_vec_mul_dev": (_i, [_vp, _vp, _vp, ctypes.c_size_t, _vp]),
    "usct_vec_axpy_dev": (_i, [_vp, _d, _vp, _vp, ctypes.c_size_t, _vp]),
    "usct_model_trial_dev": (_i, [_vp, _d, _vp, _vp, _vp, _vp, _vp, ctypes.c_size_t, _vp]),
    "usct_vec_absmax_dev": (_i, [_vp, ctypes.c_size_t, _vp, _vp]),
    "usct_vec_dot_dev": (_i, [_vp, _vp, ctypes.c_size_t, _vp, _vp]),
    "usct_analytic_dev": (_i, [_vp, _vp, _i, _i, _i, _vp, _vp]),
    "usct_tfm_dev": (_i, [_vp, _i, _i, _i, _vp, _vp, _i, _vp, _i, _d, _d, _vp, _vp, _vp]),
    "usct_pwindow_dev": (_i, [_vp, _i, _i, _i, _d, _d, _d, _vp, _vp]),
    "usct_plain_bytes": (ctypes.c_size_t, [_vp, _i]),
    "usct_plain_forward_fmc_dev": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "usct_plain_misfit_and_gradient_dev": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "usct_forward_fmc": (_i, [_dp, _ip, _i, _d, _d, _i, _ip, _i, _ip, _i, _dp, _dp]),
    "usct_misfit_and_gradient": (_i, [_dp, _ip, _i, _d, _d, _i, _ip, _i, _ip, _i, _dp, _dp, _dp,
                                      _dp]),
    "usct_misfit_and_gradient_mt": (_i, [_dp, _ip, _i, _d, _d, _i, _ip, _i, _ip, _i, _dp, _dp,
                                         _dp, _i, _dp]),
    "usct_plan_set_channel_models": (_i, [_vp, _i, _ip]),
    "usct_model_prepare_channels": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "usct_forward_fmc_noalloc": (_i, [_i, _ip, _d, _d, _i, _i, _ip, _lp, _dp, _i, _ip, _lp, _dp,
                                      _vp, _vp, _vp, _vp, _vp]),
}


class USCTError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code, message):
        super().__init__(f"usct error {code}: {message}")
        self.code = code


class USCTMemoryError(USCTError, MemoryError):
    pass


def load():
    """Load the library (building it first if the sources are newer)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB):
                raise ImportError(
                    f"{LIB} is missing: build it with `python -c 'import __graft_entry__ as g; "
                    "g.build()'` (the CUDA extension is required; there is no CPU fallback)")
            lib = ctypes.CDLL(LIB)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def check(code):
    if code != USCT_OK:
        msg = load().usct_last_error().decode(errors="replace")
        if code == USCT_ERR_NOMEM:
            raise USCTMemoryError(code, msg)
        if code == USCT_ERR_ARG:
            raise ValueError(f"usct: {msg}")
        raise USCTError(code, msg)
