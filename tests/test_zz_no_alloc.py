"""The forward FMC entry point that allocates no device memory.

It exists for callers that may not allocate device memory themselves -- a
host application whose GPU memory is owned by its own pool allocator, a plugin
inside such a host, a real-time loop that must not enter the CUDA allocator.
Its scratch is a fixed static device array inside the library, so the check
here is that it returns exactly what the regular, workspace-based entry point
returns, on two calls in a row (the second, smaller problem must not see
anything left over from the first), and that a problem too large for the
static array is refused with a clear error before any device work.

This file is collected last on purpose.
"""

import ctypes

import numpy as np
import pytest

from golden_util import load, rel_l2
from openusct_gb300 import _lib
from openusct_gb300.geometry import element_csr


def _call(lib, c, m_dev, wav_dev, out_dev, stream):
    shape = c["m_true"].shape
    tx, rx = element_csr(c.geom, shape, c.src_list, c.footprints)
    dims = (ctypes.c_int * len(shape))(*shape)
    return lib.usct_forward_fmc_noalloc(
        len(shape), dims, c.h, c.dt, c.nt, tx.rows, tx.ptr.ctypes.data_as(_lib._ip),
        tx.cell.ctypes.data_as(_lib._lp), tx.w.ctypes.data_as(_lib._dp), rx.rows,
        rx.ptr.ctypes.data_as(_lib._ip), rx.cell.ctypes.data_as(_lib._lp),
        rx.w.ctypes.data_as(_lib._dp), m_dev, None, wav_dev, out_dev, stream)


def test_noalloc_refuses_problems_larger_than_its_static_area():
    from openusct_gb300 import build
    build.build()
    lib = _lib.load()
    dims = (ctypes.c_int * 3)(192, 192, 192)
    one = (ctypes.c_int * 2)(0, 1)
    cell = (ctypes.c_int64 * 1)(1000)
    w = (ctypes.c_double * 1)(1.0)
    dummy = ctypes.c_void_p(256)   # never dereferenced: the size check comes first
    rc = lib.usct_forward_fmc_noalloc(3, dims, 2e-4, 4e-8, 2000, 1, one, cell, w, 1, one, cell, w,
                                      dummy, None, dummy, dummy, None)
    assert rc == _lib.USCT_ERR_ARG
    assert b"static no-alloc area" in lib.usct_last_error()


@pytest.mark.gpu
def test_noalloc_forward_matches_workspace_entry_point_twice():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    from openusct_gb300 import build
    import openusct_gb300.backend as gb
    build.build()
    lib = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for name in ("gpu3d", "ring2d_aperture"):   # a 3D problem, then a smaller 2D one
        c = load(name)
        m = torch.from_numpy(c["m_true"]).cuda()
        wav = torch.from_numpy(c.wavelet).cuda()
        ref = gb.forward_fmc(m, c.geom, c.wavelet, c.dt, c.h, c.nt, None, c.src_list,
                             c.footprints).cpu().numpy()
        out = torch.full(ref.shape, float("nan"), dtype=torch.float32, device="cuda")
        _lib.check(_call(lib, c, ctypes.c_void_p(m.data_ptr()), ctypes.c_void_p(wav.data_ptr()),
                         ctypes.c_void_p(out.data_ptr()), stream))
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel_l2(got, ref) <= 1e-5     # the trace tolerance of the parity tests
        assert rel_l2(got, c["dobs"]) <= 1e-5
