"""The forward FMC entry point that allocates no device memory.

It exists for callers that may not allocate device memory themselves -- a
host application whose GPU memory is owned by its own pool allocator, a plugin
inside such a host, a real-time loop that must not enter the CUDA allocator.
Its scratch is a fixed static device array inside the library, so the check
here is that it returns exactly what the regular, workspace-based entry point
returns (the same stencil in the same op order: bit for bit), on calls in a
row (each later, smaller problem must not see anything left over from the one
before), with and without a sponge; that a problem too large for the static
array, or with a missing entry array, is refused with a clear error before any
device work; and that a call on a capturing stream is refused.

This file is collected last on purpose.
"""

import ctypes

import numpy as np
import pytest

from golden_util import load
from openusct_gb300 import _lib
from openusct_gb300.geometry import element_csr


def _call(lib, c, m_dev, sp_dev, wav_dev, out_dev, stream):
    shape = c["m_true"].shape
    tx, rx = element_csr(c.geom, shape, c.src_list, c.footprints)
    dims = (ctypes.c_int * len(shape))(*shape)
    return lib.usct_forward_fmc_noalloc(
        len(shape), dims, c.h, c.dt, c.nt, tx.rows, tx.ptr.ctypes.data_as(_lib._ip),
        tx.cell.ctypes.data_as(_lib._lp), tx.w.ctypes.data_as(_lib._dp), rx.rows,
        rx.ptr.ctypes.data_as(_lib._ip), rx.cell.ctypes.data_as(_lib._lp),
        rx.w.ctypes.data_as(_lib._dp), m_dev, sp_dev, wav_dev, out_dev, stream)


def test_noalloc_refuses_problems_larger_than_its_static_area_and_missing_arrays():
    from openusct_gb300 import build
    build.build()
    lib = _lib.load()
    dims = (ctypes.c_int * 3)(192, 192, 192)
    one = (ctypes.c_int * 2)(0, 1)
    cell = (ctypes.c_int64 * 1)(1000)
    w = (ctypes.c_double * 1)(1.0)
    dummy = ctypes.c_void_p(256)   # never dereferenced: the host-side checks come first
    rc = lib.usct_forward_fmc_noalloc(3, dims, 2e-4, 4e-8, 2000, 1, one, cell, w, 1, one, cell, w,
                                      dummy, None, dummy, dummy, None)
    assert rc == _lib.USCT_ERR_ARG
    assert b"static no-alloc area" in lib.usct_last_error()
    small = (ctypes.c_int * 2)(16, 16)
    for txc, txw, rxc, rxw in ((None, w, cell, w), (cell, None, cell, w), (cell, w, None, w),
                               (cell, w, cell, None)):
        rc = lib.usct_forward_fmc_noalloc(2, small, 1e-3, 1e-7, 10, 1, one, txc, txw, 1, one, rxc,
                                          rxw, dummy, None, dummy, dummy, None)
        assert rc == _lib.USCT_ERR_ARG
        assert b"null" in lib.usct_last_error()


@pytest.mark.gpu
def test_noalloc_forward_equals_workspace_entry_point_on_calls_in_a_row():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    from openusct_gb300 import build
    import openusct_gb300.backend as gb
    build.build()
    lib = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # a 3D problem, then smaller 2D ones (footprint elements; a sponge)
    for name in ("gpu3d", "ring2d_aperture", "ring2d_sponge"):
        c = load(name)
        m = torch.from_numpy(c["m_true"]).cuda()
        wav = torch.from_numpy(c.wavelet).cuda()
        sp = torch.from_numpy(np.ascontiguousarray(c.sponge, np.float64)).cuda() \
            if c.sponge is not None else None
        ref = gb.forward_fmc(m, c.geom, c.wavelet, c.dt, c.h, c.nt, sp, c.src_list,
                             c.footprints).cpu().numpy()
        out = torch.full(ref.shape, float("nan"), dtype=torch.float32, device="cuda")
        _lib.check(_call(lib, c, ctypes.c_void_p(m.data_ptr()),
                         ctypes.c_void_p(sp.data_ptr()) if sp is not None else None,
                         ctypes.c_void_p(wav.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                         stream))
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert np.array_equal(got, ref), name


@pytest.mark.gpu
def test_noalloc_refuses_a_capturing_stream():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    from openusct_gb300 import build
    build.build()
    lib = _lib.load()
    c = load("ring2d_point")
    m = torch.from_numpy(c["m_true"]).cuda()
    wav = torch.from_numpy(c.wavelet).cuda()
    out = torch.empty((len(c.src_list), c.nt, len(c.geom.idx)), dtype=torch.float32,
                      device="cuda")
    side = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    rc = None
    torch.cuda.synchronize()
    with torch.cuda.graph(graph, stream=side):
        rc = _call(lib, c, ctypes.c_void_p(m.data_ptr()), None, ctypes.c_void_p(wav.data_ptr()),
                   ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(side.cuda_stream))
        out.zero_()   # something to capture, so the graph is not empty
    assert rc == _lib.USCT_ERR_ARG
    assert b"capturing" in lib.usct_last_error()
