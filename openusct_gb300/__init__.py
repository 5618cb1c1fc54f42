"""openusct_gb300 -- GB300-native acoustic FWI hot path for openUSCT.

The forward leapfrog solve, its exact discrete adjoint and the squared-
slowness gradient of simulation/ringfwi/fwi.py, run over every transmit of a
full-matrix capture by hand-written sm_103a CUDA kernels behind the C ABI of
include/usct_gb300.h.

    import openusct_gb300.backend as gb300     # drop-in ``backend=`` module
    J, g = gb300.misfit_and_gradient(m, geom, wavelet, dt, h, nt, dobs)
"""

from .build import LIB  # noqa: F401

__all__ = ["backend", "geometry", "build"]
__version__ = "0.1.0"
