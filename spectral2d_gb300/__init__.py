"""spectral2d_gb300 -- GB300 (sm_103a) time-step hot path of Spectral2D.

The vorticity-streamfunction right-hand side and the TVD-RK3 step run as
hand-written CUDA kernels in ``libspectral2d_gb300.so`` behind the C-ABI of
``include/s2d.h``.  This package is the Python host side over that ABI.
"""

from ._lib import S2DError, lib  # noqa: F401
from .solver import Ensemble, Spectral2D, get_grid_size, probe_fp64_peak, turbulent_ic_host  # noqa: F401

__all__ = ["Spectral2D", "Ensemble", "get_grid_size", "turbulent_ic_host", "probe_fp64_peak", "S2DError", "lib"]
