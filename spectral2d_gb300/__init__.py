"""spectral2d_gb300 -- GB300 (sm_103a) time-step hot path of Spectral2D.

The vorticity-streamfunction right-hand side and the TVD-RK3 step run as
hand-written CUDA kernels in ``libspectral2d_gb300.so`` behind the C-ABI of
``include/s2d.h``.  This package is the Python host side over that ABI.
"""

from ._lib import S2DError, lib  # noqa: F401
from .solver import (ClosureNet, Ensemble, Spectral2D, filter_state, get_grid_size,  # noqa: F401
                     les_integrate_steps, les_set_closure, les_time_steps, probe_fp64_peak, subgrid_flux,
                     turbulent_ic_host)

__all__ = ["Spectral2D", "Ensemble", "get_grid_size", "turbulent_ic_host", "probe_fp64_peak", "S2DError", "lib"]
