"""CPU oracle for the Spectral2D time-step hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product path (``spectral2d_gb300``)
imports this package.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may use it, and
only as the checker or as the timed CPU baseline.

Parity status: the reference (Fortran 2003 + FFTW-MPI 3.3.3 + parallel HDF5)
cannot be compiled in this environment (no Fortran compiler, no FFTW, no MPI),
and it ships no tests, fixtures or golden vectors.  The oracle is pinned
instead by (1) exact rational-arithmetic golden vectors of the reference's
RHS algorithm (cyclic convolution on the 3/2 grid, ``tests/golden``), and
(2) the analytic Taylor-Green decay that the reference's own verification
script uses (analysis/TaylorGreen.py:88-96).
"""

from .spectral_oracle import *  # noqa: F401,F403
