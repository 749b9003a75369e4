"""The allocation-free right-hand side, s2d_compute_rhs_noalloc.

It serves callers that must not allocate device memory (their device memory
belongs to another runtime or pool, or an allocation is not allowed on their
code path): the caller passes device input and output arrays and the library
uses only its static device scratch array.

The tests call it through the C-ABI:
  * twice in a row on two different states, each result against the
    handle-based entry point s2d_compute_rhs (relative L2 1e-13, the
    tolerance of the RHS parity tests);
  * over the size sequence 64, 128, 64, 256, 96, 96, so that the cached
    twiddle and 1/k^2 tables are replaced when nx changes, reused when it
    does not, and the largest size the static array holds
    (S2D_NOALLOC_MAX_NX = 256) runs -- each result against the oracle's
    ComputeRHS (src/Spectral.F90:396-482) directly, relative L2 1e-13;
  * with sizes beyond the static array and null arrays, which it rejects.

This file sorts last so that a run stopping at the first failure has already
run every other test; it passes alone in a fresh process as well.
"""

import ctypes as C

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _noalloc_rhs(lib, torch, n, nu, w):
    g = O.get_grid_size(n, n)
    w_dev = torch.from_numpy(w.view(np.float64).copy()).cuda()
    dW_dev = torch.full_like(w_dev, float("nan"))
    torch.cuda.synchronize()
    rc = lib.s2d_compute_rhs_noalloc(n, nu, C.c_void_p(w_dev.data_ptr()), C.c_void_p(dW_dev.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    return dW_dev.cpu().numpy().view(np.complex128).reshape(g.nyG, g.cISize)


def test_noalloc_rhs_matches_handle_rhs_on_two_calls(built_lib):
    torch = pytest.importorskip("torch")
    from spectral2d_gb300 import Spectral2D, _lib as L

    lib = L.lib()
    n, nu = 64, 0.01
    g = O.get_grid_size(n, n)
    torch.cuda.set_device(0)
    for seed in (5, 6):
        w = O.truncate(O.random_state(g, seed), g)
        with Spectral2D(n, nu=nu) as s:
            s.set_state(w)
            expected = s.compute_rhs()
        got = _noalloc_rhs(lib, torch, n, nu, w)
        assert O.rel_l2(got, expected) < 1e-13


def test_noalloc_rhs_vs_oracle_over_changing_sizes(built_lib):
    torch = pytest.importorskip("torch")
    from spectral2d_gb300 import _lib as L

    lib = L.lib()
    nu = 0.003
    torch.cuda.set_device(0)
    for i, n in enumerate([64, 128, 64, 256, 96, 96]):
        g = O.get_grid_size(n, n)
        w = O.truncate(O.random_state(g, 40 + i), g)
        psi = O.truncate(O.compute_psi(w, g), g)
        ref, _ = O.compute_rhs(w, psi, g, nu, round_trip=False)
        got = _noalloc_rhs(lib, torch, n, nu, w)
        err = O.rel_l2(got, O.truncate(ref, g))
        assert np.all(np.isfinite(got)), n
        # modes outside |k| <= n/2 are written as zero
        assert np.all(got[O.truncation_mask(g)] == 0), n
        assert err < 1e-13, (n, err)


def test_noalloc_rejects_sizes_beyond_the_static_scratch(built_lib):
    from spectral2d_gb300 import _lib as L

    lib = L.lib()
    dummy = C.c_void_p(16)   # never dereferenced: the size check comes first
    assert lib.s2d_compute_rhs_noalloc(512, 0.01, dummy, dummy, None) == L.S2D_ERR_INVALID
    assert lib.s2d_compute_rhs_noalloc(264, 0.01, dummy, dummy, None) == L.S2D_ERR_INVALID
    assert lib.s2d_compute_rhs_noalloc(12, 0.01, dummy, dummy, None) == L.S2D_ERR_INVALID
    assert lib.s2d_compute_rhs_noalloc(64, 0.01, None, None, None) == L.S2D_ERR_INVALID
