"""The turbulent initial condition computed on the device (s2d_set_turbulent)
against the library's host generator (s2d_turbulent_ic_host) and the oracle
(set_turbulent), which restate FourierVelocity (src/SetIC.F90:175-364).

The device and host generators do the same FP64 operations in the same
order; they differ only where the device's exp / sin / cos and the order of
the TKE sum (a fixed-order device reduction against a host loop) round
differently, so omega agrees to a relative L2 of 1e-15.  The FP32 handle
holds the FP64 result rounded once (relative L2 within 1e-7).
"""

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

CASES = [(16, "k4gauss", 2.0, 0.5), (64, "k4gauss", 10.0, 0.5), (256, "schumann", 4.0, 0.5),
         (512, "k4gauss", 10.0, 0.0), (2048, "k4gauss", 10.0, 0.5)]


@pytest.mark.parametrize("nx,spectrum,k0,tke", CASES)
def test_device_ic_matches_host_generator(built_lib, nx, spectrum, k0, tke):
    from spectral2d_gb300 import Spectral2D
    from spectral2d_gb300.solver import turbulent_ic_host
    seed = 11 + nx
    host = turbulent_ic_host(nx, seed, spectrum, k0, 1.0, tke)
    with Spectral2D(nx, nu=1e-3) as s:
        s.set_turbulent_velocity(seed=seed, spectrum=spectrum, k0=k0, tke=tke)
        dev, psi = s.get_state()
    g = O.get_grid_size(nx, nx)
    err = O.rel_l2(dev, host)
    assert err < 1e-15, err
    # zero outside the retained set, Hermitian kx = 0 column, no mean mode
    assert np.all(dev[O.truncation_mask(g)] == 0)
    assert dev[0, 0] == 0
    K = nx // 2
    for ky in range(1, K + 1):
        assert dev[g.nyG - ky, 0] == np.conj(dev[ky, 0])
    if tke > 0:
        with Spectral2D(nx, nu=1e-3) as s:
            s.set_state(dev)
            _, _, t, _, _ = s.compute_spectrum()
        assert abs(t - tke) < 1e-13 * tke


@pytest.mark.parametrize("spectrum,kind", [("k4gauss", O.SPECTRUM_K4_GAUSS), ("schumann", O.SPECTRUM_SCHUMANN)])
def test_device_ic_matches_oracle(built_lib, spectrum, kind):
    from spectral2d_gb300 import Spectral2D
    nx, seed, k0 = 128, 3, 6.0
    g = O.get_grid_size(nx, nx)
    wo, _ = O.set_turbulent(g, seed, kind=kind, k0=k0, urms=1.0, tke_target=0.5)
    with Spectral2D(nx, nu=1e-3) as s:
        s.set_turbulent_velocity(seed=seed, spectrum=spectrum, k0=k0, tke=0.5)
        dev, _ = s.get_state()
    assert O.rel_l2(dev, wo) < 1e-14


def test_device_ic_fp32_is_the_fp64_ic_rounded(built_lib):
    from spectral2d_gb300 import Spectral2D
    from spectral2d_gb300.solver import turbulent_ic_host
    nx, seed = 256, 5
    host = turbulent_ic_host(nx, seed, "k4gauss", 10.0, 1.0, 0.5)
    with Spectral2D(nx, nu=1e-3, precision="fp32") as s:
        s.set_turbulent_velocity(seed=seed, spectrum="k4gauss", k0=10.0, tke=0.5)
        dev, _ = s.get_state()
    assert O.rel_l2(dev, host) < 1e-7
