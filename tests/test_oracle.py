"""CPU tests of the oracle itself: it must reproduce the exact golden vectors
(tests/golden, exact rational arithmetic of the reference's algorithm) and the
analytic Taylor-Green decay the reference's own verification script uses
(analysis/TaylorGreen.py:88-96)."""

import math
import os

import numpy as np
import pytest

import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("n", [8, 16])
@pytest.mark.parametrize("round_trip", [True, False])
def test_rhs_matches_exact_golden(n, round_trip):
    d = np.load(os.path.join(GOLD, f"rhs_exact_n{n}.npz"))
    g = O.get_grid_size(n, n)
    w = d["w"]
    dW, _ = O.compute_rhs(w, O.compute_psi(w, g), g, float(d["nu"]), round_trip=round_trip)
    assert O.rel_l2(O.truncate(dW, g), d["dW"]) < 2e-15
    # dW outside the circle is -nu k^2 w of the round-tripped w: round-off only
    assert np.abs(dW[O.truncation_mask(g)]).max() < 1e-13


def test_one_step_matches_exact_golden():
    d = np.load(os.path.join(GOLD, "step_exact_n8.npz"))
    g = O.get_grid_size(8, 8)
    w = d["w"]
    w1, p1 = O.integrate_one_step(w, O.truncate(O.compute_psi(w, g), g), g,
                                  float(d["nu"]), float(d["dt"]))
    assert O.rel_l2(w1, d["w_new"]) < 2e-15
    assert O.rel_l2(p1, d["psi_new"]) < 2e-15


def test_grid_size_reference_default():
    # the driver's defaults: nx = ny = 96 with the 3/2 rule (src/Spectral2D.F90:73-82)
    g = O.get_grid_size(96, 96)
    assert (g.nxG, g.nyG, g.cISize, g.rISize) == (144, 144, 73, 146)
    assert (g.kxMG, g.kyMG, g.kyLG, g.kMax) == (72, 72, -71, 48.0)
    assert g.kyG[72] == 72 and g.kyG[73] == -71
    assert g.xMaskInd == 72 and g.yMaskInd == 72


@pytest.mark.parametrize("n", [8, 96, 256])
def test_truncation_is_the_circle(n):
    g = O.get_grid_size(n, n)
    k2 = g.kx ** 2 + g.ky ** 2
    assert np.array_equal(O.truncation_mask(g), k2 > (n // 2) ** 2)


def test_single_mode_operators():
    g = O.get_grid_size(16, 16)
    w = np.zeros((g.nyG, g.cISize), complex)
    w[3, 2] = 1.0 + 2.0j          # kx=2, ky=3
    psi = O.compute_psi(w, g)
    assert psi[3, 2] == (1.0 + 2.0j) / 13.0
    u, v = O.compute_velocity(psi, g)
    assert np.isclose(u[3, 2], 1j * 3 * psi[3, 2]) and np.isclose(v[3, 2], -1j * 2 * psi[3, 2])
    assert np.allclose(O.compute_vorticity(u, v, g), w)


def test_binary_search_vectorised_matches_literal():
    g = O.get_grid_size(16, 16)
    edges, _ = O.spectrum_bin_edges(g)
    rng = np.random.default_rng(0)
    f = np.concatenate([rng.uniform(0, edges[-1], 500), edges, [edges[-1]]])
    lit = np.array([O.binary_search(edges, x) for x in f])
    assert np.array_equal(O.binary_search_vec(edges, f), lit)


def test_taylor_green_analytic_decay():
    """RK3 of the TG vortex against exp(-2 nu t) in spectral and physical space."""
    g = O.get_grid_size(32, 32)
    nu, dt, n = 0.01, 1e-3, 200
    w, psi = O.set_taylor_green(g)
    w0 = O.truncate(w, g)
    for _ in range(n):
        w, psi = O.integrate_one_step(w, psi, g, nu, dt)
    F = math.exp(-2.0 * nu * n * dt)
    assert O.rel_l2(w, w0 * F) < 1e-11
    psiE, wE, uE, vE = O.taylor_green_exact(g, nu, n * dt)
    wN = O.transform_c2r(w, g)
    dx = 2 * np.pi / g.nxG
    assert O.l2_error(dx, dx, wE, wN) < 1e-11
    assert O.linf_error(wE, wN) < 1e-11


def test_turbulent_ic_properties():
    g = O.get_grid_size(64, 64)
    w, psi = O.set_turbulent(g, seed=3, kind=O.SPECTRUM_K4_GAUSS, k0=10.0, tke_target=0.5)
    _, Ek, tke, _, _ = O.spectrum_of_vorticity(w, g, 0.0)
    assert abs(tke - 0.5) < 1e-14
    # Hermitian kx=0 column and zero mean
    for ky in range(1, 33):
        assert w[(-ky) % g.nyG, 0] == np.conj(w[ky, 0])
    assert w[0, 0] == 0
    # physical field is real: C2R -> R2C returns the state
    rt = O.transform_r2c(O.transform_c2r(w, g), g)
    assert O.rel_l2(rt, w) < 1e-14
    # seeded: reproducible, and a different seed differs
    w2, _ = O.set_turbulent(g, seed=3)
    w3, _ = O.set_turbulent(g, seed=4)
    assert np.array_equal(w, w2) and not np.allclose(w, w3)


def test_inviscid_energy_conservation_of_rhs():
    """With nu = 0 the nonlinear term conserves energy up to the aliasing of
    the kept |k| = N/2 modes; for a field without those modes it is exact."""
    g = O.get_grid_size(32, 32)
    w = O.random_state(g, 5, decay=0.3)
    w[:, 16] = 0
    w[16, :] = 0
    w[(-16) % g.nyG, :] = 0
    psi = O.compute_psi(w, g)
    dW, _ = O.compute_rhs(w, psi, g, 0.0, round_trip=False)
    wt = np.where(g.kxG[None, :] == 0, 1.0, 2.0)
    dE = np.sum(wt * (np.conj(psi) * dW).real)       # d/dt of energy
    dZ = np.sum(wt * (np.conj(w) * dW).real)         # d/dt of enstrophy
    scale = np.sum(wt * np.abs(psi) * np.abs(dW))
    assert abs(dE) / scale < 1e-13
    assert abs(dZ) / np.sum(wt * np.abs(w) * np.abs(dW)) < 1e-13
