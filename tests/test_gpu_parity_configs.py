"""GPU-vs-oracle parity at the sizes and parameters of the benchmark
configurations, over 1000 steps (the reference's long-run bar is a relative
L2 of 1e-9 in omega after 1000 steps, its one-step bar 1e-12).

* Decaying turbulence at N = 512 (768^2 collocation grid, the 3 * 2^k
  transform family of the 2048^2 workload), nu = 1e-4 (the 2048^2 workload's
  viscosity), dt from CFL 0.5 of the seeded k^4 exp(-2(k/10)^2) initial
  condition: GPU against the oracle run with and without the reference's
  omega round trip (src/Spectral.F90:435,453).
* Taylor-Green at N = 256, nu = 0.01, dt = 1e-3, 1000 steps (t = 1): GPU
  against the oracle's trajectory, beside the analytic check of
  test_gpu_parity.py.
* The 2048^2 decaying-turbulence workload itself, 1000 steps: opt-in
  (S2D_SLOW_PARITY=1), since the oracle needs about 11 minutes on 16 cores.

The oracle integrates src/TimeIntegration.F90:130-210 with
src/Spectral.F90:396-482 in numpy (FP64, pocketfft).
"""

import os

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S2D(built_lib):
    from spectral2d_gb300 import Spectral2D
    O.set_workers(O.cpu_count())
    return Spectral2D


def _oracle_state(w, g):
    w = O.truncate(w, g)
    return w, O.truncate(O.compute_psi(w, g), g)


def _turbulence_run(S2D, n, nu, steps, seed, checkpoints):
    """GPU states after each step count in checkpoints (ascending), from the
    seeded initial condition, with the CFL-0.5 dt of that state."""
    out = {}
    with S2D(n, nu=nu) as s:
        s.set_turbulent_velocity(seed=seed, spectrum="k4gauss", k0=10.0, tke=0.5)
        w0, _ = s.get_state()
        dt = s.compute_time_step(0.5)
        done = 0
        for c in checkpoints:
            s.integrate_steps(c - done, dt)
            done = c
            s.check_finite()
            out[c] = s.get_state()[0]
    return w0, dt, out


def _oracle_trajectory(w0, g, nu, dt, checkpoints, round_trip):
    wo, po = _oracle_state(w0, g)
    out, done = {}, 0
    for c in checkpoints:
        for _ in range(c - done):
            wo, po = O.integrate_one_step(wo, po, g, nu, dt, round_trip=round_trip)
        done = c
        out[c] = wo.copy()
    return out


def test_turbulence_n512_nu1e4_1000_steps_vs_oracle(S2D):
    """N = 512, nu = 1e-4, CFL 0.5: one step <= 1e-12, 1000 steps <= 1e-9,
    against the oracle with and without the omega round trip."""
    n, nu, seed = 512, 1e-4, 3
    g = O.get_grid_size(n, n)
    w0, dt, gpu = _turbulence_run(S2D, n, nu, 1000, seed, [1, 1000])
    wo, _ = _oracle_state(w0, g)
    assert abs(dt - O.cfl_dt(wo, g, 0.5)) < 1e-12 * dt
    for rt in (False, True):
        ref = _oracle_trajectory(w0, g, nu, dt, [1, 1000], rt)
        e1, e1000 = O.rel_l2(gpu[1], ref[1]), O.rel_l2(gpu[1000], ref[1000])
        print(f"N={n} nu={nu} dt={dt:.4e} round_trip={rt}: rel-L2 1 step {e1:.3e}, 1000 steps {e1000:.3e}")
        assert e1 < 1e-12
        assert e1000 < 1e-9


def test_taylor_green_n256_1000_steps_vs_oracle_trajectory(S2D):
    """The Taylor-Green workload (N = 256, nu = 0.01, dt = 1e-3, 1000 steps)
    against the oracle's own 1000-step trajectory from the oracle's IC."""
    n, nu, dt, steps = 256, 0.01, 1e-3, 1000
    g = O.get_grid_size(n, n)
    with S2D(n, nu=nu) as s:
        s.set_taylor_green()
        s.integrate_steps(steps, dt)
        s.check_finite()
        wg, pg = s.get_state()
    wo, po = O.set_taylor_green(g)
    wo, po = _oracle_state(wo, g)
    for _ in range(steps):
        wo, po = O.integrate_one_step(wo, po, g, nu, dt, round_trip=True)
    e_w, e_p = O.rel_l2(wg, wo), O.rel_l2(pg, po)
    print(f"Taylor-Green N={n}, {steps} steps vs oracle: rel-L2 omega {e_w:.3e}, psi {e_p:.3e}")
    assert e_w < 1e-9
    assert e_p < 1e-9


@pytest.mark.skipif(os.environ.get("S2D_SLOW_PARITY") != "1",
                    reason="opt-in: the 2048^2 oracle takes ~11 min on 16 cores (S2D_SLOW_PARITY=1)")
def test_turbulence_n2048_1000_steps_vs_oracle(S2D):
    """The 2048^2 decaying-turbulence workload (nu = 1e-4, CFL 0.5, seed 0):
    1 and 1000 steps against the oracle without the omega round trip."""
    n, nu, seed = 2048, 1e-4, 0
    g = O.get_grid_size(n, n)
    w0, dt, gpu = _turbulence_run(S2D, n, nu, 1000, seed, [1, 1000])
    ref = _oracle_trajectory(w0, g, nu, dt, [1, 1000], False)
    e1, e1000 = O.rel_l2(gpu[1], ref[1]), O.rel_l2(gpu[1000], ref[1000])
    print(f"N={n} nu={nu} dt={dt:.4e}: rel-L2 1 step {e1:.3e}, 1000 steps {e1000:.3e}")
    assert e1 < 1e-12
    assert e1000 < 1e-9
