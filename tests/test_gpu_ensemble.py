"""GPU tests of the batched ensemble: runs of uneven sizes advanced by one
persistent launch per RK3 stage must reproduce the single-run path exactly
(the same kernels' arithmetic), in FP64 and FP32; the FP32 runs' error
against the FP64 oracle is stated; the tuner must leave the state intact."""

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods(built_lib):
    from spectral2d_gb300 import Ensemble, Spectral2D
    return Ensemble, Spectral2D


def _setup(ens, nxs, seeds):
    dts = []
    for r, s in zip(ens.runs, seeds):
        r.set_turbulent_velocity(seed=s, spectrum="k4gauss", k0=min(10.0, r.nx / 8), tke=0.5)
        dts.append(r.compute_time_step(0.5))
    ens.set_dt(dts)
    return dts


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_ensemble_equals_single_runs(mods, precision):
    Ensemble, Spectral2D = mods
    nxs = [16, 64, 128, 32, 256, 128]
    nus = [5e-3, 2e-3, 1e-3, 4e-3, 5e-4, 8e-4]
    seeds = [11, 12, 13, 14, 15, 16]
    steps = 12
    with Ensemble(nxs, nus, precision=precision) as ens:
        dts = _setup(ens, nxs, seeds)
        w0 = [r.get_state()[0] for r in ens.runs]
        ens.integrate_steps(steps)
        ens.status()
        wb = [r.get_state()[0] for r in ens.runs]
    for i, n in enumerate(nxs):
        with Spectral2D(n, nu=nus[i], precision=precision) as s:
            s.set_state(w0[i])
            s.integrate_steps(steps, dts[i])
            ws, _ = s.get_state()
        assert O.rel_l2(wb[i], ws) <= 1e-15, (n, O.rel_l2(wb[i], ws))


def test_ensemble_fp32_error_vs_fp64_oracle(mods):
    Ensemble, _ = mods
    nxs, nus, seeds, steps = [64, 128], [2e-3, 1e-3], [3, 4], 20
    with Ensemble(nxs, nus, precision="fp32") as ens:
        dts = _setup(ens, nxs, seeds)
        w0 = [r.get_state()[0] for r in ens.runs]
        ens.integrate_steps(steps)
        wb = [r.get_state()[0] for r in ens.runs]
    for i, n in enumerate(nxs):
        g = O.get_grid_size(n, n)
        w = O.truncate(w0[i], g)
        p = O.truncate(O.compute_psi(w, g), g)
        for _ in range(steps):
            w, p = O.integrate_one_step(w, p, g, nus[i], dts[i], round_trip=False)
        err = O.rel_l2(wb[i], w)
        print(f"ensemble fp32 N={n}: {steps} steps rel-L2 vs FP64 oracle {err:.2e}")
        assert err < 1e-5


def test_tuner_keeps_state_and_results(mods):
    Ensemble, Spectral2D = mods
    nxs, nus, seeds = [32, 128, 64], [3e-3, 1e-3, 2e-3], [7, 8, 9]
    with Ensemble(nxs, nus) as ens:
        dts = _setup(ens, nxs, seeds)
        before = [r.get_state()[0] for r in ens.runs]
        threads, cps, ms = ens.tune()
        assert threads in (128, 256, 512) and cps >= 1 and ms > 0
        plans = [r.fft_plan for r in ens.runs]
        assert all(0 <= p < 3 for p in plans)
        after = [r.get_state()[0] for r in ens.runs]
        for a, b in zip(before, after):
            assert np.array_equal(a, b)
        ens.integrate_steps(5)
        wb = [r.get_state()[0] for r in ens.runs]
    for i, n in enumerate(nxs):
        with Spectral2D(n, nu=nus[i]) as s:   # the single run on the plan the tuner chose
            s.fft_plan = plans[i]
            s.set_state(before[i])
            s.integrate_steps(5, dts[i])
            assert O.rel_l2(wb[i], s.get_state()[0]) <= 1e-15


def test_uneven_ensemble_of_the_ensemble_workload_shape(mods):
    """96 runs (32 x 128^2, 32 x 256^2, 32 x 512^2), nu in U[5e-4, 5e-3]:
    a few steps, every run finite and its energy decaying, three runs
    checked against single runs."""
    Ensemble, Spectral2D = mods
    rng = np.random.default_rng(0)
    nxs = [128] * 32 + [256] * 32 + [512] * 32
    nus = list(rng.uniform(5e-4, 5e-3, 96))
    with Ensemble(nxs, nus) as ens:
        dts = _setup(ens, nxs, range(96))
        e0 = [r.compute_spectrum()[2] for r in ens.runs]
        picks = [0, 40, 95]
        w0 = {i: ens.runs[i].get_state()[0] for i in picks}
        ens.integrate_steps(4)
        ens.status()
        e1 = [r.compute_spectrum()[2] for r in ens.runs]
        wb = {i: ens.runs[i].get_state()[0] for i in picks}
    assert all(b < a for a, b in zip(e0, e1))
    for i in picks:
        with Spectral2D(nxs[i], nu=nus[i]) as s:
            s.set_state(w0[i])
            s.integrate_steps(4, dts[i])
            assert O.rel_l2(wb[i], s.get_state()[0]) <= 1e-15


def test_bounded_wait_times_out_and_the_context_stays_usable(mods):
    """Failure detection without a GPU fault: run 1's x-pass tiles are made
    to wait for a tile that never comes (injected on the host); each wait
    gives up after its iteration limit, the step ends, the status is
    S2D_ERR_TIMEOUT, and once the stall is removed the batch steps normally
    and the untouched run is exactly the single-run result."""
    import time
    from spectral2d_gb300 import S2DError
    Ensemble, Spectral2D = mods
    nxs, nus, seeds = [32, 16], [2e-3, 2e-3], [21, 22]
    with Ensemble(nxs, nus) as ens:
        dts = _setup(ens, nxs, seeds)
        w0 = ens.runs[0].get_state()[0]
        ens.inject_stall(1)
        t0 = time.perf_counter()
        ens.integrate_steps(1)
        with pytest.raises(S2DError) as ei:
            ens.status()
        waited = time.perf_counter() - t0
        assert ei.value.code == -4   # S2D_ERR_TIMEOUT
        assert 0.2 < waited < 60.0
        w1 = ens.runs[0].get_state()[0]
        ens.inject_stall(-1)
        ens.integrate_steps(2)
        ens.status()
        w3 = ens.runs[0].get_state()[0]
    with Spectral2D(32, nu=2e-3) as s:
        s.set_state(w0)
        s.integrate_steps(1, dts[0])
        assert np.array_equal(s.get_state()[0], w1)
        s.integrate_steps(2, dts[0])
        assert np.array_equal(s.get_state()[0], w3)
