"""GPU parity tests: the sm_103a path through the C-ABI against the oracle
(the FP64 numpy restatement of the reference) and the exact golden vectors.

Tolerances (relative L2 in omega unless stated):
  * one RHS: 1e-13; one RK3 step: 1e-12 (the reference's one-step bar);
  * 1000 steps of decaying turbulence: 1e-9 (the reference's 1000-step bar);
  * Taylor-Green after 1000 steps vs exp(-2 nu t): 1e-10;
  * FP32 variant vs FP64 oracle: stated per test (round-off of FP32 FFTs).
"""

import math
import os

import numpy as np
import pytest

import oracle as O
from spectral2d_gb300 import _lib as L

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def S2D(built_lib):
    from spectral2d_gb300 import Spectral2D
    return Spectral2D


def _oracle_state(w, g):
    w = O.truncate(w, g)
    return w, O.truncate(O.compute_psi(w, g), g)


@pytest.mark.parametrize("n", [8, 16])
def test_rhs_exact_golden(S2D, n):
    d = np.load(os.path.join(GOLD, f"rhs_exact_n{n}.npz"))
    with S2D(n, nu=float(d["nu"])) as s:
        s.set_state(d["w"])
        dW = s.compute_rhs()
    assert O.rel_l2(dW, d["dW"]) < 1e-14


def test_step_exact_golden(S2D):
    d = np.load(os.path.join(GOLD, "step_exact_n8.npz"))
    with S2D(8, nu=float(d["nu"])) as s:
        s.set_state(d["w"])
        s.integrate_one_step(float(d["dt"]))
        w, p = s.get_state()
    assert O.rel_l2(w, d["w_new"]) < 1e-14
    assert O.rel_l2(p, d["psi_new"]) < 1e-14


@pytest.mark.parametrize("n", [8, 32, 64, 96, 128, 256, 512])
def test_rhs_vs_oracle(S2D, n):
    g = O.get_grid_size(n, n)
    w = O.random_state(g, 100 + n)
    with S2D(n, nu=0.01) as s:
        s.set_state(w)
        dW = s.compute_rhs()
        w_back, psi_back = s.get_state()
    wo, po = _oracle_state(w, g)
    assert np.array_equal(w_back, wo)
    assert O.rel_l2(psi_back, po) < 1e-15
    ref, _ = O.compute_rhs(wo, po, g, 0.01, round_trip=False)
    assert O.rel_l2(dW, O.truncate(ref, g)) < 1e-13


@pytest.mark.parametrize("n", [8, 64, 256])
def test_conservative_form_vs_oracle_and_basdevant(S2D, n):
    """The reference's own form of the nonlinear term on the GPU, and its
    agreement with the default (Basdevant) form."""
    g = O.get_grid_size(n, n)
    w = O.random_state(g, 300 + n)
    with S2D(n, nu=0.01, nonlinear_form="conservative") as a, S2D(n, nu=0.01) as b:
        a.set_state(w)
        b.set_state(w)
        da, db = a.compute_rhs(), b.compute_rhs()
        a.integrate_steps(3, 1e-3)
        b.integrate_steps(3, 1e-3)
        wa, _ = a.get_state()
        wb, _ = b.get_state()
    wo, po = _oracle_state(w, g)
    ref, _ = O.compute_rhs(wo, po, g, 0.01, round_trip=False)
    assert O.rel_l2(da, O.truncate(ref, g)) < 1e-13
    assert O.rel_l2(db, da) < 1e-13
    assert O.rel_l2(wb, wa) < 1e-13


@pytest.mark.parametrize("n", [16, 64, 256])
def test_one_step_vs_oracle(S2D, n):
    g = O.get_grid_size(n, n)
    w = O.random_state(g, 7 + n, decay=0.05)
    nu, dt = 0.005, 1e-3
    with S2D(n, nu=nu) as s:
        s.set_state(w)
        s.integrate_one_step(dt)
        wg, pg = s.get_state()
    wo, po = _oracle_state(w, g)
    for rt in (False, True):   # with and without the reference's omega round trip
        w1, p1 = O.integrate_one_step(wo, po, g, nu, dt, round_trip=rt)
        assert O.rel_l2(wg, w1) < 1e-12
        assert O.rel_l2(pg, p1) < 1e-12


def test_taylor_green_ic_matches_oracle(S2D):
    g = O.get_grid_size(64, 64)
    with S2D(64, nu=0.01) as s:
        s.set_taylor_green()
        w, p = s.get_state()
    wo, po = O.set_taylor_green(g)
    assert O.rel_l2(w, O.truncate(wo, g)) < 1e-14
    assert O.rel_l2(p, O.truncate(po, g)) < 1e-14


def test_taylor_green_1000_steps_analytic(S2D):
    """The Taylor-Green workload: N=256 (384^2 padded), nu=0.01, dt=1e-3,
    1000 steps, against the analytic decay exp(-2 nu t)."""
    n, nu, dt, steps = 256, 0.01, 1e-3, 1000
    g = O.get_grid_size(n, n)
    with S2D(n, nu=nu) as s:
        s.set_taylor_green()
        w0, _ = s.get_state()
        s.integrate_steps(steps, dt)
        w, p = s.get_state()
    F = math.exp(-2.0 * nu * steps * dt)
    assert O.rel_l2(w, w0 * F) < 1e-10
    psiE, wE, uE, vE = O.taylor_green_exact(g, nu, steps * dt)
    dx = 2 * np.pi / g.nxG
    wN = O.transform_c2r(w, g)
    pN = O.transform_c2r(p, g)
    # the error norms of analysis/TaylorGreen.py:43-60
    assert O.l2_error(dx, dx, wE, wN) < 1e-10 * 2 * np.pi
    assert O.linf_error(wE, wN) < 1e-10
    assert O.linf_error(psiE, pN) < 1e-10


def test_turbulence_1000_steps_vs_oracle(S2D):
    """Decaying turbulence from the seeded k^4 exp(-2(k/10)^2) spectrum,
    N=128, nu=1e-3, CFL dt, 1000 steps: GPU vs oracle."""
    n, nu, steps = 128, 1e-3, 1000
    g = O.get_grid_size(n, n)
    with S2D(n, nu=nu) as s:
        s.set_turbulent_velocity(seed=1, spectrum="k4gauss", k0=10.0, tke=0.5)
        w0, _ = s.get_state()
        dt = s.compute_time_step(0.5)
        s.integrate_steps(steps, dt)
        s.check_finite()
        wg, _ = s.get_state()
    wo, po = _oracle_state(w0, g)
    assert abs(dt - O.cfl_dt(wo, g, 0.5)) < 1e-12 * dt
    for _ in range(steps):
        wo, po = O.integrate_one_step(wo, po, g, nu, dt, round_trip=False)
    err = O.rel_l2(wg, wo)
    print(f"turbulence N={n}, {steps} steps: rel-L2 = {err:.3e}")
    assert err < 1e-9


def test_graph_replay_equals_single_steps(S2D):
    n = 64
    g = O.get_grid_size(n, n)
    w = O.random_state(g, 3, decay=0.1)
    with S2D(n, nu=0.01) as a, S2D(n, nu=0.01) as b:
        a.set_state(w)
        b.set_state(w)
        for _ in range(5):
            a.integrate_one_step(1e-3)
        b.integrate_steps(5, 1e-3)
        wa, _ = a.get_state()
        wb, _ = b.get_state()
    assert np.array_equal(wa, wb)


def test_host_array_step_equals_device_step(S2D):
    n = 64
    g = O.get_grid_size(n, n)
    w = O.random_state(g, 4, decay=0.1)
    with S2D(n, nu=0.01) as s:
        w1, p1 = s.integrate_one_step_host(w, 1e-3)
        s.set_state(w)
        s.integrate_one_step(1e-3)
        w2, p2 = s.get_state()
    assert np.array_equal(w1, w2) and np.array_equal(p1, p2)


def _host_buf(shape, mem):
    """NaN-filled host array; "fresh" is an untouched np.zeros array (its pages
    are not resident yet, so the library stages it through copies)."""
    from spectral2d_gb300.solver import pinned_array
    if mem == "fresh":
        return np.zeros(shape, dtype=np.complex128)
    a = pinned_array(shape) if mem == "pinned" else np.empty(shape, dtype=np.complex128)
    a[...] = np.nan + 1j * np.nan
    return a


@pytest.mark.parametrize("n", [8, 96])
@pytest.mark.parametrize("mem", ["pageable", "pinned", "fresh"])
@pytest.mark.parametrize("io", ["in_place", "copy"])
def test_host_array_io_paths(S2D, n, mem, io, monkeypatch):
    """Host-array calls on pageable and page-locked arrays, read and written
    in place by the kernels or (S2D_HOST_IO=copy) through staging copies: the
    truncated part of every output is zero whatever the array held, the
    truncated part of the input is not read, and all paths give the same bits
    as the device-resident step."""
    from spectral2d_gb300.solver import _dptr
    g = O.get_grid_size(n, n)
    w = O.random_state(g, 5, decay=0.1)
    K, M = n // 2, g.nyG
    keep = np.zeros(w.shape, dtype=bool)
    keep[: K + 1, : K + 1] = True
    keep[M - K:, : K + 1] = True
    with S2D(n, nu=0.01) as r:
        r.set_state(w)
        dW_ref = r.compute_rhs()
        r.integrate_one_step(1e-3)
        w_ref, p_ref = r.get_state()
    if io == "copy":
        monkeypatch.setenv("S2D_HOST_IO", "copy")
    with S2D(n, nu=0.01) as s:
        ny, cx = w.shape
        wh = _host_buf(w.shape, "pageable" if mem == "fresh" else mem)
        wh[keep] = w[keep]
        ph = _host_buf(w.shape, mem)
        s.set_state(wh)                     # reads the rectangle only
        dh = _host_buf(w.shape, mem)
        L.check(s._L.s2d_compute_rhs(s._h, _dptr(dh.view(np.float64)), cx, ny))
        s.integrate_one_step_host(wh, 1e-3, ph, inplace=True)
        gw, gp = _host_buf(w.shape, mem), _host_buf(w.shape, mem)
        L.check(s._L.s2d_get_state(s._h, _dptr(gw.view(np.float64)), _dptr(gp.view(np.float64)), cx, ny))
    for a in (wh, ph, dh, gw, gp):
        assert not (a[~keep] != 0).any()
    assert np.array_equal(dh, dW_ref)
    assert np.array_equal(wh, w_ref) and np.array_equal(ph, p_ref)
    assert np.array_equal(gw, w_ref) and np.array_equal(gp, p_ref)


def test_spectrum_minmax_enstrophy_vs_oracle(S2D):
    n = 128
    g = O.get_grid_size(n, n)
    w = O.random_state(g, 9, decay=0.05)
    nu = 0.002
    with S2D(n, nu=nu) as s:
        s.set_state(w)
        kb, Ek, tke, eps, enst = s.compute_spectrum()
        mm = s.minmax_abs()
        Z = s.enstrophy()
    wo, po = _oracle_state(w, g)
    kbo, Eko, tkeo, epso, ensto = O.spectrum_of_vorticity(wo, g, nu)
    assert len(Ek) == len(Eko) == 2 * 0 + int(math.sqrt(2 * (3 * n // 4) ** 2) + 1.0) + 1
    assert np.allclose(Ek, Eko, rtol=1e-13, atol=1e-300)
    for a, b in ((tke, tkeo), (eps, epso), (enst, ensto)):
        assert abs(a - b) <= 1e-13 * abs(b)
    mo = O.minmax_abs(wo, po)
    assert np.allclose(mm, mo, rtol=1e-15, atol=0)
    assert abs(Z - O.enstrophy(wo, g)) <= 1e-13 * Z


def test_forcing_and_drag_vs_oracle(S2D):
    n, nu, alpha, amp, kf, dt = 64, 1e-3, 0.1, 4.0, 4, 1e-3
    g = O.get_grid_size(n, n)
    w = O.random_state(g, 11, decay=0.1)
    with S2D(n, nu=nu, alpha=alpha, forcing_amp=amp, forcing_k=kf) as s:
        s.set_state(w)
        s.integrate_steps(3, dt)
        wg, _ = s.get_state()
    wo, po = _oracle_state(w, g)
    F = O.kolmogorov_forcing(g, amp, kf)
    for _ in range(3):
        wo, po = O.integrate_one_step(wo, po, g, nu, dt, round_trip=False, forcing=F, alpha=alpha)
    assert O.rel_l2(wg, wo) < 1e-12


@pytest.mark.parametrize("n", [64, 256])
def test_fp32_variant_error_vs_fp64_oracle(S2D, n):
    """FP32 FFTs and products (1/k^2 in FP64): one RHS within 1e-5 and ten
    steps within 1e-5 of the FP64 oracle."""
    g = O.get_grid_size(n, n)
    w = O.random_state(g, 21, decay=0.05)
    nu, dt = 0.005, 1e-3
    with S2D(n, nu=nu, precision="fp32") as s:
        s.set_state(w)
        dW = s.compute_rhs()
        s.integrate_steps(10, dt)
        wg, _ = s.get_state()
    wo, po = _oracle_state(w, g)
    ref, _ = O.compute_rhs(wo, po, g, nu, round_trip=False)
    e_rhs = O.rel_l2(dW, O.truncate(ref, g))
    for _ in range(10):
        wo, po = O.integrate_one_step(wo, po, g, nu, dt, round_trip=False)
    e_step = O.rel_l2(wg, wo)
    print(f"fp32 N={n}: rhs rel-L2 {e_rhs:.2e}, 10 steps rel-L2 {e_step:.2e}")
    assert e_rhs < 1e-5 and e_step < 1e-5


def test_nonfinite_state_is_reported(S2D):
    from spectral2d_gb300 import S2DError
    n = 32
    g = O.get_grid_size(n, n)
    w = O.random_state(g, 2)
    w[1, 1] = np.nan
    with S2D(n, nu=0.01) as s:
        s.set_state(w)
        s.integrate_one_step(1e-3)
        with pytest.raises(S2DError) as ei:
            s.check_finite()
        assert ei.value.code == -3
        s.check_finite()   # flag was cleared


def test_full_size_one_step_vs_oracle(S2D):
    """The 2048^2 (3072^2 padded) FP64 decaying-turbulence workload: one RK3
    step from the seeded IC against the oracle, and size-independent checks
    (energy and enstrophy decay, Hermitian kx=0 column)."""
    n, nu = 2048, 1e-4
    g = O.get_grid_size(n, n)
    O.set_workers(O.cpu_count())
    with S2D(n, nu=nu) as s:
        s.set_turbulent_velocity(seed=0, spectrum="k4gauss", k0=10.0, tke=0.5)
        w0, _ = s.get_state()
        dt = s.compute_time_step(0.5)
        _, _, e0, _, _ = s.compute_spectrum()
        z0 = s.enstrophy()
        s.integrate_one_step(dt)
        s.check_finite()
        w1, _ = s.get_state()
        _, _, e1, _, _ = s.compute_spectrum()
        z1 = s.enstrophy()
    assert abs(e0 - 0.5) < 1e-13
    assert e1 < e0 and z1 < z0
    assert np.allclose(w1[1:n // 2 + 1, 0], np.conj(w1[(-np.arange(1, n // 2 + 1)) % g.nyG, 0]),
                       rtol=0, atol=1e-14 * np.abs(w1).max())
    wo, po = _oracle_state(w0, g)
    wr, _ = O.integrate_one_step(wo, po, g, nu, dt, round_trip=False)
    err = O.rel_l2(w1, wr)
    print(f"2048^2 one step: rel-L2 {err:.3e}")
    assert err < 1e-12


def test_kolmogorov_4096_one_step_vs_oracle(S2D):
    """The 4096^2 (6144^2 padded) Kolmogorov-flow workload, F = 4 cos(4y),
    drag 0.1, nu = 1e-5: one FP64 RK3 step from a seeded state against the
    oracle, and the FP32 form against the same oracle step."""
    n, nu, alpha, amp, kf = 4096, 1e-5, 0.1, 4.0, 4
    g = O.get_grid_size(n, n)
    O.set_workers(O.cpu_count())
    with S2D(n, nu=nu, alpha=alpha, forcing_amp=amp, forcing_k=kf) as s:
        s.set_turbulent_velocity(seed=1, spectrum="k4gauss", k0=10.0, tke=0.5)
        w0, _ = s.get_state()
        dt = s.compute_time_step(0.5)
        s.integrate_one_step(dt)
        s.check_finite()
        w1, _ = s.get_state()
    with S2D(n, nu=nu, alpha=alpha, forcing_amp=amp, forcing_k=kf, precision="fp32") as s:
        s.set_state(w0)
        s.integrate_one_step(dt)
        w32, _ = s.get_state()
    wo, po = _oracle_state(w0, g)
    F = O.kolmogorov_forcing(g, amp, kf)
    wr, _ = O.integrate_one_step(wo, po, g, nu, dt, round_trip=False, forcing=F, alpha=alpha)
    err, err32 = O.rel_l2(w1, wr), O.rel_l2(w32, wr)
    print(f"4096^2 Kolmogorov one step: FP64 rel-L2 {err:.3e}, FP32 rel-L2 {err32:.3e}")
    assert err < 1e-12 and err32 < 1e-5


@pytest.mark.parametrize("n", [256, 2048])
def test_inviscid_rhs_conserves_energy_and_enstrophy(S2D, n):
    """A size-independent property at the full workload size: with nu = 0 the
    dealiased nonlinear term of the truncated system conserves energy and
    enstrophy, sum Re(conj(psi) dW) = sum Re(conj(w) dW) = 0 (half-spectrum
    weights 1 at kx = 0, 2 elsewhere), to round-off.  The seeded
    k^4 exp(-2 (k/10)^2) state has no energy at |k| = N/2."""
    g = O.get_grid_size(n, n)
    with S2D(n, nu=0.0) as s:
        s.set_turbulent_velocity(seed=7, spectrum="k4gauss", k0=10.0, tke=0.5)
        w, psi = s.get_state()
        dW = s.compute_rhs()
    wt = np.where(g.kxG[None, :] == 0, 1.0, 2.0)
    dE = np.sum(wt * (np.conj(psi) * dW).real)
    dZ = np.sum(wt * (np.conj(w) * dW).real)
    rel_e = abs(dE) / np.sum(wt * np.abs(psi) * np.abs(dW))
    rel_z = abs(dZ) / np.sum(wt * np.abs(w) * np.abs(dW))
    print(f"N={n}: inviscid dE/dt rel {rel_e:.2e}, dZ/dt rel {rel_z:.2e}")
    assert rel_e < 1e-12 and rel_z < 1e-12


def test_handles_from_several_host_threads(S2D):
    """Handles created, stepped and read from four host threads at once (the
    per-device one-time kernel set-up is shared) give the serial bits."""
    import threading
    n = 64
    g = O.get_grid_size(n, n)
    states = [O.random_state(g, 40 + i, decay=0.1) for i in range(4)]

    def run(w):
        with S2D(n, nu=0.01) as s:
            s.set_state(w)
            s.integrate_steps(5, 1e-3)
            return s.get_state()[0]

    serial = [run(w) for w in states]
    out, errs = [None] * 4, []

    def worker(i):
        try:
            out[i] = run(states[i])
        except Exception as e:  # reported below
            errs.append(e)

    ts = [threading.Thread(target=worker, args=(i,)) for i in range(4)]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=120)
    assert not errs, errs
    for a, b in zip(out, serial):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("n", [96, 1024])
def test_programmatic_launches_give_the_plain_order_bits(S2D, monkeypatch, precision, n):
    """Every kernel of a step is launched as a programmatic dependent of the
    one before it (it waits for its predecessor's completion before touching
    memory): the state after 20 steps is bit-identical to plain stream order
    (S2D_PDL=0, read when the handle is created).  FP64 handles take the split
    K3 (column FFTs, then the stage kernel), FP32 the fused one."""
    g = O.get_grid_size(n, n)
    w0 = O.random_state(g, 60, decay=0.1)
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("S2D_PDL", mode)
        with S2D(n, nu=1e-3, precision=precision) as s:
            s.set_state(w0)
            dt = s.compute_time_step(0.5)
            s.integrate_steps(20, dt)
            s.check_finite()
            out[mode] = s.get_state()[0]
    assert np.array_equal(out["0"], out["1"])


@pytest.mark.parametrize("n", [64, 96, 256])
@pytest.mark.parametrize("plan", [0, 1, 2])
def test_every_radix_plan_vs_oracle(S2D, n, plan):
    """Each radix order of the FFTs (s2d_set_fft_plan) gives the oracle's RHS
    and step to round-off; the plans differ in rounding only."""
    g = O.get_grid_size(n, n)
    w = O.random_state(g, 500 + n, decay=0.05)
    nu, dt = 0.005, 1e-3
    with S2D(n, nu=nu) as s:
        s.fft_plan = plan
        assert s.fft_plan == plan
        s.set_state(w)
        dW = s.compute_rhs()
        s.integrate_steps(2, dt)
        wg, _ = s.get_state()
    wo, po = _oracle_state(w, g)
    ref, _ = O.compute_rhs(wo, po, g, nu, round_trip=False)
    assert O.rel_l2(dW, O.truncate(ref, g)) < 1e-13
    for _ in range(2):
        wo, po = O.integrate_one_step(wo, po, g, nu, dt, round_trip=False)
    assert O.rel_l2(wg, wo) < 1e-12


def test_fft_plan_tuner_keeps_the_state(S2D):
    n, nu, dt = 256, 1e-3, 1e-3
    g = O.get_grid_size(n, n)
    w = O.truncate(O.random_state(g, 77, decay=0.05), g)
    with S2D(n, nu=nu) as s:
        s.set_state(w)
        plan, ms = s.tune_fft_plan(dt)
        assert 0 <= plan < 3 and s.fft_plan == plan and np.all(ms > 0)
        print(f"N={n}: ms per step by plan {ms}, chosen {plan}")
        w_after, _ = s.get_state()
        assert np.array_equal(w_after, w)


def test_fp32_xpass_2048_register_radix_vs_generic_and_oracle(S2D, monkeypatch):
    """FP32 at 2048^2 runs its x-pass with register radix-12/16 passes
    (k_xpass32); the generic engine (S2D_XPASS_GENERIC=1) computes the same
    RHS up to FP32 round-off, and both stay within the FP32 error of the FP64
    oracle; an FP32 2048^2 run in a batch equals the single run bit for bit."""
    from spectral2d_gb300 import Ensemble
    n, nu, dt = 2048, 1e-4, 2e-4
    g = O.get_grid_size(n, n)
    w = O.truncate(O.random_state(g, 2048, decay=0.02), g)
    out = {}
    for mode in ("register", "generic"):
        if mode == "generic":
            monkeypatch.setenv("S2D_XPASS_GENERIC", "1")
        with S2D(n, nu=nu, precision="fp32") as s:
            s.set_state(w)
            out[mode] = s.compute_rhs()
            if mode == "register":
                s.integrate_steps(2, dt)
                out["steps"] = s.get_state()[0]
        monkeypatch.delenv("S2D_XPASS_GENERIC", raising=False)
    wo, po = _oracle_state(w, g)
    ref = O.truncate(O.compute_rhs(wo, po, g, nu, round_trip=False)[0], g)
    e_reg, e_gen = O.rel_l2(out["register"], ref), O.rel_l2(out["generic"], ref)
    print(f"FP32 2048^2 RHS vs FP64 oracle: register radix {e_reg:.2e}, generic {e_gen:.2e}, "
          f"between them {O.rel_l2(out['register'], out['generic']):.2e}")
    # the FP32 RHS error grows with N (the k^2 weights of the derivative
    # terms): 8.2e-5 for both x-passes at 2048^2 on GB300
    assert e_reg < 2e-4 and e_gen < 2e-4
    assert e_reg < 1.25 * e_gen
    with Ensemble([n], [nu], precision="fp32") as ens:
        ens.runs[0].set_state(w)
        ens.set_dt([dt])
        ens.integrate_steps(2)
        ens.status()
        wb = ens.runs[0].get_state()[0]
    assert np.array_equal(wb, out["steps"])


@pytest.mark.parametrize("n,precision", [(512, "fp64"), (2048, "fp64"), (2048, "fp32")])
def test_host_array_step_at_workload_sizes_equals_device_step(S2D, n, precision):
    """The host-array step on the caller's page-locked arrays (read and
    written in place by the conversion kernels) at the workload sizes, FP64
    and FP32 (the register radix x-pass): the device-resident step's bits."""
    from spectral2d_gb300.solver import pinned_array
    g = O.get_grid_size(n, n)
    w = O.truncate(O.random_state(g, 9, decay=0.02), g)
    with S2D(n, nu=1e-4, precision=precision) as s:
        s.set_state(w)
        s.integrate_one_step(1e-4)
        w_ref, p_ref = s.get_state()
    with S2D(n, nu=1e-4, precision=precision) as s:
        wh, ph = pinned_array(w.shape), pinned_array(w.shape)
        wh[...] = w
        ph[...] = np.nan
        s.integrate_one_step_host(wh, 1e-4, ph, inplace=True)
    assert np.array_equal(wh, w_ref) and np.array_equal(ph, p_ref)
