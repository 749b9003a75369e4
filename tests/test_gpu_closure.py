"""GPU tests of the learned-closure pieces: the CNN's forward pass and
gradients against the FP64 numpy oracle (oracle/cnn_oracle.py, fed the same
BF16-rounded weights and inputs; tolerances cover the BF16 rounding of the
GPU's intermediate activations), the subgrid flux against the spectral
oracle, training reducing the loss, and the LES step with the closure."""

import numpy as np
import pytest

import oracle as O
from oracle import cnn_oracle as CO

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S(built_lib):
    import spectral2d_gb300 as S
    return S


def _oracle_params(p, bf=True):
    out, o = [], 0
    for l in range(6):
        ci, co = CO.CHANNELS[l], CO.CHANNELS[l + 1]
        W = p[o:o + co * 9 * ci].reshape(co, 9, ci).astype(np.float64)
        o += co * 9 * ci
        b = p[o:o + co].astype(np.float64)
        o += co
        out.append((CO.bf16(W) if bf else W, b))
    return out


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_cnn_forward_and_gradients_vs_oracle(S):
    grid, B = 24, 2
    rng = np.random.default_rng(0)
    with S.ClosureNet(grid, max_batch=4, seed=3) as net:
        net.set_scales([1.0, 1.0, 1.0])
        p = net.get_params()
        assert p.size == 608 + 4 * 9248 + 289
        x = rng.standard_normal((B, grid, grid, 2)).astype(np.float32)
        t = (0.3 * rng.standard_normal((B, grid, grid))).astype(np.float32)
        y = net.forward(x)
        loss, g = net.grad(x, t)
    params = _oracle_params(p)
    xb = CO.bf16(x)
    yo, _ = CO.forward(params, xb)
    assert _rel(y, yo) < 2e-2
    lo, go, _ = CO.loss_and_grads(params, xb, t.astype(np.float64))
    assert abs(loss - lo) < 2e-2 * lo
    gp = _oracle_params(g, bf=False)
    for l in range(6):
        eW, eb = _rel(gp[l][0], go[l][0]), _rel(gp[l][1], go[l][1])
        print(f"layer {l}: dW rel {eW:.2e}, db rel {eb:.2e}")
        assert eW < 5e-2 and eb < 5e-2


def _bf(a):
    return CO.bf16(np.asarray(a, dtype=np.float64))


def test_cnn_every_layer_vs_oracle_on_the_gpus_own_intermediates(S):
    """Each layer's kernels checked on their own inputs: the GPU exports its
    BF16 activations a_l, pre-activations z_l and layer gradients dL/dz_l
    (s2d_cnn_get_tensor), and the FP64 oracle recomputes from those exact
    values (BF16 weights) each layer's forward output (z_{l+1}, a_{l+1},
    y), weight and bias gradient (FP32 accumulation on the GPU) and data
    gradient dL/dz_{l-1}.  Outputs the GPU stores in BF16 are compared after
    the oracle's value is rounded to BF16 as well; every relative error must
    stay below 1e-3 (in practice far below: only a rounding-boundary crossing
    between FP32 and FP64 sums can differ)."""
    grid, B = 24, 2
    rng = np.random.default_rng(7)
    with S.ClosureNet(grid, max_batch=4, seed=3) as net:
        net.set_scales([1.0, 1.0, 1.0])
        net.keep_layer_grads(True)
        p = net.get_params()
        x = rng.standard_normal((B, grid, grid, 2)).astype(np.float32)
        t = (0.3 * rng.standard_normal((B, grid, grid))).astype(np.float32)
        y = net.forward(x)
        loss, g = net.grad(x, t)
        A = [net.tensor(0, l, B).astype(np.float64) for l in range(6)]
        Z = [net.tensor(1, l, B).astype(np.float64) for l in range(5)]
        D = [net.tensor(2, l, B).astype(np.float64) for l in range(6)]
    params = _oracle_params(p)
    gp = _oracle_params(g, bf=False)
    n = B * grid * grid
    # loss gradient dL/dy = 2 (y - t) / n, stored in BF16
    assert _rel(D[5][..., 0], _bf(2.0 * (y.astype(np.float64) - t) / n)) < 1e-3
    errs = {}
    for l in range(6):
        ci, co = CO.CHANNELS[l], CO.CHANNELS[l + 1]
        a_in = A[l][..., :ci]
        W, b = params[l]
        z = CO.conv(a_in, W, b)
        if l < 5:
            errs[f"z{l}"] = _rel(Z[l][..., :co], _bf(z))
            errs[f"a{l + 1}"] = _rel(A[l + 1][..., :co], _bf(CO.gelu(z)))
        else:
            errs["y"] = _rel(y, z[..., 0])
        dz = D[l][..., :co]
        dW = np.zeros_like(W)
        for tp, (dy, dx) in enumerate(CO.TAPS):
            dW[:, tp, :] = np.einsum("bhwo,bhwi->oi", dz, CO.shift(a_in, dy, dx))
        errs[f"dW{l}"] = _rel(gp[l][0], dW)
        errs[f"db{l}"] = _rel(gp[l][1], dz.sum(axis=(0, 1, 2)))
        if l > 0:
            da = np.zeros(dz.shape[:3] + (ci,))
            for tp, (dy, dx) in enumerate(CO.TAPS):
                da += CO.shift(dz @ W[:, tp, :], -dy, -dx)
            errs[f"dz{l - 1}"] = _rel(D[l - 1][..., :ci], _bf(da * CO.gelu_grad(Z[l - 1][..., :ci])))
    print({k: f"{v:.1e}" for k, v in errs.items()})
    for k, v in errs.items():
        assert v < 1e-3, (k, v)


@pytest.mark.parametrize("grid, B", [(8, 3), (20, 2), (40, 1)])
def test_cnn_forward_edge_tiles_vs_oracle(S, grid, B):
    """The tensor-core convolution at grids whose 8 x 16 tiles are ragged or
    whose halo wraps twice (8: every pixel is an edge pixel), against the
    oracle's circular convolution, forward and gradients."""
    rng = np.random.default_rng(grid)
    with S.ClosureNet(grid, max_batch=4, seed=5) as net:
        net.set_scales([1.0, 1.0, 1.0])
        p = net.get_params()
        x = rng.standard_normal((B, grid, grid, 2)).astype(np.float32)
        t = (0.3 * rng.standard_normal((B, grid, grid))).astype(np.float32)
        y = net.forward(x)
        loss, g = net.grad(x, t)
    params = _oracle_params(p)
    xb = CO.bf16(x)
    yo, _ = CO.forward(params, xb)
    assert _rel(y, yo) < 2e-2
    lo, go, _ = CO.loss_and_grads(params, xb, t.astype(np.float64))
    assert abs(loss - lo) < 2e-2 * lo
    gp = _oracle_params(g, bf=False)
    for l in range(6):
        assert _rel(gp[l][0], go[l][0]) < 5e-2 and _rel(gp[l][1], go[l][1]) < 5e-2


@pytest.mark.parametrize("grid, B", [(8, 3), (20, 2), (40, 1), (192, 1), (192, 9)])
def test_fused_forward_equals_the_layerwise_forward(S, grid, B):
    """The fused inference forward (all six layers in one persistent launch,
    activations in framed images, grid barriers between layers, the three
    column taps summed in the epilogue) against one launch per layer (all nine
    taps summed in the tensor core): the same products in FP32 in another
    order, so equal to FP32 rounding (and the rare BF16 rounding flip it
    causes in an activation) -- at ragged and doubly wrapped tiles (8, 20,
    40) and at the 128^2 LES grid (192^2 pixels), one image and nine (several
    tiles per CTA, every slot and accumulator phase reused across layers).
    Two fused calls give the same bits."""
    rng = np.random.default_rng(100 + grid + B)
    with S.ClosureNet(grid, max_batch=B, seed=11) as net:
        net.set_scales([1.0, 1.0, 1.0])
        x = rng.standard_normal((B, grid, grid, 2)).astype(np.float32)
        net.set_fused(True)
        yf = net.forward(x)
        yf2 = net.forward(x)
        net.set_fused(False)
        yl = net.forward(x)
        net.status()
    assert np.all(np.isfinite(yf))
    assert np.array_equal(yf, yf2)
    e = _rel(yf, yl)
    emax = float(np.max(np.abs(yf - yl)) / np.sqrt(np.mean(yl.astype(np.float64) ** 2)))
    print(f"grid {grid} batch {B}: fused vs per-layer rel-L2 {e:.1e}, max/rms {emax:.1e}")
    # a wrong tap or edge would be O(1) at the pixels it touches
    assert e < 2e-3 and emax < 2e-2


@pytest.mark.parametrize("grid, B", [(8, 3), (24, 2), (40, 2), (192, 2)])
def test_tensor_core_weight_gradient_matches_the_fp32_pipes(S, grid, B, monkeypatch):
    """The weight and bias gradients from the tensor cores (k_wgrad_tc: one
    accumulator per CTA over its tiles, MN-major operands, the bias gradient
    from a block of ones) against the FP32-pipe kernel on the same dL/dz and
    activations: the same sums in another order, at ragged and doubly wrapped
    tiles and at the 192^2 LES grid."""
    rng = np.random.default_rng(300 + grid)
    x = rng.standard_normal((B, grid, grid, 2)).astype(np.float32)
    t = (0.3 * rng.standard_normal((B, grid, grid))).astype(np.float32)
    with S.ClosureNet(grid, max_batch=B, seed=17) as net:
        net.set_scales([1.0, 1.0, 1.0])
        monkeypatch.setenv("S2D_WGRAD_FP32", "1")
        l32, g32 = net.grad(x, t)
        monkeypatch.setenv("S2D_WGRAD_FP32", "0")
        ltc, gtc = net.grad(x, t)
        net.status()
    assert ltc == l32
    a, b = _oracle_params(gtc, bf=False), _oracle_params(g32, bf=False)
    for l in range(6):
        eW, eb = _rel(a[l][0], b[l][0]), _rel(a[l][1], b[l][1])
        print(f"grid {grid} layer {l}: dW rel {eW:.1e}, db rel {eb:.1e}")
        assert eW < 1e-5 and eb < 1e-5


def test_fused_forward_barrier_timeout_is_reported_and_recovers(S):
    """Failure detection of the fused forward's grid barrier, the fault made
    on the host: CTA 0 skips its first arrival, the others' bounded waits
    run out (about 1 s), the forward returns S2D_ERR_TIMEOUT through
    s2d_cnn_status instead of hanging, and once the stall is removed the
    next forward gives the clean result bit for bit."""
    import time
    from spectral2d_gb300 import S2DError
    grid, B = 192, 2
    x = np.random.default_rng(5).standard_normal((B, grid, grid, 2)).astype(np.float32)
    with S.ClosureNet(grid, max_batch=B, seed=19) as net:
        net.set_scales([1.0, 1.0, 1.0])
        y0 = net.forward(x)
        net.inject_stall(True)
        t0 = time.perf_counter()
        with pytest.raises(S2DError) as ei:
            net.forward(x)
        waited = time.perf_counter() - t0
        assert ei.value.code == -4   # S2D_ERR_TIMEOUT
        assert 0.5 < waited < 60.0
        net.inject_stall(False)
        y1 = net.forward(x)
        net.status()
    assert np.array_equal(y0, y1)


def test_subgrid_flux_vs_oracle(S):
    nd, nl, nu = 64, 16, 2e-3
    gd, gl = O.get_grid_size(nd, nd), O.get_grid_size(nl, nl)
    w = O.random_state(gd, 17, decay=0.05)
    with S.Spectral2D(nd, nu=nu) as dns, S.Spectral2D(nl, nu=nu) as les:
        dns.set_state(w)
        pi = S.subgrid_flux(dns, les, host=True)
        wl, _ = les.get_state()
    wo = O.truncate(w, gd)
    po = O.truncate(O.compute_psi(wo, gd), gd)
    dW, _ = O.compute_rhs(wo, po, gd, nu, round_trip=False)
    Nd = -(O.truncate(dW, gd) + nu * (gd.kx ** 2 + gd.ky ** 2) * wo)
    # sharp filter to the LES modes |k| <= nl/2
    def to_les(a):
        out = np.zeros((gl.nyG, gl.cISize), complex)
        K = nl // 2
        for ky in range(-K, K + 1):
            for kx in range(0, K + 1):
                if kx * kx + ky * ky <= K * K:
                    out[ky % gl.nyG, kx] = a[ky % gd.nyG, kx]
        return out
    wf = to_les(wo)
    assert O.rel_l2(wl, wf) < 1e-15
    pf = O.truncate(O.compute_psi(wf, gl), gl)
    dWl, _ = O.compute_rhs(wf, pf, gl, nu, round_trip=False)
    Nl = -(O.truncate(dWl, gl) + nu * (gl.kx ** 2 + gl.ky ** 2) * wf)
    pio = O.truncate(to_les(Nd) - Nl, gl)
    assert O.rel_l2(pi, pio) < 1e-12


def _dataset(S, net, nd=64, nl=16, nsnap=48, every=4):
    with S.Spectral2D(nd, nu=2e-3) as dns, S.Spectral2D(nl, nu=2e-3) as les:
        dns.set_turbulent_velocity(seed=5, spectrum="k4gauss", k0=4.0, tke=0.5)
        dt = dns.compute_time_step(0.5)
        net.reserve(nsnap)
        for _ in range(nsnap):
            dns.integrate_steps(every, dt)
            S.subgrid_flux(dns, les)
            net.add_sample(les)
    return dt


def test_training_reduces_loss(S):
    with S.ClosureNet(24, max_batch=8, seed=1) as net:
        _dataset(S, net)
        assert net.dataset_size == 48
        rms = net.dataset_stats()
        assert np.all(rms > 0)
        net.set_scales(rms)
        l0 = net.eval(0, 48)
        losses = [net.train_epoch(0, 40, 8, 1e-3, seed=e) for e in range(40)]
        l1 = net.eval(0, 48)
        print(f"loss {l0:.3f} -> {l1:.3f}; epoch losses {losses[0]:.3f} ... {losses[-1]:.3f}")
        assert l1 < 0.7 * l0


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_les_with_closure_runs_and_changes_the_solution(S, precision):
    with S.ClosureNet(24, max_batch=8, seed=2) as net:
        dt = _dataset(S, net, nsnap=16)
        net.set_scales(net.dataset_stats())
        for e in range(5):
            net.train_epoch(0, 16, 8, 1e-3, seed=e)
        with S.Spectral2D(16, nu=2e-3, precision=precision) as a, \
                S.Spectral2D(16, nu=2e-3, precision=precision) as b:
            w0 = O.random_state(O.get_grid_size(16, 16), 4, decay=0.2)
            a.set_state(w0)
            b.set_state(w0)
            S.les_set_closure(a, net)
            S.les_integrate_steps(a, 20, dt)
            S.les_integrate_steps(b, 20, dt)
            a.check_finite()
            wa, _ = a.get_state()
            wb, _ = b.get_state()
            S.les_set_closure(a, None)
    assert np.all(np.isfinite(wa))
    d = O.rel_l2(wa, wb)
    print(f"{precision}: closure changes the 20-step LES state by rel-L2 {d:.2e}")
    assert 1e-8 < d < 0.5


def test_timed_closure_steps_match_untimed_ones(S):
    """s2d_les_time_steps runs the same step graph as s2d_les_integrate_steps
    (closure term on a second stream beside the first stage's transforms):
    same bits after the same steps, and a positive device time."""
    n, nu, steps = 16, 2e-3, 8
    with S.ClosureNet(24, max_batch=8, seed=7) as net:
        dt = _dataset(S, net, nsnap=8)
        net.set_scales(net.dataset_stats())
        w0 = O.random_state(O.get_grid_size(n, n), 21, decay=0.2)
        out = []
        for timed in (False, True):
            with S.Spectral2D(n, nu=nu, precision="fp32") as a:
                a.set_state(w0)
                S.les_set_closure(a, net)
                if timed:
                    ms = S.les_time_steps(a, steps, dt)
                    assert ms > 0.0
                else:
                    S.les_integrate_steps(a, steps, dt)
                out.append(a.get_state()[0])
                S.les_set_closure(a, None)
        net.status()
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batched_closure_les_matches_single_runs(S, precision):
    """A batch of LES runs with one closure network (one forward over all
    runs per step) against each run advanced alone with the same network."""
    n, nu, steps = 16, 2e-3, 12
    with S.ClosureNet(24, max_batch=8, seed=5) as net:
        dt = _dataset(S, net, nsnap=8)
        net.set_scales(net.dataset_stats())
        net.train_epoch(0, 8, 8, 1e-3, seed=0)
        w0 = [O.random_state(O.get_grid_size(n, n), 30 + i, decay=0.2) for i in range(3)]
        with S.Ensemble([n] * 3, [nu] * 3, precision=precision) as ens:
            for i in range(3):
                ens.runs[i].set_state(w0[i])
            ens.set_dt([dt] * 3)
            ens.set_closure(net)
            ens.integrate_steps(steps)
            ens.status()
            wb = [r.get_state()[0] for r in ens.runs]
            ens.set_closure(None)
        for i in range(3):
            with S.Spectral2D(n, nu=nu, precision=precision) as a:
                a.set_state(w0[i])
                S.les_set_closure(a, net)
                S.les_integrate_steps(a, steps, dt)
                wa, _ = a.get_state()
                S.les_set_closure(a, None)
            assert np.array_equal(wa, wb[i]), O.rel_l2(wb[i], wa)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_les_closure_fused_network_matches_layerwise(S, precision):
    """The LES step's closure term with the fused network (the layer-1 input
    written framed by the transform kernel) against the per-layer launches:
    the same states to FP32 rounding of the network after the same steps,
    single run and batch; the batch equals the single run bit for bit."""
    n, nu, steps = 128, 1e-3, 6
    with S.ClosureNet(192, max_batch=2, seed=13) as net:
        net.set_scales([1.0, 1.0, 0.05])
        w0 = [O.random_state(O.get_grid_size(n, n), 40 + i, decay=0.2) for i in range(2)]
        dt = 2e-3
        out = {}
        for fused in (True, False):
            net.set_fused(fused)
            with S.Spectral2D(n, nu=nu, precision=precision) as a:
                a.set_state(w0[0])
                S.les_set_closure(a, net)
                S.les_integrate_steps(a, steps, dt)
                out[("single", fused)] = a.get_state()[0]
                S.les_set_closure(a, None)
            with S.Ensemble([n] * 2, [nu] * 2, precision=precision) as ens:
                for i in range(2):
                    ens.runs[i].set_state(w0[i])
                ens.set_dt([dt] * 2)
                ens.set_closure(net)
                ens.integrate_steps(steps)
                ens.status()
                out[("batch", fused)] = [r.get_state()[0] for r in ens.runs]
                ens.set_closure(None)
        net.status()
    assert np.all(np.isfinite(out[("single", True)]))
    e = O.rel_l2(out[("single", True)], out[("single", False)])
    print(f"{precision}: LES state fused vs per-layer network rel-L2 {e:.1e}")
    bar = 1e-6 if precision == "fp64" else 1e-5
    assert e < bar
    for i in range(2):
        assert O.rel_l2(out[("batch", True)][i], out[("batch", False)][i]) < bar
    assert np.array_equal(out[("single", True)], out[("batch", True)][0])
    assert np.array_equal(out[("single", False)], out[("batch", False)][0])


def test_trained_closure_beats_the_closure_free_les(S):
    """The packaged closure (trained on the FP64 2048^2 DNS of seeds 0-7)
    against the closure-free 128^2 LES on held-out seed 9: both start from
    the filtered DNS state and advance 5000 steps with the DNS's dt; the
    closure's energy-spectrum error (1 <= k <= 40) is well below the
    fallback's, and the LES with closure is >= 20x cheaper than the DNS."""
    import os
    import time
    from spectral2d_gb300 import closure
    path = os.path.join(os.path.dirname(S.__file__), "data", "closure_les128.npz")
    assert os.path.exists(path), "trained closure weights are missing"
    steps, k = 5000, slice(1, 41)
    with S.ClosureNet(192, max_batch=1) as net:
        closure.load_weights(net, path)
        with S.Spectral2D(2048, nu=1e-4) as dns, S.Spectral2D(128, nu=1e-4) as filt, \
                S.Spectral2D(128, nu=1e-4, precision="fp32") as les_c, \
                S.Spectral2D(128, nu=1e-4, precision="fp32") as les_0:
            dns.set_turbulent_velocity(seed=9, spectrum="k4gauss", k0=10.0, tke=0.5)
            dt = dns.compute_time_step(0.5)
            S.filter_state(dns, les_c)
            S.filter_state(dns, les_0)
            S.les_set_closure(les_c, net)
            dns.synchronize()
            t0 = time.perf_counter()
            dns.integrate_steps(steps, dt)
            dns.synchronize()
            t1 = time.perf_counter()
            S.les_integrate_steps(les_c, steps, dt)
            les_c.synchronize()
            t2 = time.perf_counter()
            les_0.integrate_steps(steps, dt)
            S.filter_state(dns, filt)
            Ef = filt.compute_spectrum()[1][k]
            Ec = les_c.compute_spectrum()[1][k]
            E0 = les_0.compute_spectrum()[1][k]
            S.les_set_closure(les_c, None)
    ec = float(np.mean(np.abs(Ec - Ef) / Ef))
    e0 = float(np.mean(np.abs(E0 - Ef) / Ef))
    speedup = (t1 - t0) / (t2 - t1)
    print(f"seed 9, {steps} steps: E(k) mean rel err closure {ec:.3f}, none {e0:.3f}; speedup {speedup:.1f}x")
    assert ec < 0.6 * e0
    assert speedup >= 20.0


def test_trained_closure_meets_the_spectrum_bar_on_a_held_out_seed(S):
    """The accuracy metric of the closure, per seed and time-averaged
    (closure.spectrum_errors: E(k) of the LES and of the filtered DNS each
    averaged over the report times, relative error per k, mean over
    1 <= k <= 40), on held-out seed 9 over the first 5000 DNS steps with a
    report every 500: below 10 %, and under half the closure-free LES's.
    The full 20000-step evaluation of seeds 8 and 9 is in
    profiles/closure_les128_eval.json."""
    import os
    from spectral2d_gb300 import closure
    path = os.path.join(os.path.dirname(S.__file__), "data", "closure_les128.npz")
    with S.ClosureNet(192, max_batch=1) as net:
        closure.load_weights(net, path)
        band = net.band
        recs = closure.evaluate(net, [9], 2048, 128, 1e-4, 0.5, 5000, 500, bands=(band,), log=lambda *a: None)
    r = recs[0]
    mc, xc = closure.spectrum_errors(r["E"][f"closure_k{band:g}"], r["E"]["dns"])
    m0, x0 = closure.spectrum_errors(r["E"]["none"], r["E"]["dns"])
    print(f"seed 9, 5000 steps, time-averaged E(k), 1 <= k <= 40: closure mean {mc:.4f} max {xc:.3f}; "
          f"none mean {m0:.4f} max {x0:.3f}")
    assert mc < 0.10
    assert mc < 0.5 * m0
