"""One run decomposed into slabs (s2d_slab_*), the ranks emulated in one
process on one GPU: every slab's phases run on the GPU in lockstep and the
all-to-alls are device copies (no kernel waits on another).  The slab
kernels are the single-run kernels on column views and row ranges, so the
decomposed run must equal the single run bit for bit."""

import os
import socket

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _single(n, nu, w0, dt, steps, precision="fp64"):
    from spectral2d_gb300 import Spectral2D
    with Spectral2D(n, nu=nu, precision=precision) as s:
        s.set_state(w0)
        for _ in range(steps):
            s.integrate_one_step(dt)
        s.check_finite()
        return s.get_state()


@pytest.mark.parametrize("n,nranks,precision,steps", [
    (64, 2, "fp64", 3), (96, 3, "fp64", 3), (256, 4, "fp64", 2), (128, 5, "fp64", 2),
    (128, 2, "fp32", 3), (2048, 4, "fp64", 1)])
def test_slabs_equal_the_single_run_bit_for_bit(built_lib, n, nranks, precision, steps):
    from spectral2d_gb300.slab import LocalSlabGroup
    nu, dt = 1e-3, 1e-3
    g = O.get_grid_size(n, n)
    w0 = O.truncate(O.random_state(g, 30 + n, decay=0.05), g)
    wref, pref = _single(n, nu, w0, dt, steps, precision)
    with LocalSlabGroup(n, nu, nranks, precision) as grp:
        grp.set_state(w0)
        for _ in range(steps):
            grp.step(dt)
        for s in grp.slabs:
            s.handle.check_finite()
        w, p = grp.get_state()
    assert np.array_equal(w, wref), O.rel_l2(w, wref)
    assert np.array_equal(p, pref), O.rel_l2(p, pref)


def test_slab_run_vs_oracle(built_lib):
    from spectral2d_gb300.slab import LocalSlabGroup
    n, nu, dt, steps = 64, 0.005, 1e-3, 3
    g = O.get_grid_size(n, n)
    w0 = O.truncate(O.random_state(g, 21, decay=0.05), g)
    with LocalSlabGroup(n, nu, 3) as grp:
        grp.set_state(w0)
        for _ in range(steps):
            grp.step(dt)
        w, p = grp.get_state()
    wo, po = w0, O.truncate(O.compute_psi(w0, g), g)
    for _ in range(steps):
        wo, po = O.integrate_one_step(wo, po, g, nu, dt, round_trip=False)
    assert O.rel_l2(w, wo) < 1e-13
    assert O.rel_l2(p, po) < 1e-13


def test_slab_rk3_step_through_torch_distributed_on_one_rank(built_lib):
    """rk3_step with dist_exchange (all_to_all_single on the slab's device
    buffers over NCCL) on a one-rank process group: the pointer wrapping and
    the byte counts of the multi-process path, on this GPU."""
    torch = pytest.importorskip("torch")
    import torch.distributed as dist
    from spectral2d_gb300.slab import Slab, dist_exchange, rk3_step
    if not dist.is_nccl_available():
        pytest.skip("NCCL not available")
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    torch.cuda.set_device(0)
    dist.init_process_group("nccl", init_method=f"tcp://127.0.0.1:{port}", rank=0, world_size=1)
    try:
        n, nu, dt = 64, 1e-3, 1e-3
        g = O.get_grid_size(n, n)
        w0 = O.truncate(O.random_state(g, 8, decay=0.05), g)
        wref, pref = _single(n, nu, w0, dt, 2)
        with Slab(n, nu, 0, 1) as s:
            s.handle.set_state(w0)
            for _ in range(2):
                rk3_step(s, dt, dist_exchange)
            s.synchronize()
            w, p = s.get_columns()
        assert np.array_equal(w, wref) and np.array_equal(p, pref)
    finally:
        dist.destroy_process_group()
