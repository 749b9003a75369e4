"""The decomposed run's host side on CPU: the slab partition of the C-ABI
(s2d_slab_partition, no GPU needed) and the orchestration of
spectral2d_gb300.slab (rk3_step with dist_exchange) over two gloo ranks, each
rank's phases done by the CPU restatement oracle/slab_oracle.py, against the
whole-run oracle (src/TimeIntegration.F90:130-210)."""

import os
import socket

import numpy as np
import pytest

import oracle as O
from oracle.slab_oracle import SlabPhasesCPU, partition


@pytest.mark.parametrize("nx", [8, 16, 64, 2048])
@pytest.mark.parametrize("nranks", [1, 2, 3, 4, 8])
def test_library_partition_matches_the_restatement(built_lib, nx, nranks):
    from spectral2d_gb300.slab import partition as lib_partition
    if nranks > nx // 2 + 1:
        pytest.skip("more ranks than kx columns (rejected)")
    parts = partition(nx, nranks)
    assert [lib_partition(nx, nranks, r) for r in range(nranks)] == parts
    # contiguous, complete and balanced
    K, M = nx // 2, 3 * nx // 2
    assert parts[0][0] == 0 and parts[-1][0] + parts[-1][1] == K + 1
    assert parts[0][2] == 0 and parts[-1][2] + parts[-1][3] == M
    for a, b in zip(parts, parts[1:]):
        assert a[0] + a[1] == b[0] and a[2] + a[3] == b[2]
    assert max(p[1] for p in parts) - min(p[1] for p in parts) <= 1


def test_partition_rejects_bad_arguments(built_lib):
    import ctypes as C
    from spectral2d_gb300 import _lib as L
    part = (C.c_int32 * 4)()
    lib = L.lib()
    assert lib.s2d_slab_partition(64, 0, 0, part) == L.S2D_ERR_INVALID
    assert lib.s2d_slab_partition(64, 2, 2, part) == L.S2D_ERR_INVALID
    assert lib.s2d_slab_partition(8, 6, 0, part) == L.S2D_ERR_INVALID   # more ranks than kx columns
    assert lib.s2d_slab_partition(64, 17, 0, part) == L.S2D_ERR_INVALID


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n, nu, dt, steps, q):
    import torch.distributed as dist
    from spectral2d_gb300.slab import dist_exchange, rk3_step
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo")
    g = O.get_grid_size(n, n)
    w0 = O.truncate(O.random_state(g, 21, decay=0.05), g)
    slab = SlabPhasesCPU(n, nu, rank, world)
    slab.set_state(w0)
    for _ in range(steps):
        rk3_step(slab, dt, dist_exchange)
    w, psi = slab.get_columns()
    cols = slab.kx0, slab.nkx
    everyone = [None] * world
    dist.all_gather_object(everyone, (cols, w[:, cols[0]:cols[0] + cols[1]], psi[:, cols[0]:cols[0] + cols[1]]))
    dist.destroy_process_group()
    q.put((rank, everyone))


@pytest.mark.parametrize("world", [2, 3])
def test_decomposed_run_over_gloo_ranks_equals_the_whole_run(world):
    """Two (three) processes, each one slab, exchanging over gloo with
    all_to_all_single: after 3 RK3 steps at N = 64 the assembled state equals
    the whole-run oracle to round-off."""
    import torch.multiprocessing as mp
    n, nu, dt, steps = 64, 0.005, 1e-3, 3
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, n, nu, dt, steps, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=300) for _ in procs), key=lambda x: x[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    g = O.get_grid_size(n, n)
    w = np.zeros((g.nyG, g.cISize), dtype=np.complex128)
    psi = np.zeros_like(w)
    for (c0, nc), wc, pc in res[0][1]:
        w[:, c0:c0 + nc] = wc
        psi[:, c0:c0 + nc] = pc
    w0 = O.truncate(O.random_state(g, 21, decay=0.05), g)
    wo, po = w0, O.truncate(O.compute_psi(w0, g), g)
    for _ in range(steps):
        wo, po = O.integrate_one_step(wo, po, g, nu, dt, round_trip=False)
    assert O.rel_l2(w, wo) < 1e-13
    assert O.rel_l2(psi, po) < 1e-13
