"""One run decomposed over several ranks: the host side of the s2d_slab_*
C-ABI (include/s2d.h).

The reference runs one simulation on several MPI ranks in slabs, and
FFTW-MPI transposes inside every transform (src/Alloc.F90:90-100,
src/Spectral.F90:340-349).  Here rank r owns the kx columns
[kx0_r, kx0_r + nkx_r) of the spectral state for the y-passes and the
physical rows [y0_r, y0_r + ny_r) for the x-pass; every RK3 stage is three
phases with an all-to-all after the first two (:func:`rk3_step`).  The
library moves no data between ranks: the exchange is a function the caller
supplies --

* :func:`dist_exchange` -- ``torch.distributed.all_to_all_single`` over the
  default process group (NCCL for GPU buffers; gloo for host buffers), one
  process per GPU;
* :class:`LocalSlabGroup` -- every slab of a run in one process (on one or
  several devices), the exchange done by device copies.

PyTorch is used here only to reach the communication library and to copy
device buffers; the phases are the library's kernels.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .solver import _FP, Spectral2D, get_grid_size


def partition(nx: int, nranks: int, rank: int):
    """(kx0, nkx, y0, ny) of ``rank``: contiguous, balanced column and row
    ranges (the same arithmetic as the library's)."""
    part = (C.c_int32 * 4)()
    L.check(L.lib().s2d_slab_partition(nx, nranks, rank, part))
    return tuple(int(x) for x in part)


class Slab:
    """Rank ``rank`` of ``nranks`` of one run (s2d_slab_create).  ``handle``
    is a :class:`Spectral2D` view of the slab's handle (initial conditions,
    set_state, CFL dt, synchronize)."""

    def __init__(self, nx: int, nu: float, rank: int, nranks: int, precision: str = "fp64", device: int = 0):
        self._L = L.lib()
        cfg = L.S2DConfig(nx=nx, ny=nx, dealias=L.S2D_DEALIAS_3_2_RULE, precision=_FP[precision], nu=nu,
                          alpha=0.0, forcing_amp=0.0, forcing_k=0, device=device,
                          nonlinear_form=L.S2D_NL_BASDEVANT)
        s = C.c_void_p()
        L.check(self._L.s2d_slab_create(C.byref(cfg), rank, nranks, C.byref(s)))
        self._s = s
        h = C.c_void_p()
        L.check(self._L.s2d_slab_handle(s, C.byref(h)))
        self.handle = Spectral2D._borrow(h, nx, nu, precision)
        self.nx, self.rank, self.nranks, self.device = nx, rank, nranks, device
        self.part = partition(nx, nranks, rank)

    def close(self) -> None:
        if getattr(self, "_s", None):
            self.handle._h = None
            self._L.s2d_slab_destroy(self._s)
            self._s = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    def exchange_layout(self, e: int):
        """(send pointer, receive pointer, bytes to each rank, bytes from each rank)."""
        snd, rcv = C.c_void_p(), C.c_void_p()
        sb, rb = (C.c_int64 * self.nranks)(), (C.c_int64 * self.nranks)()
        L.check(self._L.s2d_slab_exchange(self._s, e, C.byref(snd), C.byref(rcv), sb, rb))
        return snd.value, rcv.value, list(sb), list(rb)

    def phase(self, stage: int, phase: int, dt: float) -> None:
        L.check(self._L.s2d_slab_phase(self._s, stage, phase, dt))

    def synchronize(self) -> None:
        self.handle.synchronize()

    def get_columns(self, w: np.ndarray | None = None, psi: np.ndarray | None = None):
        """This rank's columns of (wC, psiC) written into reference-layout
        arrays (new zero arrays when not given); other columns untouched."""
        g = get_grid_size(self.nx, self.nx)
        if w is None:
            w = np.zeros((g.nyG, g.cISize), dtype=np.complex128)
        if psi is None:
            psi = np.zeros_like(w)
        dp = C.POINTER(C.c_double)
        L.check(self._L.s2d_slab_get_columns(self._s, w.ctypes.data_as(dp), psi.ctypes.data_as(dp), g.cISize,
                                             g.nyG))
        return w, psi


def rk3_step(slab, dt: float, exchange) -> None:
    """One IntegrateOneStep (src/TimeIntegration.F90:130-210) of a slab:
    per stage, phase 0 (K1 on the rank's columns), exchange 0, phase 1 (K2 on
    its rows), exchange 1, phase 2 (K3 and the stage update).  ``slab`` is a
    :class:`Slab` (or any object with the same phase / synchronize /
    exchange_layout methods); ``exchange(slab, e)`` moves segment q of the
    send buffer of every rank to rank q."""
    for stage in (1, 2, 3):
        slab.phase(stage, 0, dt)
        slab.synchronize()
        exchange(slab, 0)
        slab.phase(stage, 1, dt)
        slab.synchronize()
        exchange(slab, 1)
        slab.phase(stage, 2, dt)


class _CudaBuf:
    """A device buffer as a 1-D uint8 array for torch.as_tensor."""

    def __init__(self, ptr: int, nbytes: int):
        self.__cuda_array_interface__ = {"shape": (nbytes,), "typestr": "|u1", "data": (ptr, False),
                                         "version": 3}


def device_bytes(ptr: int, nbytes: int, device: int):
    """A uint8 torch tensor aliasing nbytes of device memory at ptr."""
    import torch
    with torch.cuda.device(device):
        return torch.as_tensor(_CudaBuf(ptr, max(nbytes, 1)), device=f"cuda:{device}")[:nbytes]


def dist_exchange(slab, e: int) -> None:
    """The all-to-all of exchange e over torch.distributed's default group
    (one rank per process): ``all_to_all_single`` of the slab's send buffer
    into its receive buffer with the per-rank byte counts."""
    import torch
    import torch.distributed as dist
    snd, rcv, sb, rb = slab.exchange_layout(e)
    if isinstance(snd, np.ndarray):   # host buffers (gloo)
        st, rt = torch.from_numpy(snd.view(np.uint8)), torch.from_numpy(rcv.view(np.uint8))
    else:
        st, rt = device_bytes(snd, sum(sb), slab.device), device_bytes(rcv, sum(rb), slab.device)
    dist.all_to_all_single(rt[:sum(rb)], st[:sum(sb)], output_split_sizes=rb, input_split_sizes=sb)
    if not isinstance(snd, np.ndarray):
        torch.cuda.synchronize(slab.device)


class LocalSlabGroup:
    """Every slab of one run in this process (devices[r] for rank r; one
    device for all by default), stepped in lockstep, the all-to-alls done as
    device copies.  The same kernels as the multi-process run."""

    def __init__(self, nx: int, nu: float, nranks: int, precision: str = "fp64", devices=None):
        devices = list(devices) if devices is not None else [0] * nranks
        self.slabs = [Slab(nx, nu, r, nranks, precision, devices[r]) for r in range(nranks)]
        self.nx = nx

    def close(self) -> None:
        for s in self.slabs:
            s.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_state(self, w: np.ndarray) -> None:
        for s in self.slabs:
            s.handle.set_state(w)

    def _exchange(self, e: int) -> None:
        import torch
        lay = [s.exchange_layout(e) for s in self.slabs]
        for r, s in enumerate(self.slabs):       # r receives segment r of every q's send buffer
            _, rcv, _, rb = lay[r]
            roff = 0
            for q, t in enumerate(self.slabs):
                snd, _, sb, _ = lay[q]
                soff = sum(sb[:r])
                n = sb[r]
                assert n == rb[q]
                if n:
                    dst = device_bytes(rcv + roff, n, s.device)
                    dst.copy_(device_bytes(snd + soff, n, t.device))
                roff += rb[q]
        for s in self.slabs:
            torch.cuda.synchronize(s.device)

    def step(self, dt: float) -> None:
        for stage in (1, 2, 3):
            for ph in (0, 1, 2):
                for s in self.slabs:
                    s.phase(stage, ph, dt)
                if ph < 2:
                    for s in self.slabs:
                        s.synchronize()
                    self._exchange(ph)
        for s in self.slabs:
            s.synchronize()

    def get_state(self):
        """(wC, psiC) of the whole run, assembled from every slab's columns."""
        w = psi = None
        for s in self.slabs:
            w, psi = s.get_columns(w, psi)
        return w, psi
