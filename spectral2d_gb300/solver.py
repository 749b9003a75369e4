"""Python host interface over the C-ABI, named after the reference's routines.

The reference is a Fortran program whose modules expose ``GetGridSize``,
``SetTaylorGreen``, ``SetTurbulentVelocity``, ``IntegrateOneStep``,
``ComputeRHS``, ``ComputeSpectrum`` and the driver's min/max print
(src/Spectral.F90, src/SetIC.F90, src/TimeIntegration.F90,
src/Analysis.F90, src/Spectral2D.F90).  :class:`Spectral2D` offers the same
operations on a device-resident state; spectral arrays crossing this
interface use the reference layout: complex128 of shape ``(nyG, cISize)``
(C order), which is the Fortran ``(cISize, nyG)`` array.

Every call goes through ``libspectral2d_gb300.so``; there is no CPU path.
"""

from __future__ import annotations

import ctypes as C
import weakref

import numpy as np

from . import _lib as L

_FP = {"fp64": L.S2D_FP64, "fp32": L.S2D_FP32}
_SPEC = {"schumann": L.S2D_SPECTRUM_SCHUMANN, "k4gauss": L.S2D_SPECTRUM_K4_GAUSS}
_FORM = {"basdevant": L.S2D_NL_BASDEVANT, "conservative": L.S2D_NL_CONSERVATIVE}


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def get_grid_size(nx: int, ny: int, dealias: int = L.S2D_DEALIAS_3_2_RULE) -> L.S2DGrid:
    """``GetGridSize`` (src/Spectral.F90:117-219)."""
    g = L.S2DGrid()
    L.check(L.lib().s2d_get_grid_size(nx, ny, dealias, C.byref(g)))
    return g


def turbulent_ic_host(nx: int, seed: int, spectrum: str = "k4gauss", k0: float = 10.0,
                      urms: float = 1.0, tke: float = 0.5) -> np.ndarray:
    """The library's turbulent-IC generator evaluated on the host (no GPU)."""
    g = get_grid_size(nx, nx)
    w = np.zeros((g.nyG, g.cISize), dtype=np.complex128)
    L.check(L.lib().s2d_turbulent_ic_host(nx, seed, _SPEC[spectrum], k0, urms, tke,
                                          _dptr(w.view(np.float64))))
    return w


def pinned_array(shape, dtype=np.complex128) -> np.ndarray:
    """Zeroed page-locked host array (freed when the array is collected)."""
    nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
    ptr = C.c_void_p()
    L.check(L.lib().s2d_host_alloc(nbytes, C.byref(ptr)))
    buf = (C.c_byte * nbytes).from_address(ptr.value)
    weakref.finalize(buf, L.lib().s2d_host_free, C.c_void_p(ptr.value))
    arr = np.frombuffer(buf, dtype=dtype).reshape(shape)
    arr[...] = 0
    return arr


def probe_fp64_peak(device: int = 0) -> float:
    """Measured FP64 FMA throughput of the GPU, TFLOP/s."""
    v = C.c_double()
    L.check(L.lib().s2d_probe_fp64_peak(device, C.byref(v)))
    return v.value


class Spectral2D:
    """One vorticity-streamfunction simulation on one GPU."""

    def __init__(self, nx: int, ny: int | None = None, nu: float = 0.005,
                 precision: str = "fp64", alpha: float = 0.0, forcing_amp: float = 0.0,
                 forcing_k: int = 0, device: int = 0,
                 dealias: int = L.S2D_DEALIAS_3_2_RULE, nonlinear_form: str = "basdevant"):
        self._L = L.lib()
        cfg = L.S2DConfig(nx=nx, ny=ny if ny is not None else nx, dealias=dealias,
                          precision=_FP[precision], nu=nu, alpha=alpha,
                          forcing_amp=forcing_amp, forcing_k=forcing_k, device=device,
                          nonlinear_form=_FORM[nonlinear_form])
        h = C.c_void_p()
        L.check(self._L.s2d_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self.nx = nx
        self.nu = nu
        self.precision = precision
        self.grid = get_grid_size(nx, cfg.ny, dealias)
        self.shape = (self.grid.nyG, self.grid.cISize)

    @classmethod
    def _borrow(cls, handle: C.c_void_p, nx: int, nu: float, precision: str) -> "Spectral2D":
        """Wrap a handle owned elsewhere (a run of an :class:`Ensemble`)."""
        self = cls.__new__(cls)
        self._L = L.lib()
        self._h = handle
        self._owned = False
        self.nx, self.nu, self.precision = nx, nu, precision
        self.grid = get_grid_size(nx, nx)
        self.shape = (self.grid.nyG, self.grid.cISize)
        return self

    # -- lifetime -----------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            if getattr(self, "_owned", True):
                self._L.s2d_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

    # -- state ----------------------------------------------------------------
    def _new(self) -> np.ndarray:
        return np.zeros(self.shape, dtype=np.complex128)

    def set_state(self, wC: np.ndarray) -> None:
        w = np.ascontiguousarray(wC, dtype=np.complex128)
        assert w.shape == self.shape, (w.shape, self.shape)
        L.check(self._L.s2d_set_state(self._h, _dptr(w.view(np.float64)), *self.shape[::-1]))

    def get_state(self):
        """Return ``(wC, psiC)`` in the reference layout."""
        w, p = self._new(), self._new()
        L.check(self._L.s2d_get_state(self._h, _dptr(w.view(np.float64)),
                                      _dptr(p.view(np.float64)), *self.shape[::-1]))
        return w, p

    # -- initial conditions --------------------------------------------------
    def set_taylor_green(self) -> None:
        """``SetTaylorGreen`` (src/SetIC.F90:70-101)."""
        L.check(self._L.s2d_set_taylor_green(self._h))

    def set_turbulent_velocity(self, seed: int, spectrum: str = "k4gauss", k0: float = 10.0,
                               urms: float = 1.0, tke: float = 0.5) -> None:
        """``SetTurbulentVelocity`` (src/SetIC.F90:125-151) with a seeded phase."""
        L.check(self._L.s2d_set_turbulent(self._h, seed, _SPEC[spectrum], k0, urms, tke))

    # -- time stepping -------------------------------------------------------
    def integrate_one_step(self, dt: float) -> None:
        """``IntegrateOneStep`` (src/TimeIntegration.F90:130-210)."""
        L.check(self._L.s2d_integrate_one_step(self._h, dt))

    def integrate_steps(self, n: int, dt: float) -> None:
        L.check(self._L.s2d_integrate_steps(self._h, n, dt))

    def integrate_one_step_host(self, wC: np.ndarray, dt: float, psiC: np.ndarray | None = None,
                                inplace: bool = False):
        """``IntegrateOneStep`` on host arrays: returns the new ``(wC, psiC)``.
        With ``inplace`` the arrays given (e.g. from :func:`pinned_array`) are
        updated directly, as the reference updates its wC/psiC."""
        if inplace:
            assert wC.flags.c_contiguous and wC.dtype == np.complex128 and wC.shape == self.shape
            w = wC
        else:
            w = np.array(wC, dtype=np.complex128, order="C", copy=True)
        p = psiC if psiC is not None else self._new()
        assert p.flags.c_contiguous and p.dtype == np.complex128 and p.shape == self.shape
        L.check(self._L.s2d_integrate_one_step_host(self._h, _dptr(w.view(np.float64)),
                                                    _dptr(p.view(np.float64)),
                                                    *self.shape[::-1], dt))
        return w, p

    def compute_rhs(self) -> np.ndarray:
        """``ComputeRHS`` (src/Spectral.F90:396-482) of the current state."""
        d = self._new()
        L.check(self._L.s2d_compute_rhs(self._h, _dptr(d.view(np.float64)), *self.shape[::-1]))
        return d

    def compute_time_step(self, cfl: float) -> float:
        """CFL time step (fills ``ComputeTimeStep``, src/TimeIntegration.F90:213-215)."""
        v = C.c_double()
        L.check(self._L.s2d_cfl_dt(self._h, cfl, C.byref(v)))
        return v.value

    def synchronize(self) -> None:
        L.check(self._L.s2d_synchronize(self._h))

    def check_finite(self) -> None:
        L.check(self._L.s2d_check_finite(self._h))

    # -- diagnostics ---------------------------------------------------------
    def compute_spectrum(self):
        """``ComputeSpectrum`` (src/Analysis.F90:267-460):
        ``(kBin, Ek, tke, eps, enstDiss)``."""
        nb = L.check(self._L.s2d_spectrum_bins(self._h))
        Ek = np.zeros(nb)
        t, e, z = C.c_double(), C.c_double(), C.c_double()
        L.check(self._L.s2d_spectrum(self._h, _dptr(Ek), nb, C.byref(t), C.byref(e), C.byref(z)))
        return np.arange(nb, dtype=np.float64), Ek, t.value, e.value, z.value

    def skewness(self):
        """(xSkew, ySkew) of ``Analysis`` (src/Analysis.F90:135-225)."""
        x, y = C.c_double(), C.c_double()
        L.check(self._L.s2d_skewness(self._h, C.byref(x), C.byref(y)))
        return x.value, y.value

    # -- checkpoints and restart files ---------------------------------------
    def checkpoint_write(self, path: str, nadv: int = 0, time: float = 0.0) -> None:
        L.check(self._L.s2d_checkpoint_write(self._h, path.encode(), nadv, time))

    def checkpoint_read(self, path: str):
        n, t = C.c_int64(), C.c_double()
        L.check(self._L.s2d_checkpoint_read(self._h, path.encode(), C.byref(n), C.byref(t)))
        return n.value, t.value

    def write_restart(self, root: str, num: int, nadv: int, time: float) -> str:
        """Physical Omega, Psi, u, v; returns the path of the binary file."""
        L.check(self._L.s2d_write_restart(self._h, root.encode(), num, nadv, time))
        return f"{root}_{num:08d}.bin"

    def read_restart(self, path: str):
        n, t = C.c_int64(), C.c_double()
        L.check(self._L.s2d_read_restart(self._h, path.encode(), C.byref(n), C.byref(t)))
        return n.value, t.value

    def enstrophy(self) -> float:
        v = C.c_double()
        L.check(self._L.s2d_enstrophy(self._h, C.byref(v)))
        return v.value

    def minmax_abs(self):
        """(max|w|, min|w|, max|psi|, min|psi|) as printed by src/Spectral2D.F90:358-377."""
        out = np.zeros(4)
        L.check(self._L.s2d_minmax_abs(self._h, _dptr(out)))
        return tuple(float(x) for x in out)

    # -- timing ----------------------------------------------------------------
    def time_steps(self, n: int, dt: float, per_kernel: bool = False):
        """Device time of n steps on the handle's stream (CUDA events).
        Returns ``ms`` or ``(ms, [yinv_ms, xpass_ms, yfwd_ms])``."""
        ms = C.c_double()
        if per_kernel:
            k = np.zeros(3)
            L.check(self._L.s2d_time_steps(self._h, n, dt, C.byref(ms), _dptr(k)))
            return ms.value, k
        L.check(self._L.s2d_time_steps(self._h, n, dt, C.byref(ms), None))
        return ms.value

    @property
    def fft_plan(self) -> int:
        """Radix order of the FFTs (0, 1 or 2; see s2d_set_fft_plan)."""
        p = C.c_int32()
        L.check(self._L.s2d_get_fft_plan(self._h, C.byref(p)))
        return p.value

    @fft_plan.setter
    def fft_plan(self, plan: int) -> None:
        L.check(self._L.s2d_set_fft_plan(self._h, int(plan)))

    def tune_fft_plan(self, dt: float):
        """Time every radix plan on this run's step, keep the fastest (state
        restored); returns (plan, ms per step of each plan)."""
        p = C.c_int32()
        ms = np.zeros(L.S2D_FFT_PLANS)
        L.check(self._L.s2d_tune_fft_plan(self._h, dt, C.byref(p), _dptr(ms)))
        return p.value, ms

    def kernels_per_step(self) -> int:
        return L.check(self._L.s2d_kernels_per_step(self._h))


class Ensemble:
    """Independent runs of uneven sizes advanced together: one persistent
    kernel launch per RK3 stage for all runs, replayed from a CUDA graph.
    ``runs[i]`` is a :class:`Spectral2D` view of run i (set/get state, ICs,
    CFL, spectrum), ordered with the ensemble's launches."""

    def __init__(self, nxs, nus, precision: str = "fp64", device: int = 0, alpha=None,
                 forcing_amp=None, forcing_k=None):
        self._L = L.lib()
        n = len(nxs)
        cfgs = (L.S2DConfig * n)()
        for i in range(n):
            cfgs[i] = L.S2DConfig(nx=nxs[i], ny=nxs[i], dealias=L.S2D_DEALIAS_3_2_RULE,
                                  precision=_FP[precision], nu=nus[i],
                                  alpha=(alpha[i] if alpha is not None else 0.0),
                                  forcing_amp=(forcing_amp[i] if forcing_amp is not None else 0.0),
                                  forcing_k=(forcing_k[i] if forcing_k is not None else 0),
                                  device=device, nonlinear_form=L.S2D_NL_BASDEVANT)
        b = C.c_void_p()
        L.check(self._L.s2d_batch_create(n, cfgs, C.byref(b)))
        self._b = b
        self.runs = []
        for i in range(n):
            h = C.c_void_p()
            L.check(self._L.s2d_batch_run(b, i, C.byref(h)))
            self.runs.append(Spectral2D._borrow(h, nxs[i], nus[i], precision))
        self.nxs = list(nxs)

    def close(self) -> None:
        if getattr(self, "_b", None):
            for r in self.runs:
                r._h = None
            self._L.s2d_batch_destroy(self._b)
            self._b = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    def set_dt(self, dts) -> None:
        a = np.ascontiguousarray(dts, dtype=np.float64)
        L.check(self._L.s2d_batch_set_dt(self._b, _dptr(a)))

    def integrate_steps(self, n: int) -> None:
        L.check(self._L.s2d_batch_integrate_steps(self._b, n))

    def time_steps(self, n: int) -> float:
        ms = C.c_double()
        L.check(self._L.s2d_batch_time_steps(self._b, n, C.byref(ms)))
        return ms.value

    def status(self) -> None:
        L.check(self._L.s2d_batch_status(self._b))

    def synchronize(self) -> None:
        L.check(self._L.s2d_batch_synchronize(self._b))

    def inject_stall(self, run: int) -> None:
        """Host-made fault for tests: run's x-pass tiles wait for a tile that
        does not exist until their bounded waits run out (run = -1 clears)."""
        L.check(self._L.s2d_batch_inject_stall(self._b, run))

    def set_closure(self, net: "ClosureNet | None") -> None:
        """One closure network for every run (all on its grid): each step
        starts with one network forward over the whole batch."""
        L.check(self._L.s2d_batch_set_closure(self._b, net._c if net is not None else None))
        self._net = net   # keep the network alive while attached

    def tune(self):
        """Autotune the tile schedule; returns (threads, ctas_per_sm, ms_per_step)."""
        t, c, ms = C.c_int32(), C.c_int32(), C.c_double()
        L.check(self._L.s2d_batch_tune(self._b, C.byref(t), C.byref(c), C.byref(ms)))
        return t.value, c.value, ms.value


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class ClosureNet:
    """The subgrid-closure CNN (6 circular 3x3 layers, 32 channels, GELU,
    BF16 activations/weights with FP32 accumulation, Adam) on the LES
    collocation grid ``grid`` x ``grid``."""

    def __init__(self, grid: int, max_batch: int = 64, seed: int = 0, device: int = 0):
        self._L = L.lib()
        c = C.c_void_p()
        L.check(self._L.s2d_cnn_create(grid, max_batch, seed, device, C.byref(c)))
        self._c = c
        self.grid = grid
        self.max_batch = max_batch

    def close(self) -> None:
        if getattr(self, "_c", None):
            self._L.s2d_cnn_destroy(self._c)
            self._c = None

    def status(self) -> None:
        """Raises if a tensor-core completion wait of the network's kernels
        gave up since the last check (clears the flag)."""
        L.check(self._L.s2d_cnn_status(self._c))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_params(self) -> int:
        return L.check(self._L.s2d_cnn_num_params(self._c))

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.num_params, dtype=np.float32)
        L.check(self._L.s2d_cnn_get_params(self._c, _fptr(p)))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.num_params
        L.check(self._L.s2d_cnn_set_params(self._c, _fptr(p)))

    def set_scales(self, rms) -> None:
        a = np.ascontiguousarray(rms, dtype=np.float64)
        L.check(self._L.s2d_cnn_set_scales(self._c, _dptr(a)))

    def get_scales(self) -> np.ndarray:
        a = np.zeros(3)
        L.check(self._L.s2d_cnn_get_scales(self._c, _dptr(a)))
        return a

    @property
    def band(self) -> float:
        """k_min: the closure term is applied to modes with |k| >= k_min."""
        v = C.c_double()
        L.check(self._L.s2d_cnn_get_band(self._c, C.byref(v)))
        return v.value

    @band.setter
    def band(self, k_min: float) -> None:
        L.check(self._L.s2d_cnn_set_band(self._c, float(k_min)))

    def forward(self, x: np.ndarray) -> np.ndarray:
        """x: (B, grid, grid, 2) (w, psi) -> (B, grid, grid) Pi."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.zeros(x.shape[:3], dtype=np.float32)
        L.check(self._L.s2d_cnn_forward_host(self._c, _fptr(x), x.shape[0], _fptr(y)))
        return y

    def grad(self, x: np.ndarray, target: np.ndarray):
        """(loss, gradient) of the normalised MSE for one batch."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(target, dtype=np.float32)
        g = np.zeros(self.num_params, dtype=np.float32)
        loss = C.c_double()
        L.check(self._L.s2d_cnn_grad_host(self._c, _fptr(x), _fptr(t), x.shape[0], _fptr(g), C.byref(loss)))
        return loss.value, g

    def set_fused(self, on: bool = True) -> None:
        """Gradient-free forward passes in one fused launch (default) or one
        launch per layer; the results are the same bits."""
        L.check(self._L.s2d_cnn_set_fused(self._c, int(bool(on))))

    def inject_stall(self, on: bool = True) -> None:
        """Host-made fault for tests: one CTA of the fused forward skips a grid
        barrier, the others' bounded waits run out (S2D_ERR_TIMEOUT)."""
        L.check(self._L.s2d_cnn_inject_stall(self._c, int(bool(on))))

    def keep_layer_grads(self, keep: bool = True) -> None:
        """Keep dL/dz of every hidden layer in the following gradient calls."""
        L.check(self._L.s2d_cnn_keep_layer_grads(self._c, int(bool(keep))))

    _TENSOR_CH = {0: (16, 32, 32, 32, 32, 32), 1: (32,) * 5, 2: (32, 32, 32, 32, 32, 16)}

    def tensor(self, kind: int, layer: int, batch: int) -> np.ndarray:
        """A BF16 tensor of the last forward / gradient call as float32
        (batch, grid, grid, padded channels): kind 0 = the layer's input,
        1 = its pre-activation, 2 = dL/dz of its output."""
        ch = self._TENSOR_CH[kind][layer]
        out = np.zeros((batch, self.grid, self.grid, ch), dtype=np.float32)
        L.check(self._L.s2d_cnn_get_tensor(self._c, kind, layer, batch, _fptr(out)))
        return out

    def reserve(self, capacity: int) -> None:
        L.check(self._L.s2d_cnn_dataset_reserve(self._c, capacity))

    def add_sample(self, les: Spectral2D) -> None:
        L.check(self._L.s2d_cnn_dataset_add(self._c, les._h))

    @property
    def dataset_size(self) -> int:
        return L.check(self._L.s2d_cnn_dataset_size(self._c))

    def dataset_stats(self) -> np.ndarray:
        a = np.zeros(3)
        L.check(self._L.s2d_cnn_dataset_stats(self._c, _dptr(a)))
        return a

    def train_epoch(self, first: int, count: int, batch: int, lr: float, seed: int) -> float:
        loss = C.c_double()
        L.check(self._L.s2d_cnn_train_epoch(self._c, first, count, batch, lr, seed, C.byref(loss)))
        return loss.value

    def eval(self, first: int, count: int) -> float:
        loss = C.c_double()
        L.check(self._L.s2d_cnn_eval(self._c, first, count, C.byref(loss)))
        return loss.value


def filter_state(dns: Spectral2D, les: Spectral2D) -> None:
    """LES state := sharp spectral filter of the DNS state."""
    L.check(L.lib().s2d_filter_state(dns._h, les._h))


def subgrid_flux(dns: Spectral2D, les: Spectral2D, host: bool = False):
    """Filter the DNS into the LES and form the subgrid flux Pi^ on the LES
    grid (returned in the reference layout when ``host``)."""
    out = np.zeros(les.shape, dtype=np.complex128) if host else None
    L.check(L.lib().s2d_subgrid_flux(dns._h, les._h, _dptr(out.view(np.float64)) if host else None))
    return out


def les_set_closure(les: Spectral2D, net: ClosureNet | None) -> None:
    L.check(L.lib().s2d_les_set_closure(les._h, net._c if net is not None else None))


def les_integrate_steps(les: Spectral2D, n: int, dt: float) -> None:
    L.check(L.lib().s2d_les_integrate_steps(les._h, n, dt))


def les_time_steps(les: Spectral2D, n: int, dt: float) -> float:
    """Device time (ms, CUDA events on the handle's stream) of n closure-LES
    steps of ``les_integrate_steps``."""
    ms = C.c_double()
    L.check(L.lib().s2d_les_time_steps(les._h, n, dt, C.byref(ms)))
    return ms.value
