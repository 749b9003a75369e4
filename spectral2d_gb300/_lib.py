"""ctypes binding of ``libspectral2d_gb300.so`` (the C-ABI of include/s2d.h).

Loading fails loudly when the library has not been built: there is no CPU
fallback anywhere in this package.
"""

from __future__ import annotations

import ctypes as C
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB_PATH = os.path.join(PKG, "libspectral2d_gb300.so")
HEADER = os.path.join(ROOT, "include", "s2d.h")

S2D_OK = 0
S2D_ERR_INVALID = -1
S2D_ERR_CUDA = -2
S2D_ERR_NONFINITE = -3
S2D_ERR_TIMEOUT = -4
S2D_ERR_UNSUPPORTED = -5
S2D_ERR_NOMEM = -6

S2D_NO_DEALIASING = 0
S2D_DEALIAS_3_2_RULE = 1
S2D_FP64 = 0
S2D_FP32 = 1
S2D_SPECTRUM_SCHUMANN = 0
S2D_SPECTRUM_K4_GAUSS = 1
S2D_NL_BASDEVANT = 0
S2D_NL_CONSERVATIVE = 1
S2D_FFT_PLANS = 3


class S2DGrid(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("nx", "ny", "dealias", "nxG", "nyG", "kxLG", "kyLG",
                                         "kxMG", "kyMG", "kxLU", "kyLU", "kxMU", "kyMU")] + [
        ("kMax", C.c_double), ("rISize", C.c_int32), ("cISize", C.c_int32)]


class S2DConfig(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("dealias", C.c_int32),
                ("precision", C.c_int32), ("nu", C.c_double), ("alpha", C.c_double),
                ("forcing_amp", C.c_double), ("forcing_k", C.c_int32), ("device", C.c_int32),
                ("nonlinear_form", C.c_int32)]


class S2DError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"s2d error {code}: {msg}")
        self.code = code


_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_h = C.c_void_p

# name -> (restype, argtypes)
SIGNATURES = {
    "s2d_version": (C.c_int, []),
    "s2d_last_error": (C.c_char_p, []),
    "s2d_get_grid_size": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.POINTER(S2DGrid)]),
    "s2d_create": (C.c_int, [C.POINTER(S2DConfig), C.POINTER(C.c_void_p)]),
    "s2d_destroy": (None, [_h]),
    "s2d_set_state": (C.c_int, [_h, _dp, C.c_int32, C.c_int32]),
    "s2d_get_state": (C.c_int, [_h, _dp, _dp, C.c_int32, C.c_int32]),
    "s2d_integrate_one_step": (C.c_int, [_h, C.c_double]),
    "s2d_integrate_steps": (C.c_int, [_h, C.c_int32, C.c_double]),
    "s2d_integrate_one_step_host": (C.c_int, [_h, _dp, _dp, C.c_int32, C.c_int32, C.c_double]),
    "s2d_compute_rhs": (C.c_int, [_h, _dp, C.c_int32, C.c_int32]),
    "s2d_spectrum_bins": (C.c_int, [_h]),
    "s2d_spectrum": (C.c_int, [_h, _dp, C.c_int32, _dp, _dp, _dp]),
    "s2d_enstrophy": (C.c_int, [_h, _dp]),
    "s2d_minmax_abs": (C.c_int, [_h, _dp]),
    "s2d_set_taylor_green": (C.c_int, [_h]),
    "s2d_set_turbulent": (C.c_int, [_h, C.c_uint64, C.c_int32, C.c_double, C.c_double, C.c_double]),
    "s2d_turbulent_ic_host": (C.c_int, [C.c_int32, C.c_uint64, C.c_int32, C.c_double, C.c_double,
                                        C.c_double, _dp]),
    "s2d_cfl_dt": (C.c_int, [_h, C.c_double, _dp]),
    "s2d_check_finite": (C.c_int, [_h]),
    "s2d_synchronize": (C.c_int, [_h]),
    "s2d_time_steps": (C.c_int, [_h, C.c_int32, C.c_double, _dp, _dp]),
    "s2d_kernels_per_step": (C.c_int, [_h]),
    "s2d_set_fft_plan": (C.c_int, [_h, C.c_int32]),
    "s2d_get_fft_plan": (C.c_int, [_h, C.POINTER(C.c_int32)]),
    "s2d_tune_fft_plan": (C.c_int, [_h, C.c_double, C.POINTER(C.c_int32), _dp]),
    "s2d_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(C.c_void_p)]),
    "s2d_host_free": (C.c_int, [C.c_void_p]),
    "s2d_probe_fp64_peak": (C.c_int, [C.c_int32, _dp]),
    "s2d_compute_rhs_noalloc": (C.c_int, [C.c_int32, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]),
    "s2d_slab_partition": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_int32)]),
    "s2d_slab_create": (C.c_int, [C.POINTER(S2DConfig), C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "s2d_slab_destroy": (None, [C.c_void_p]),
    "s2d_slab_handle": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "s2d_slab_exchange": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                    C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "s2d_slab_phase": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_double]),
    "s2d_slab_get_columns": (C.c_int, [C.c_void_p, _dp, _dp, C.c_int32, C.c_int32]),
    "s2d_batch_create": (C.c_int, [C.c_int32, C.POINTER(S2DConfig), C.POINTER(C.c_void_p)]),
    "s2d_batch_destroy": (None, [C.c_void_p]),
    "s2d_batch_size": (C.c_int, [C.c_void_p]),
    "s2d_batch_run": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p)]),
    "s2d_batch_set_dt": (C.c_int, [C.c_void_p, _dp]),
    "s2d_batch_integrate_steps": (C.c_int, [C.c_void_p, C.c_int32]),
    "s2d_batch_time_steps": (C.c_int, [C.c_void_p, C.c_int32, _dp]),
    "s2d_batch_status": (C.c_int, [C.c_void_p]),
    "s2d_batch_synchronize": (C.c_int, [C.c_void_p]),
    "s2d_batch_tune": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), _dp]),
    "s2d_batch_inject_stall": (C.c_int, [C.c_void_p, C.c_int32]),
    "s2d_cnn_create": (C.c_int, [C.c_int32, C.c_int32, C.c_uint64, C.c_int32, C.POINTER(C.c_void_p)]),
    "s2d_cnn_destroy": (None, [C.c_void_p]),
    "s2d_cnn_num_params": (C.c_int, [C.c_void_p]),
    "s2d_cnn_get_params": (C.c_int, [C.c_void_p, _fp]),
    "s2d_cnn_set_params": (C.c_int, [C.c_void_p, _fp]),
    "s2d_cnn_set_scales": (C.c_int, [C.c_void_p, _dp]),
    "s2d_cnn_get_scales": (C.c_int, [C.c_void_p, _dp]),
    "s2d_cnn_set_band": (C.c_int, [C.c_void_p, C.c_double]),
    "s2d_cnn_get_band": (C.c_int, [C.c_void_p, _dp]),
    "s2d_cnn_forward_host": (C.c_int, [C.c_void_p, _fp, C.c_int32, _fp]),
    "s2d_cnn_grad_host": (C.c_int, [C.c_void_p, _fp, _fp, C.c_int32, _fp, _dp]),
    "s2d_cnn_keep_layer_grads": (C.c_int, [C.c_void_p, C.c_int32]),
    "s2d_cnn_set_fused": (C.c_int, [C.c_void_p, C.c_int32]),
    "s2d_cnn_inject_stall": (C.c_int, [C.c_void_p, C.c_int32]),
    "s2d_cnn_get_tensor": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, _fp]),
    "s2d_cnn_dataset_reserve": (C.c_int, [C.c_void_p, C.c_int32]),
    "s2d_cnn_dataset_size": (C.c_int, [C.c_void_p]),
    "s2d_cnn_dataset_add": (C.c_int, [C.c_void_p, C.c_void_p]),
    "s2d_cnn_dataset_stats": (C.c_int, [C.c_void_p, _dp]),
    "s2d_cnn_train_epoch": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_uint64,
                                      _dp]),
    "s2d_cnn_eval": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _dp]),
    "s2d_cnn_status": (C.c_int, [C.c_void_p]),
    "s2d_filter_state": (C.c_int, [C.c_void_p, C.c_void_p]),
    "s2d_subgrid_flux": (C.c_int, [C.c_void_p, C.c_void_p, _dp]),
    "s2d_les_set_closure": (C.c_int, [C.c_void_p, C.c_void_p]),
    "s2d_les_closure_term": (C.c_int, [C.c_void_p]),
    "s2d_les_integrate_steps": (C.c_int, [C.c_void_p, C.c_int32, C.c_double]),
    "s2d_les_time_steps": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.POINTER(C.c_double)]),
    "s2d_batch_set_closure": (C.c_int, [C.c_void_p, C.c_void_p]),
    "s2d_skewness": (C.c_int, [_h, _dp, _dp]),
    "s2d_checkpoint_write": (C.c_int, [_h, C.c_char_p, C.c_int64, C.c_double]),
    "s2d_checkpoint_read": (C.c_int, [_h, C.c_char_p, C.POINTER(C.c_int64), _dp]),
    "s2d_write_restart": (C.c_int, [_h, C.c_char_p, C.c_int32, C.c_int64, C.c_double]),
    "s2d_read_restart": (C.c_int, [_h, C.c_char_p, C.POINTER(C.c_int64), _dp]),
}

_lib = None


def header_symbols(path: str = HEADER) -> list[str]:
    """Names of every ``S2D_API`` function declared in include/*.h."""
    names = []
    inc = os.path.dirname(path)
    for fn in sorted(os.listdir(inc)):
        if fn.endswith(".h"):
            txt = open(os.path.join(inc, fn)).read()
            names += re.findall(r"S2D_API\s+[\w\s\*]+?\b(s2d_\w+)\s*\(", txt)
    return names


def lib():
    """Load (once) and return the shared library with typed signatures."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -m spectral2d_gb300.build` "
                "(the GPU path has no fallback)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    return lib().s2d_last_error().decode(errors="replace")


def check(code: int) -> int:
    """Raise :class:`S2DError` for a negative status."""
    if code < 0:
        raise S2DError(code, last_error())
    return code
