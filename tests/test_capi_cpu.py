"""CPU tests of the C-ABI library: it loads without a GPU, exports every
symbol include/*.h declares, and its host-only entry points agree with the
oracle.  No compute call here touches a GPU."""

import ctypes as C
import os
import re

import numpy as np
import pytest

import oracle as O
from spectral2d_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_header_symbol(built_lib):
    names = L.header_symbols()
    assert len(names) >= 25
    lib = C.CDLL(built_lib)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the ctypes table covers the header exactly
    assert sorted(names) == sorted(L.SIGNATURES)


@pytest.mark.parametrize("nx", [8, 96, 256, 2048, 4096])
def test_get_grid_size_matches_oracle(gpu_lib, nx):
    g = L.S2DGrid()
    assert gpu_lib.s2d_get_grid_size(nx, nx, 1, C.byref(g)) == 0
    o = O.get_grid_size(nx, nx)
    for f in ("nxG", "nyG", "kxLG", "kyLG", "kxMG", "kyMG", "kxLU", "kyLU", "kxMU", "kyMU",
              "rISize", "cISize"):
        assert getattr(g, f) == getattr(o, f), f
    assert g.kMax == o.kMax


def test_grid_size_rejects_unimplemented_dealiasing(gpu_lib):
    g = L.S2DGrid()
    assert gpu_lib.s2d_get_grid_size(16, 16, 2, C.byref(g)) == L.S2D_ERR_UNSUPPORTED
    assert "empty case" in L.last_error()


@pytest.mark.parametrize("kind,k0", [(1, 10.0), (0, 1.5)])
def test_turbulent_ic_host_matches_oracle(gpu_lib, kind, k0):
    from spectral2d_gb300.solver import turbulent_ic_host
    nx = 64
    w = turbulent_ic_host(nx, 7, "k4gauss" if kind == 1 else "schumann", k0, 1.0, 0.5)
    g = O.get_grid_size(nx, nx)
    wo, _ = O.set_turbulent(g, 7, kind=kind, k0=k0, urms=1.0, tke_target=0.5)
    assert O.rel_l2(w, wo) < 1e-13


@pytest.mark.parametrize("cfg", [
    dict(nx=0), dict(nx=12), dict(nx=16, ny=32), dict(nx=16, dealias=0),
    dict(nx=16, precision=7), dict(nx=16, nu=float("nan")), dict(nx=16, forcing_amp=1.0, forcing_k=99),
])
def test_create_rejects_bad_config_before_touching_a_gpu(gpu_lib, cfg):
    c = L.S2DConfig(nx=cfg.get("nx", 16), ny=cfg.get("ny", cfg.get("nx", 16)),
                    dealias=cfg.get("dealias", 1), precision=cfg.get("precision", 0),
                    nu=cfg.get("nu", 0.01), alpha=0.0, forcing_amp=cfg.get("forcing_amp", 0.0),
                    forcing_k=cfg.get("forcing_k", 0), device=0)
    h = C.c_void_p()
    r = gpu_lib.s2d_create(C.byref(c), C.byref(h))
    assert r in (L.S2D_ERR_INVALID, L.S2D_ERR_UNSUPPORTED), (r, L.last_error())
    assert not h.value


@pytest.mark.parametrize("cfg, msg", [
    (dict(nx=40), "padded grid 60 "),                              # 60 = 4 * 15: no FFT plan
    (dict(nx=16, forcing_amp=1.0, forcing_k=99), "outside [0, 8]"),
])
def test_create_error_messages_name_the_rejected_values(gpu_lib, cfg, msg):
    """The messages of rejected handles report values read before the
    half-built handle is freed."""
    c = L.S2DConfig(nx=cfg["nx"], ny=cfg["nx"], dealias=1, precision=0, nu=0.01, alpha=0.0,
                    forcing_amp=cfg.get("forcing_amp", 0.0), forcing_k=cfg.get("forcing_k", 0), device=0)
    h = C.c_void_p()
    assert gpu_lib.s2d_create(C.byref(c), C.byref(h)) != 0
    assert msg in L.last_error(), L.last_error()


def test_null_arguments_are_rejected(gpu_lib):
    assert gpu_lib.s2d_get_grid_size(16, 16, 1, None) == L.S2D_ERR_INVALID
    assert gpu_lib.s2d_create(None, None) == L.S2D_ERR_INVALID
    assert gpu_lib.s2d_integrate_one_step(None, 0.1) == L.S2D_ERR_INVALID
    assert gpu_lib.s2d_set_state(None, None, 0, 0) == L.S2D_ERR_INVALID
    assert gpu_lib.s2d_turbulent_ic_host(16, 1, 1, 10.0, 1.0, 0.5, None) == L.S2D_ERR_INVALID


def test_product_package_does_not_import_the_oracle():
    import pathlib
    pkg = pathlib.Path(L.PKG)
    for p in pkg.rglob("*"):
        if p.suffix in (".py", ".cu", ".cpp", ".h", ".cuh"):
            assert "oracle" not in p.read_text().replace("the oracle", ""), p


def _header_params():
    """name -> (return type, parameter count) of every S2D_API declaration."""
    hdr = open(os.path.join(ROOT, "include", "s2d.h")).read()
    out = {}
    for m in re.finditer(r"S2D_API\s+(.+?)\b(s2d_\w+)\s*\(([^;]*?)\)\s*;", hdr, re.S):
        ret, name, params = m.group(1).strip(), m.group(2), m.group(3).strip()
        out[name] = (ret, 0 if params in ("", "void") else params.count(",") + 1)
    return out


def test_fortran_interfaces_match_the_header(built_lib):
    """Every BIND(C) interface of the Fortran module names an exported entry
    point of the header, with its argument count, as a FUNCTION when the C
    function returns a value and a SUBROUTINE when it returns void (no
    Fortran compiler is available to check the module itself)."""
    src = open(os.path.join(ROOT, "spectral2d_gb300", "fortran", "s2d_mod.F90")).read()
    src = re.sub(r"&\s*\n\s*&?", " ", src)   # join continuation lines
    pat = re.compile(r"(INTEGER\(C_INT\)\s+FUNCTION|SUBROUTINE)\s+(\w+)\s*\(([^)]*)\)\s*BIND\(C,\s*NAME='(\w+)'\)")
    found = pat.findall(src)
    assert len(found) >= 20
    hdr = _header_params()
    lib = C.CDLL(built_lib)
    for kind, fname, args, cname in found:
        assert fname == cname and cname in hdr, cname
        nargs = len([a for a in args.split(",") if a.strip()])
        ret, nparams = hdr[cname]
        assert nargs == nparams, (cname, nargs, nparams)
        assert ("SUBROUTINE" in kind) == (ret == "void"), (cname, kind, ret)
        assert hasattr(lib, cname), cname


def test_multiply_high_quotients_are_exact_over_the_kernels_index_ranges():
    """The kernels split indices with q = floor(n m / 2^32), m = ceil(2^32 / d)
    (FFT passes: j mod Ns; column gathers and stores: n / G, n / M, n / KY)
    instead of an integer division.  The bound n (m d - 2^32) < 2^32 makes q
    exact for n < 2^17, d < 2^14; checked here for every d of that range that
    a plan can produce (G, Ns, M, KY: 1..4097 and the M = 3 * 2^a * 3^b up to
    6144) and every n < 2^17."""
    import numpy as np
    n = np.arange(1 << 17, dtype=np.uint64)
    ds = set(range(1, 4098))
    ds |= {m for m in range(12, 6145, 12) if all(p in (2, 3) for p in _prime_factors(m))}
    for d in sorted(ds):
        m = np.uint64((0xFFFFFFFF // d + 1) & 0xFFFFFFFF if d > 1 else 0)
        q = n if d == 1 else (n * m) >> np.uint64(32)
        assert np.array_equal(q, n // np.uint64(d)), d


def _prime_factors(m):
    out, p = [], 2
    while p * p <= m:
        while m % p == 0:
            out.append(p)
            m //= p
        p += 1
    if m > 1:
        out.append(m)
    return out
