"""FP64 numpy restatement of Spectral2D's hot path (the CPU oracle).

TEST INFRASTRUCTURE ONLY -- never imported by the product package.

Every function restates one routine of the reference, in the reference's own
memory layout and conventions, and cites the file:line it follows (paths are
relative to the reference project root):

* complex spectral arrays are C-order ``(nyG, cISize)`` complex128, which is
  the Fortran ``(cISize, nyP)`` layout of the reference with ``nyP == nyG``
  (one MPI rank); row ``j`` holds ``ky = kyG[j]``, column ``i`` holds
  ``kx = i``;
* real physical arrays are C-order ``(nyG, nxG)`` float64; element
  ``[jj, ii]`` is the reference's 1-based point ``(ii+1, jj+1)``;
* forward transforms are divided by ``nxG*nyG``, inverse transforms are not
  normalised (src/Spectral.F90:749-781).

The 2-D real DFTs come from FFTW 3.3.3 in the reference (a third-party
dependency that is not vendored: README:9-10, CMakeLists.txt:35-39).  FFTW
computes the textbook DFT ``X[k] = sum_n x[n] exp(-2 pi i k n / M)``
(FFTW_FORWARD, sign -1) and its unnormalised inverse; the oracle computes the
same transforms with pocketfft (``scipy.fft``), which implements the same
definition.  FFTW's c2r ignores the imaginary parts of the kx=0 and kx=M/2
columns' self-conjugate entries exactly as pocketfft's irfft does.

Quirks of the reference that are kept (see the reference's own line numbers):

* Q1: ``compute_psi`` uses the single-rank semantics (row 0 is ky=0).
* Q2: circular truncation ``|k| <= nx/2 (+1e-10)``.
* Q3: ``compute_rhs`` round-trips omega through C2R/R2C when
  ``round_trip=True`` (the default, as in the reference).
* Q4: physical sample ``i`` (1-based) sits at ``x = 2 pi i / nxG``.
* Q5: forward transform normalised, inverse not.
"""

from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

try:  # scipy's pocketfft is multi-threaded; numpy's is the fallback.
    import scipy.fft as _sfft

    def _rfft2(x, workers):
        return _sfft.rfft2(x, norm="forward", workers=workers)

    def _irfft2(c, shape, workers):
        return _sfft.irfft2(c, s=shape, norm="forward", workers=workers)

except ImportError:  # pragma: no cover - scipy is present on both machines
    def _rfft2(x, workers):
        return np.fft.rfft2(x, norm="forward")

    def _irfft2(c, shape, workers):
        return np.fft.irfft2(c, s=shape, norm="forward")


NO_DEALIASING = 0       # src/Spectral.F90:41
DEALIAS_3_2_RULE = 1    # src/Spectral.F90:43

#: number of FFT worker threads (results do not depend on it)
WORKERS = 1


def set_workers(n: int) -> None:
    """Set the pocketfft thread count used by the oracle's transforms."""
    global WORKERS
    WORKERS = max(1, int(n))


# --------------------------------------------------------------------------
# Grid, wavenumbers, masks and truncation
# --------------------------------------------------------------------------

@dataclass
class Grid:
    """Output of ``GetGridSize`` plus the masks and truncation bounds."""
    nx: int
    ny: int
    dealias: int
    nxG: int
    nyG: int
    kxLG: int
    kyLG: int
    kxMG: int
    kyMG: int
    kxLU: int
    kyLU: int
    kxMU: int
    kyMU: int
    kMax: float
    rISize: int
    cISize: int
    kxG: np.ndarray
    kyG: np.ndarray
    trunc_i1: np.ndarray = field(default=None)   # 0-based first truncated i per row
    xMaskInd: int = -1                           # 0-based, -1 = absent
    yMaskInd: int = -1

    @property
    def kx(self) -> np.ndarray:
        """kx as float64 broadcastable over ``(nyG, cISize)``."""
        return self.kxG.astype(np.float64)[None, :]

    @property
    def ky(self) -> np.ndarray:
        """ky as float64 broadcastable over ``(nyG, cISize)``."""
        return self.kyG.astype(np.float64)[:, None]


def get_grid_size(nx: int, ny: int, dealias: int = DEALIAS_3_2_RULE) -> Grid:
    """Restates ``GetGridSize`` (src/Spectral.F90:117-219).

    Fortran integer division truncates toward zero; all operands here are
    non-negative so ``//`` matches except ``-nyG/2``, written out explicitly.
    """
    if dealias == NO_DEALIASING:                      # :141-159
        nxG, nyG = nx, ny
        kxLG, kyLG = 0, -(nyG // 2) + 1
        kxMG, kyMG = nxG // 2, nyG // 2
        kxLU, kyLU = 0, -(ny // 2) + 1
        kxMU, kyMU = nx // 2, ny // 2
        kMax = float(kxMU)
    elif dealias == DEALIAS_3_2_RULE:                 # :160-179
        nxG, nyG = 3 * nx // 2, 3 * ny // 2
        kxLG, kyLG = 0, -(nyG // 2) + 1
        kxMG, kyMG = nxG // 2, nyG // 2
        kxLU, kyLU = 0, -(ny // 2) + 1
        kxMU, kyMU = nx // 2, ny // 2
        kMax = float(kxMU)
    else:
        # :180-185 -- 2/3 rule and grid shift are empty cases in the
        # reference (quirk Q7); the default case keeps the grid and leaves
        # the other outputs unset.  The oracle refuses instead.
        raise ValueError(f"dealias={dealias} is not implemented by the reference")
    rISize = 2 * (nxG // 2 + 1)                       # :189
    cISize = nxG // 2 + 1                             # :190
    kxG = np.arange(cISize, dtype=np.int64)           # :204-207
    kyt = np.arange(nyG, dtype=np.int64)              # :210-218
    kyG = np.where(kyt > nyG // 2, kyt - nyG, kyt)
    g = Grid(nx, ny, dealias, nxG, nyG, kxLG, kyLG, kxMG, kyMG,
             kxLU, kyLU, kxMU, kyMU, kMax, rISize, cISize, kxG, kyG)
    setup_mask(g)
    setup_truncation(g)
    return g


def setup_mask(g: Grid) -> None:
    """Restates ``SetupMask`` (src/Spectral.F90:229-260): index of kx==kxMG
    and ky==kyMG (0-based here), -1 when absent."""
    xs = np.nonzero(g.kxG == g.kxMG)[0]
    ys = np.nonzero(g.kyG == g.kyMG)[0]
    g.xMaskInd = int(xs[0]) if xs.size else -1
    g.yMaskInd = int(ys[0]) if ys.size else -1


def setup_truncation(g: Grid) -> None:
    """Restates ``SetupTruncation`` (src/Spectral.F90:272-313).

    For each row the first i with ``sqrt(kx**2+ky**2) > kMax + 1e-10`` starts
    the truncated range ``[i1, cISize)``.  A row with no such mode leaves
    ``trunc(j)`` unset in the reference (quirk Q7, only possible without
    dealiasing); the oracle then truncates nothing in that row.
    """
    eps = 1.0e-10
    kx = g.kxG.astype(np.float64)
    i1 = np.full(g.nyG, g.cISize, dtype=np.int64)
    for j in range(g.nyG):
        ky = float(g.kyG[j])
        kmag = np.sqrt(kx ** 2 + ky ** 2)
        hit = np.nonzero(kmag > g.kMax + eps)[0]
        if hit.size:
            i1[j] = int(hit[0])
    g.trunc_i1 = i1


def truncation_mask(g: Grid) -> np.ndarray:
    """Boolean ``(nyG, cISize)`` array, True where ``Truncate`` zeroes."""
    return np.arange(g.cISize)[None, :] >= g.trunc_i1[:, None]


def truncate(c: np.ndarray, g: Grid) -> np.ndarray:
    """Restates ``Truncate`` (src/Spectral.F90:788-802); returns a copy."""
    out = c.copy()
    out[truncation_mask(g)] = 0.0
    return out


# --------------------------------------------------------------------------
# Spectral operators
# --------------------------------------------------------------------------

def dudx(c: np.ndarray, g: Grid) -> np.ndarray:
    """Restates ``DuDx`` (src/Spectral.F90:662-693): ``i*kx*c``, then zero the
    kx==kxMG column when present."""
    out = (1j * g.kx) * c
    if g.xMaskInd >= 0:
        out[:, g.xMaskInd] = 0.0
    return out


def dudy(c: np.ndarray, g: Grid) -> np.ndarray:
    """Restates ``DuDy`` (src/Spectral.F90:708-738): ``i*ky*c``, then zero the
    ky==kyMG row when present."""
    out = (1j * g.ky) * c
    if g.yMaskInd >= 0:
        out[g.yMaskInd, :] = 0.0
    return out


def compute_psi(w: np.ndarray, g: Grid) -> np.ndarray:
    """Restates ``ComputePsi`` (src/Spectral.F90:508-560) with the single-rank
    semantics (quirk Q1): psi = w/(kx^2+ky^2), psi(0,0) = 0."""
    k2 = g.kx ** 2 + g.ky ** 2
    k2 = np.where(k2 == 0.0, 1.0, k2)
    psi = w / k2
    psi[0, 0] = 0.0
    return psi


def compute_velocity(psi: np.ndarray, g: Grid):
    """Restates ``ComputeVelocity`` (src/Spectral.F90:576-610) without the
    optional C2R: u = DuDy(psi), v = -DuDx(psi)."""
    u = dudy(psi, g)
    v = -1.0 * dudx(psi, g)
    return u, v


def compute_vorticity(u: np.ndarray, v: np.ndarray, g: Grid) -> np.ndarray:
    """Restates ``ComputeVorticity`` (src/Spectral.F90:624-647):
    w = DuDx(v) - DuDy(u)."""
    return dudx(v, g) - dudy(u, g)


def transform_r2c(r: np.ndarray, g: Grid) -> np.ndarray:
    """Restates ``TransformR2C`` (src/Spectral.F90:749-763): forward 2-D real
    DFT divided by ``nxG*nyG``."""
    return _rfft2(np.ascontiguousarray(r, dtype=np.float64), WORKERS)


def transform_c2r(c: np.ndarray, g: Grid) -> np.ndarray:
    """Restates ``TransformC2R`` (src/Spectral.F90:772-781): unnormalised
    inverse 2-D real DFT."""
    return _irfft2(np.ascontiguousarray(c, dtype=np.complex128), (g.nyG, g.nxG), WORKERS)


def compute_rhs(w: np.ndarray, psi: np.ndarray, g: Grid, nu: float,
                round_trip: bool = True, forcing: np.ndarray | None = None,
                alpha: float = 0.0):
    """Restates ``ComputeRHS`` (src/Spectral.F90:396-482).

    Returns ``(dW, w_out)``.  ``w_out`` is omega after the in-place C2R/R2C
    round trip of :435/:453 when ``round_trip`` (the reference's behaviour,
    quirk Q3), else ``w`` unchanged.

    ``forcing`` (a spectral source added to dW) and ``alpha`` (linear drag,
    ``-alpha*w`` added to dW) are extensions with no counterpart in the
    reference; they enter the dW expression of :479.
    """
    u, v = compute_velocity(psi, g)                   # :424
    uR = transform_c2r(u, g)                          # :433
    vR = transform_c2r(v, g)                          # :434
    wR = transform_c2r(w, g)                          # :435
    uR = uR * wR                                      # :442-447
    vR = vR * wR
    uC = transform_r2c(uR, g)                         # :451
    vC = transform_r2c(vR, g)                         # :452
    w_out = transform_r2c(wR, g) if round_trip else w  # :453
    uC = truncate(uC, g)                              # :457
    vC = truncate(vC, g)                              # :458
    uC = dudx(uC, g)                                  # :464
    vC = dudy(vC, g)                                  # :465
    dW = -uC - vC - (nu * (g.kx ** 2 + g.ky ** 2)) * w_out   # :471-481
    if alpha != 0.0:
        dW = dW - alpha * w_out
    if forcing is not None:
        dW = dW + forcing
    return dW, w_out


def integrate_one_step(w: np.ndarray, psi: np.ndarray, g: Grid, nu: float,
                       dt: float, round_trip: bool = True,
                       forcing: np.ndarray | None = None, alpha: float = 0.0):
    """Restates ``IntegrateOneStep`` (src/TimeIntegration.F90:130-210),
    Shu-Osher TVD-RK3 in the reference's operation order.  Returns the new
    ``(wC, psiC)``."""
    kw = dict(round_trip=round_trip, forcing=forcing, alpha=alpha)
    dW, w = compute_rhs(w, psi, g, nu, **kw)                       # :152
    wS = w + dt * dW                                               # :156-160
    psiS = truncate(compute_psi(wS, g), g)                         # :163-167
    wS = truncate(wS, g)
    dW, wS = compute_rhs(wS, psiS, g, nu, **kw)                    # :171
    wS = 0.75 * w + 0.25 * wS + 0.25 * dt * dW                     # :175-181
    psiS = truncate(compute_psi(wS, g), g)                         # :184-188
    wS = truncate(wS, g)
    dW, wS = compute_rhs(wS, psiS, g, nu, **kw)                    # :192
    w = w / 3.0 + 2.0 * wS / 3.0 + dt * 2.0 * dW / 3.0             # :196-202
    psi = truncate(compute_psi(w, g), g)                           # :205-209
    w = truncate(w, g)
    return w, psi


# --------------------------------------------------------------------------
# Initial conditions
# --------------------------------------------------------------------------

def physical_grid_1based(g: Grid):
    """Physical coordinates of the reference's points (quirk Q4,
    src/SetIC.F90:91-94): ``x = 2 pi i / nxG`` for 1-based i."""
    x = 2.0 * np.pi * np.arange(1, g.nxG + 1, dtype=np.float64) / float(g.nxG)
    y = 2.0 * np.pi * np.arange(1, g.nyG + 1, dtype=np.float64) / float(g.nyG)
    return x[None, :], y[:, None]


def set_taylor_green(g: Grid):
    """Restates ``SetTaylorGreen`` (src/SetIC.F90:70-101): fill psi and omega
    on the physical grid, then R2C both.  Returns ``(wC, psiC)``."""
    i = np.arange(1, g.nxG + 1, dtype=np.float64)
    j = np.arange(1, g.nyG + 1, dtype=np.float64)
    sx = np.sin(2.0 * np.pi * i / float(g.nxG))[None, :]
    sy = np.sin(2.0 * np.pi * j / float(g.nyG))[:, None]
    psiR = sx * sy
    wR = (2.0 * sx) * sy
    return transform_r2c(wR, g), transform_r2c(psiR, g)


def taylor_green_exact(g: Grid, nu: float, t: float):
    """Exact Taylor-Green fields at time t on the reference grid
    (src/SetIC.F90:45-56, analysis/TaylorGreen.py:88-96):
    returns ``(psi, w, u, v)`` physical arrays."""
    x, y = physical_grid_1based(g)
    F = math.exp(-2.0 * nu * t)
    psi = np.sin(x) * np.sin(y) * F
    return psi, 2.0 * psi, np.sin(x) * np.cos(y) * F, -np.cos(x) * np.sin(y) * F


def l2_error(dx, dy, a, b):
    """``L2Error`` of analysis/TaylorGreen.py:43-52 for one field."""
    return float(np.sqrt(np.sum(np.square(a - b)) * dx * dy))


def linf_error(a, b):
    """``LInfError`` of analysis/TaylorGreen.py:55-60 for one field."""
    return float(np.max(np.abs(a - b)))


# --- counter-based generator for reproducible initial conditions -----------
# The reference seeds the compiler RNG from /dev/urandom (src/Random.F90:59-69)
# and is not reproducible (quirk Q8).  The replacement draws each mode's phase
# from a hash of (seed, kx, ky): splitmix64 (Steele, Lea & Flood 2014) applied
# twice to a packed key.  The product's host generator implements the same
# function; tests compare the two bit for bit.

_MASK64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        x = (x + np.uint64(0x9E3779B97F4A7C15)) & _MASK64
        z = x
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _MASK64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _MASK64
        return z ^ (z >> np.uint64(31))


def mode_phase(seed: int, kx: np.ndarray, ky: np.ndarray) -> np.ndarray:
    """Uniform phase in [0, 2 pi) of mode (kx, ky): the top 53 bits of
    splitmix64(splitmix64(key)) with key = seed<<42 ^ kx<<21 ^ (ky mod 2^21)."""
    kx = np.asarray(kx, dtype=np.int64)
    ky = np.asarray(ky, dtype=np.int64)
    key = ((np.uint64(seed) << np.uint64(42))
           ^ (kx.astype(np.uint64) << np.uint64(21))
           ^ (ky.astype(np.uint64) & np.uint64(0x1FFFFF)))
    h = _splitmix64(_splitmix64(key))
    u = (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return 2.0 * np.pi * u


SPECTRUM_SCHUMANN = 0   # src/SetIC.F90:374-381
SPECTRUM_K4_GAUSS = 1   # E ~ k^4 exp(-2 (k/k0)^2): no counterpart in the reference


def spectrum_shape(kind: int, k: np.ndarray, k0: float, urms: float) -> np.ndarray:
    """Energy spectrum of one shell: ``Schumann`` (src/SetIC.F90:374-381) or
    the k^4 Gaussian spectrum of the decaying-turbulence workload."""
    if kind == SPECTRUM_SCHUMANN:
        return 1.5 * urms ** 2 * k / k0 * np.exp(-k / k0)
    if kind == SPECTRUM_K4_GAUSS:
        return k ** 4 * np.exp(-2.0 * (k / k0) ** 2)
    raise ValueError(kind)


def spectrum_bin_edges(g: Grid):
    """Bin edges of ``ComputeSpectrum``/``FourierVelocity``
    (src/Analysis.F90:325-362, src/SetIC.F90:269-292)."""
    kMax = math.sqrt(float(g.kxMG * g.kxMG + g.kyMG * g.kyMG))
    kIntMax = int(kMax + 1.0)
    numBin = kIntMax + 1
    edges = np.empty(numBin + 1, dtype=np.float64)
    edges[0] = 0.0
    edges[1:kIntMax + 1] = 0.5 + np.arange(kIntMax, dtype=np.float64)
    edges[numBin] = float(kIntMax) + 0.1
    return edges, numBin


def binary_search(fvec: np.ndarray, f: float) -> int:
    """Restates ``BinarySearch`` (src/Analysis.F90:475-513) literally.
    Returns the reference's 1-based index."""
    n = len(fvec)
    iL, iU = 0, n
    while iU - iL > 1:
        iM = (iL + iU) // 2
        if f >= fvec[iM - 1]:
            iL = iM
        else:
            iU = iM
    return iL


def binary_search_vec(fvec: np.ndarray, f: np.ndarray) -> np.ndarray:
    """Vectorised ``BinarySearch`` (1-based result, last bin closed)."""
    idx = np.searchsorted(fvec, f, side="right")
    return np.minimum(idx, len(fvec) - 1)


def _kmag(g: Grid) -> np.ndarray:
    return np.sqrt(g.kx ** 2 + g.ky ** 2) * np.ones((g.nyG, g.cISize))


def set_turbulent(g: Grid, seed: int, kind: int = SPECTRUM_K4_GAUSS,
                  k0: float = 10.0, urms: float = 1.0,
                  tke_target: float = 0.5):
    """Turbulent initial condition following ``SetTurbulentVelocity`` /
    ``FourierVelocity`` (src/SetIC.F90:125-151, :175-364), with three stated
    changes: the phase comes from :func:`mode_phase` (quirk Q8), omega on the
    kx=0 column is made Hermitian (ky<0 rows are conjugates of ky>0), and
    omega is rescaled so that ``compute_spectrum``'s TKE equals
    ``tke_target`` (no rescale when ``tke_target <= 0``).

    Returns ``(wC, psiC)``.
    """
    kmag = _kmag(g)
    E = spectrum_shape(kind, kmag, k0, urms)                              # :245
    theta = mode_phase(seed, g.kxG[None, :] * np.ones_like(kmag, dtype=np.int64),
                       g.kyG[:, None] * np.ones_like(kmag, dtype=np.int64))  # :248-249
    a = np.sqrt(E * 1.0) * np.exp(1j * theta)                              # :252
    safe = np.where(kmag == 0.0, 1.0, kmag)
    u = -1.0 * a * g.ky / safe                                             # :259
    v = a * g.kx / safe                                                    # :260
    u[0, 0] = 0.0                                                          # :255-257
    v[0, 0] = 0.0
    edges, numBin = spectrum_bin_edges(g)                                  # :269-292
    idx = binary_search_vec(edges, kmag)                                   # :310
    cnt = np.where((g.kxG[None, :] == 0) | (g.kxG[None, :] == g.kxMG), 1, 2)  # :316-320
    cnt = np.broadcast_to(cnt, kmag.shape)
    binCnt = np.zeros(numBin + 1, dtype=np.int64)
    np.add.at(binCnt, idx, cnt)                                            # :323
    norm = np.sqrt(binCnt[idx].astype(np.float64))                         # :351-352
    u = u / norm
    v = v / norm
    u = truncate(u, g)                                                     # :357-358
    v = truncate(v, g)
    w = compute_vorticity(u, v, g)                                         # SetIC.F90:147
    w = hermitian_kx0(w, g)
    w[0, 0] = 0.0
    if tke_target > 0.0:
        psi = compute_psi(w, g)
        uu, vv = compute_velocity(psi, g)
        _, _, tke, _, _ = compute_spectrum(uu, vv, g, 0.0)
        if tke > 0.0:
            w = w * math.sqrt(tke_target / tke)
    psi = compute_psi(w, g)                                                # SetIC.F90:150
    return w, psi


def hermitian_kx0(w: np.ndarray, g: Grid) -> np.ndarray:
    """Make the kx=0 column Hermitian: w(0,-ky) = conj(w(0,ky)) for ky>0
    (and the ky=kyMG self-conjugate entry real)."""
    out = w.copy()
    for j in range(g.nyG):
        ky = int(g.kyG[j])
        if ky < 0 and -ky <= g.nyG // 2:
            jp = -ky  # row of +|ky|
            out[j, 0] = np.conj(w[jp, 0])
    if g.nyG % 2 == 0:
        jn = g.nyG // 2
        out[jn, 0] = out[jn, 0].real
    out[0, 0] = out[0, 0].real
    return out


# --------------------------------------------------------------------------
# Diagnostics
# --------------------------------------------------------------------------

def compute_spectrum(u: np.ndarray, v: np.ndarray, g: Grid, nu: float):
    """Restates ``ComputeSpectrum`` (src/Analysis.F90:267-460).

    Returns ``(kBin, Ek, tke, eps, enstDiss)``; bins are in the reference's
    1-based order (``kBin[i] = i`` here, 0-based).
    """
    edges, numBin = spectrum_bin_edges(g)
    kmag = _kmag(g)
    Ehat = (u * np.conj(u) + v * np.conj(v)).real                       # :380
    idx = binary_search_vec(edges, kmag)                                # :383
    half = (g.kxG[None, :] == 0) | (g.kxG[None, :] == g.kxMG)           # :389
    contrib = np.where(half, 0.5 * Ehat, Ehat)
    Ek = np.zeros(numBin + 1, dtype=np.float64)
    np.add.at(Ek, idx, contrib)
    Ek = Ek[1:] / 1.0                                                   # :419 (dk = 1)
    kBin = np.arange(numBin, dtype=np.float64)
    tke = float(np.sum(Ek * 1.0))                                       # :443
    eps = 2.0 * nu * float(np.sum(kBin ** 2 * Ek * 1.0))                # :444, :447
    enst = 2.0 * nu * float(np.sum(kBin ** 4 * Ek * 1.0))               # :445, :448
    return kBin, Ek, tke, eps, enst


def spectrum_of_vorticity(w: np.ndarray, g: Grid, nu: float):
    """``ComputeVelocity`` + ``ComputeSpectrum`` as called from ``Analysis``
    (src/Analysis.F90:230-234)."""
    psi = compute_psi(w, g)
    u, v = compute_velocity(psi, g)
    return compute_spectrum(u, v, g, nu)


def enstrophy(w: np.ndarray, g: Grid) -> float:
    """Mean enstrophy 1/2 <omega^2> from the stored half spectrum (kx>0
    modes counted twice).  No counterpart in the reference."""
    wt = np.where(g.kxG[None, :] == 0, 1.0, 2.0)
    return 0.5 * float(np.sum(wt * (w * np.conj(w)).real))


def minmax_abs(w: np.ndarray, psi: np.ndarray):
    """Max/min |w| and |psi| over the whole stored array, as printed by the
    driver (src/Spectral2D.F90:358-361)."""
    aw, ap = np.abs(w), np.abs(psi)
    return float(aw.max()), float(aw.min()), float(ap.max()), float(ap.min())


def skewness(w: np.ndarray, psi: np.ndarray, g: Grid):
    """x and y vorticity-gradient skewness of ``Analysis``
    (src/Analysis.F90:135-225)."""
    u, v = compute_velocity(psi, g)
    ux = dudx(u, g)
    wx = dudx(w, g)
    uR = transform_c2r(ux, g)
    vR = transform_c2r(wx, g)
    fact = float(g.nxG) * float(g.nyG)
    s1 = np.sum(uR * vR ** 2) / fact
    s2 = np.sum(uR ** 2) / fact
    s3 = np.sum(vR ** 2) / fact
    xs = -2.0 * s1 / (math.sqrt(s2) * s3)
    u, v = compute_velocity(psi, g)
    vy = dudy(v, g)
    wy = dudy(w, g)
    vR = transform_c2r(vy, g)
    uR = transform_c2r(wy, g)
    s1 = np.sum(vR * uR ** 2) / fact
    s2 = np.sum(vR ** 2) / fact
    s3 = np.sum(uR ** 2) / fact
    ys = -2.0 * s1 / (math.sqrt(s2) * s3)
    return float(xs), float(ys)


def cfl_dt(w: np.ndarray, g: Grid, cfl: float) -> float:
    """CFL time step ``cfl / max(|u|/dx + |v|/dy)`` on the collocation grid.
    Fills the empty ``ComputeTimeStep`` stub (src/TimeIntegration.F90:213-215);
    no counterpart in the reference's arithmetic."""
    psi = compute_psi(w, g)
    u, v = compute_velocity(psi, g)
    uR = transform_c2r(u, g)
    vR = transform_c2r(v, g)
    dx = 2.0 * np.pi / g.nxG
    dy = 2.0 * np.pi / g.nyG
    m = float(np.max(np.abs(uR) / dx + np.abs(vR) / dy))
    return cfl / m


def kolmogorov_forcing(g: Grid, amp: float, kf: int) -> np.ndarray:
    """Spectral source of the vorticity forcing ``amp*cos(kf*y)`` sampled on
    the reference grid (y_j = 2 pi j / nyG, 1-based, quirk Q4): coefficient
    ``amp/2 * exp(+-i kf dy)`` at (kx=0, ky=+-kf)."""
    f = np.zeros((g.nyG, g.cISize), dtype=np.complex128)
    dy = 2.0 * np.pi / g.nyG
    f[kf % g.nyG, 0] = 0.5 * amp * np.exp(1j * kf * dy)
    f[(-kf) % g.nyG, 0] = 0.5 * amp * np.exp(-1j * kf * dy)
    return f


def spectral_filter(c: np.ndarray, g: Grid, kc: float) -> np.ndarray:
    """Sharp spectral cut-off ``|k| <= kc`` (a ``Truncate``-style mask with a
    smaller radius, src/Spectral.F90:788-802)."""
    k2 = g.kx ** 2 + g.ky ** 2
    return np.where(k2 <= kc * kc + 1e-10, c, 0.0)


# --------------------------------------------------------------------------
# Layout helpers (reference layout <-> compact retained rectangle)
# --------------------------------------------------------------------------

def retained_rows(g: Grid) -> np.ndarray:
    """Reference row indices j of ky = 0..K, -K..-1 (K = nx/2), i.e. the
    compact column order used by the device state."""
    K = g.nx // 2
    ky = np.concatenate([np.arange(0, K + 1), np.arange(-K, 0)])
    return ky % g.nyG


def to_compact(c: np.ndarray, g: Grid) -> np.ndarray:
    """Reference ``(nyG, cISize)`` -> compact ``(K+1, 2K+1)`` [kx][ky']."""
    K = g.nx // 2
    return np.ascontiguousarray(c[retained_rows(g), :K + 1].T)


def from_compact(cc: np.ndarray, g: Grid) -> np.ndarray:
    """Compact ``(K+1, 2K+1)`` -> reference layout with zeros elsewhere."""
    K = g.nx // 2
    out = np.zeros((g.nyG, g.cISize), dtype=np.complex128)
    out[retained_rows(g), :K + 1] = cc.T
    return out


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    """Relative L2 error ||a-b|| / ||b||."""
    nb = float(np.linalg.norm(b))
    return float(np.linalg.norm(a - b)) / (nb if nb > 0 else 1.0)


def random_state(g: Grid, seed: int, decay: float = 0.0) -> np.ndarray:
    """Band-limited random omega for parity tests: independent Gaussian
    coefficients on every retained mode (|k| <= nx/2), Hermitian kx=0 column,
    zero mean.  ``decay`` > 0 multiplies by exp(-decay*|k|)."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((g.nyG, g.cISize)) + 1j * rng.standard_normal((g.nyG, g.cISize))
    if decay > 0:
        w = w * np.exp(-decay * _kmag(g))
    w = truncate(w, g)
    w = hermitian_kx0(w, g)
    w[0, 0] = 0.0
    return w


def cpu_count() -> int:
    """Host cores available to this process."""
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1
