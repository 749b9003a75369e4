"""Generate exact golden vectors for the Spectral2D RHS and one RK3 step.

The reference ships no tests or fixtures, and it cannot be built here
(Fortran + FFTW-MPI + HDF5 are absent).  These vectors pin its algorithm
instead, computed in exact rational arithmetic with no FFT at all:

* omega is a band-limited Fourier series with float64 coefficients (converted
  to exact ``Fraction``s), Hermitian on the kx=0 column;
* psi = omega/k^2, u = i ky psi, v = -i kx psi (src/Spectral.F90:508-610);
* the reference's C2R -> pointwise product -> R2C/(nxG*nyG) on the 3/2 grid
  (src/Spectral.F90:433-453) equals, exactly, the cyclic convolution of the
  full-plane coefficient sets with indices taken modulo (nxG, nyG) -- the
  aliasing of the kx=+-N and ky=+-N products onto the kept +-N/2 modes
  included;
* then Truncate, i kx / i ky and the viscous term (src/Spectral.F90:457-481),
  and the TVD-RK3 stage arithmetic (src/TimeIntegration.F90:146-209).

Outputs are float64 roundings of the exact results, in the reference layout
``(nyG, cISize)`` complex128.  Run ``python tests/golden/make_golden.py`` to
regenerate (a few seconds).
"""

from __future__ import annotations

import os
import sys
from fractions import Fraction as Fr

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


class Grid:
    def __init__(self, n):
        self.n = n
        self.K = n // 2
        self.M = 3 * n // 2
        self.C = self.M // 2 + 1

    def ky_of_row(self, j):
        return j - self.M if j > self.M // 2 else j

    def row_of_ky(self, ky):
        return ky % self.M

    def kept(self, kx, ky):
        return kx * kx + ky * ky <= self.K * self.K


def cmul(a, b):
    return (a[0] * b[0] - a[1] * b[1], a[0] * b[1] + a[1] * b[0])


def cadd(a, b):
    return (a[0] + b[0], a[1] + b[1])


def cscale(s, a):
    return (s * a[0], s * a[1])


ZERO = (Fr(0), Fr(0))


def random_omega(g: Grid, seed: int):
    """Half-plane dict {(kx,ky): (re,im)} with dyadic float64 coefficients."""
    rng = np.random.default_rng(seed)
    w = {}
    for kx in range(0, g.K + 1):
        for ky in range(-g.K, g.K + 1):
            if not g.kept(kx, ky) or (kx == 0 and ky <= 0):
                continue
            re = float(rng.integers(-64, 65)) / 16.0
            im = float(rng.integers(-64, 65)) / 16.0
            w[(kx, ky)] = (Fr(re), Fr(im))
    for ky in range(1, g.K + 1):   # Hermitian kx=0 column
        re, im = w[(0, ky)]
        w[(0, -ky)] = (re, -im)
    return w


def full_plane(half):
    """Hermitian extension of a half-plane dict to all (kx, ky)."""
    out = dict(half)
    for (kx, ky), c in half.items():
        if kx > 0:
            out[(-kx, -ky)] = (c[0], -c[1])
    return out


def cyclic_product(a_full, b_full, g: Grid):
    """Coefficients of the pointwise product on the M x M grid: cyclic
    convolution with wavenumbers wrapped to (-M/2, M/2]."""
    out = {}
    for (k1x, k1y), ca in a_full.items():
        for (k2x, k2y), cb in b_full.items():
            kx = (k1x + k2x) % g.M
            ky = (k1y + k2y) % g.M
            if kx > g.M // 2:
                kx -= g.M
            if ky > g.M // 2:
                ky -= g.M
            p = cmul(ca, cb)
            out[(kx, ky)] = cadd(out.get((kx, ky), ZERO), p)
    return out


def rhs(w_half, g: Grid, nu: Fr):
    """Exact dW on the kept half-plane modes, following ComputeRHS."""
    psi = {}
    for (kx, ky), c in w_half.items():
        k2 = kx * kx + ky * ky
        psi[(kx, ky)] = ZERO if k2 == 0 else cscale(Fr(1, k2), c)
    u = {k: cmul((Fr(0), Fr(k[1])), c) for k, c in psi.items()}        # i ky psi
    v = {k: cmul((Fr(0), Fr(-k[0])), c) for k, c in psi.items()}       # -i kx psi
    wf = full_plane(w_half)
    uw = cyclic_product(full_plane(u), wf, g)
    vw = cyclic_product(full_plane(v), wf, g)
    dW = {}
    for kx in range(0, g.K + 1):
        for ky in range(-g.K, g.K + 1):
            if not g.kept(kx, ky):
                continue
            a = uw.get((kx, ky), ZERO)
            b = vw.get((kx, ky), ZERO)
            nl = cadd(cmul((Fr(0), Fr(kx)), a), cmul((Fr(0), Fr(ky)), b))
            wv = w_half.get((kx, ky), ZERO)
            visc = cscale(nu * (kx * kx + ky * ky), wv)
            dW[(kx, ky)] = (-nl[0] - visc[0], -nl[1] - visc[1])
    return dW


def lin(*terms):
    """sum of s_i * dict_i over the union of keys."""
    keys = set()
    for _, d in terms:
        keys |= set(d)
    out = {}
    for k in keys:
        acc = ZERO
        for s, d in terms:
            acc = cadd(acc, cscale(s, d.get(k, ZERO)))
        out[k] = acc
    return out


def rk3_step(w, g, nu, dt):
    d1 = rhs(w, g, nu)
    w1 = lin((Fr(1), w), (dt, d1))
    d2 = rhs(w1, g, nu)
    w2 = lin((Fr(3, 4), w), (Fr(1, 4), w1), (dt / 4, d2))
    d3 = rhs(w2, g, nu)
    return lin((Fr(1, 3), w), (Fr(2, 3), w2), (dt * 2 / 3, d3))


def to_ref_layout(d, g: Grid):
    out = np.zeros((g.M, g.C), dtype=np.complex128)
    for (kx, ky), c in d.items():
        if 0 <= kx < g.C:
            out[g.row_of_ky(ky), kx] = float(c[0]) + 1j * float(c[1])
    return out


def psi_of(d, g):
    out = {}
    for (kx, ky), c in d.items():
        k2 = kx * kx + ky * ky
        out[(kx, ky)] = ZERO if k2 == 0 else cscale(Fr(1, k2), c)
    return out


def main():
    nu = Fr(0.01)
    dt = Fr(0.001)
    for n, seed in ((8, 11), (16, 12)):
        g = Grid(n)
        w = random_omega(g, seed)
        dW = rhs(w, g, nu)
        np.savez_compressed(os.path.join(HERE, f"rhs_exact_n{n}.npz"),
                            n=n, nu=float(nu), w=to_ref_layout(w, g),
                            dW=to_ref_layout(dW, g))
        print(f"rhs n={n}: {len(w)} modes", file=sys.stderr)
    g = Grid(8)
    w = random_omega(g, 13)
    w_new = rk3_step(w, g, nu, dt)
    np.savez_compressed(os.path.join(HERE, "step_exact_n8.npz"),
                        n=8, nu=float(nu), dt=float(dt), w=to_ref_layout(w, g),
                        w_new=to_ref_layout(w_new, g),
                        psi_new=to_ref_layout(psi_of(w_new, g), g))
    print("step n=8 done", file=sys.stderr)


if __name__ == "__main__":
    main()
