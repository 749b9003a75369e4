"""CPU restatement of one rank's slab of a decomposed run (test
infrastructure only).

The phases of the library's s2d_slab_* entry points (K1 on the rank's kx
columns, K2 on its physical rows, K3 and the RK3 stage update on its
columns) restated in numpy FP64 with the same partition and the same
exchange-buffer layout, so that the host-side orchestration
(``spectral2d_gb300.slab.rk3_step``) and a real all-to-all between processes
(gloo) can be run and checked on CPU, against the whole-run oracle
(``integrate_one_step``, src/TimeIntegration.F90:130-210).

The arithmetic is that of ``compute_rhs`` (src/Spectral.F90:396-482) in the
Basdevant form, split along the two transform axes:
  K1: u = i ky psi, v = -i kx psi (psi = w / k^2) on the retained modes,
      inverse y-DFT (unnormalised) of each column -> I[y, kx];
  K2: per row y, the c2r x-DFT of I[y, :] (kx <= K, the rest zero) -> u, v
      on the M-point row, the products u v and v^2 - u^2, their r2c x-DFT
      divided by M^2 (the 2-D forward normalisation), kx <= K kept;
  K3: forward y-DFT of each column, then
      dW = (kx^2 - ky^2) F[u v] + kx ky F[v^2 - u^2] - nu k^2 w,
      the TVD-RK3 stage combination and Truncate.
"""

from __future__ import annotations

import numpy as np

from . import spectral_oracle as O


def partition(nx: int, nranks: int):
    """kx0, nkx, y0, ny per rank: balanced contiguous ranges (floor(r n / P))."""
    K = nx // 2
    KX, M = K + 1, 3 * nx // 2
    out = []
    for r in range(nranks):
        a, b = r * KX // nranks, (r + 1) * KX // nranks
        c, d = r * M // nranks, (r + 1) * M // nranks
        out.append((a, b - a, c, d - c))
    return out


class SlabPhasesCPU:
    """Rank ``rank`` of ``nranks``: full-size arrays, only its own columns
    and rows computed, the library's exchange layout."""

    def __init__(self, nx: int, nu: float, rank: int, nranks: int):
        self.nx, self.nu, self.rank, self.nranks = nx, nu, rank, nranks
        self.g = O.get_grid_size(nx, nx)
        self.K, self.M = nx // 2, 3 * nx // 2
        self.parts = partition(nx, nranks)
        self.kx0, self.nkx, self.y0, self.ny = self.parts[rank]
        KX = self.K + 1
        self.I = np.zeros((2, self.M, KX), dtype=np.complex128)
        n = max(2 * self.M * self.nkx, 2 * self.ny * KX)
        self.send = np.zeros(n, dtype=np.complex128)
        self.recv = np.zeros(n, dtype=np.complex128)
        self.S0 = np.zeros((self.M, self.g.cISize), dtype=np.complex128)
        self.S1 = np.zeros_like(self.S0)
        self.mask = O.truncation_mask(self.g)   # True where Truncate zeroes

    def set_state(self, w: np.ndarray) -> None:
        self.S0 = O.truncate(w, self.g)

    def synchronize(self) -> None:
        pass

    # segment tables, as the library's: (row0, nrows, col0, ncols) per rank
    def _segments(self, e: int):
        snd, rcv = [], []
        r = self.rank
        for q in range(self.nranks):
            kq, nq, yq, mq = self.parts[q]
            if e == 0:
                snd.append((yq, mq, self.kx0, self.nkx))
                rcv.append((self.y0, self.ny, kq, nq))
            else:
                snd.append((self.y0, self.ny, kq, nq))
                rcv.append((yq, mq, self.kx0, self.nkx))
        return snd, rcv

    def exchange_layout(self, e: int):
        snd, rcv = self._segments(e)
        sb = [2 * s[1] * s[3] * 16 for s in snd]
        rb = [2 * s[1] * s[3] * 16 for s in rcv]
        return self.send, self.recv, sb, rb

    def _copy(self, segs, buf, pack: bool) -> None:
        off = 0
        for (r0, nr, c0, nc) in segs:
            for f in range(2):
                blk = buf[off:off + nr * nc].reshape(nr, nc) if nr * nc else None
                if nr * nc:
                    if pack:
                        blk[...] = self.I[f, r0:r0 + nr, c0:c0 + nc]
                    else:
                        self.I[f, r0:r0 + nr, c0:c0 + nc] = blk
                off += nr * nc

    def phase(self, stage: int, phase: int, dt: float) -> None:
        g, K, M = self.g, self.K, self.M
        cols = slice(self.kx0, self.kx0 + self.nkx)
        if phase == 0:
            w = (self.S0 if stage <= 1 else self.S1)[:, cols]
            kx = g.kxG[cols][None, :].astype(np.float64)
            ky = g.kyG[:, None].astype(np.float64)
            k2 = kx * kx + ky * ky
            psi = np.where(k2 == 0, 0.0, w / np.where(k2 == 0, 1.0, k2))
            psi[self.mask[:, cols]] = 0.0
            u = 1j * ky * psi
            v = -1j * kx * psi
            # inverse y-DFT, unnormalised
            self.I[0][:, cols] = np.fft.ifft(u, axis=0) * M
            self.I[1][:, cols] = np.fft.ifft(v, axis=0) * M
            self._copy(self._segments(0)[0], self.send, pack=True)
        elif phase == 1:
            self._copy(self._segments(0)[1], self.recv, pack=False)
            rows = slice(self.y0, self.y0 + self.ny)
            half = M // 2 + 1
            X = np.zeros((2, self.ny, half), dtype=np.complex128)
            X[:, :, :K + 1] = self.I[:, rows, :]
            u = np.fft.irfft(X[0], n=M, axis=1) * M
            v = np.fft.irfft(X[1], n=M, axis=1) * M
            a = np.fft.rfft(u * v, axis=1)[:, :K + 1] / (M * M)
            b = np.fft.rfft(v * v - u * u, axis=1)[:, :K + 1] / (M * M)
            self.I[0][rows, :] = a
            self.I[1][rows, :] = b
            self._copy(self._segments(1)[0], self.send, pack=True)
        else:
            self._copy(self._segments(1)[1], self.recv, pack=False)
            Fa = np.fft.fft(self.I[0][:, cols], axis=0)
            Fb = np.fft.fft(self.I[1][:, cols], axis=0)
            kx = g.kxG[cols][None, :].astype(np.float64)
            ky = g.kyG[:, None].astype(np.float64)
            win = (self.S0 if stage <= 1 else self.S1)[:, cols]
            dW = (kx * kx - ky * ky) * Fa + kx * ky * Fb - self.nu * (kx * kx + ky * ky) * win
            w0 = self.S0[:, cols]
            if stage == 1:
                out = w0 + dt * dW
            elif stage == 2:
                out = 0.75 * w0 + 0.25 * win + 0.25 * dt * dW
            else:
                out = w0 / 3.0 + 2.0 * win / 3.0 + 2.0 * dt * dW / 3.0
            out[self.mask[:, cols]] = 0.0
            if stage == 3:
                self.S0[:, cols] = out
            else:
                self.S1[:, cols] = out

    def get_columns(self, w=None, psi=None):
        if w is None:
            w = np.zeros_like(self.S0)
        if psi is None:
            psi = np.zeros_like(self.S0)
        cols = slice(self.kx0, self.kx0 + self.nkx)
        w[:, cols] = self.S0[:, cols]
        psi[:, cols] = O.truncate(O.compute_psi(self.S0, self.g), self.g)[:, cols]
        return w, psi
