// s2d_step.cuh -- bodies of the three right-hand-side kernels, shared by the
// single-run kernels (s2d_kernels.cu) and the persistent ensemble kernel
// (s2d_batch.cu).  A body processes one "block" (a tile of columns or rows)
// with all threads of the calling CTA and the shared memory it is given.
//
// Intermediates are read with ld.global.cg (L2, not L1): in the persistent
// kernel they were written by other CTAs of the same launch.
#pragma once

#include "s2d_fft.cuh"
#include "s2d_internal.h"
#include "s2d_xpass32.cuh"

namespace s2d {

__device__ __forceinline__ bool bits_nonfinite(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return (b & 0x7FF0000000000000ULL) == 0x7FF0000000000000ULL;
}
__device__ __forceinline__ bool bits_nonfinite(float x) {
    const unsigned int b = (unsigned int)__float_as_int(x);
    return (b & 0x7F800000u) == 0x7F800000u;
}

// compact row jc -> ky
__device__ __forceinline__ int ky_of_jc(const Dims& d, int jc) { return jc <= d.K ? jc : jc - d.KY; }

// w times the real factor s computed in FP64: in FP64 as is; in FP32 the
// factor is rounded once and the product taken in FP32, so that the FP32
// variant spends 3 FP64-pipe instructions per element (ky -> double, the
// product with 1/k^2, the rounding) instead of 8.
// With rot, i s w = (-s w.y, s w.x).
template <typename VT>
__device__ __forceinline__ VT scale_by(VT w, double s, bool rot) {
    using T = decltype(w.x);
    if constexpr (sizeof(T) == 4) {
        const T f = (T)s;
        return rot ? mk<VT>(-f * w.y, f * w.x) : mk<VT>(f * w.x, f * w.y);
    } else {
        return rot ? mk<VT>(-s * w.y, s * w.x) : mk<VT>(s * w.x, s * w.y);
    }
}

// Apply a spectral operator to omega of mode (kx, ky); 1/k^2 is FP64.
template <typename VT>
__device__ __forceinline__ VT apply_op(int op, VT w, int kx, int ky, double rk2) {
    using T = decltype(w.x);
    switch (op) {
        case OP_U:  // u = i ky psi = (-ky psi.y, ky psi.x)
            return scale_by(w, (double)ky * rk2, true);
        case OP_V:  // v = -i kx psi = (kx psi.y, -kx psi.x)
            return scale_by(w, -(double)kx * rk2, true);
        case OP_PSI:
            return scale_by(w, rk2, false);
        case OP_WX:
            return mk<VT>((T)(-kx) * w.y, (T)kx * w.x);
        case OP_WY:
            return mk<VT>((T)(-ky) * w.y, (T)ky * w.x);
        case OP_UX:  // i kx u = -kx ky psi
            return scale_by(w, -(double)kx * (double)ky * rk2, false);
        case OP_VY:  // i ky v = kx ky psi
            return scale_by(w, (double)kx * (double)ky * rk2, false);
        case OP_TU:  // as OP_U / OP_V, rk2 being the factor itself
        case OP_TV:
            return scale_by(w, rk2, true);
        default:
            return w;
    }
}

// ------------------------------------------------------------------------
// K1: inverse y-pass.  blk selects field (blk / ncg) and the column tile
// [cg*G, cg*G+G); G transforms of Tg threads each.
// ------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void yinv_body(const Dims& d, const typename Vec<T>::t* __restrict__ S,
                                          const double* __restrict__ rk2, const FieldSet& fs,
                                          const typename Vec<T>::t* __restrict__ tw, int G, int blk,
                                          typename Vec<T>::t* bufs) {
    using VT = typename Vec<T>::t;
    const int g = threadIdx.x / d.Tg;
    const int lane = threadIdx.x - g * d.Tg;
    const int ncg = (d.KX + G - 1) / G;
    const int f = blk / ncg;
    const int cg = blk - f * ncg;
    const int kx0 = cg * G;
    const int kx = kx0 + g;
    const bool active = kx < d.KX && g < G;
    // select without dynamic indexing of the parameter struct
    int op;
    void* outp;
    const double* tab;
    const float* tabf;
    switch (f) {
        case 0: op = fs.op[0]; outp = fs.out[0]; tab = fs.tab[0]; tabf = fs.tabf[0]; break;
        case 1: op = fs.op[1]; outp = fs.out[1]; tab = fs.tab[1]; tabf = fs.tabf[1]; break;
        case 2: op = fs.op[2]; outp = fs.out[2]; tab = fs.tab[2]; tabf = fs.tabf[2]; break;
        default: op = fs.op[3]; outp = fs.out[3]; tab = fs.tab[3]; tabf = fs.tabf[3]; break;
    }
    const bool tfac = op == OP_TU || op == OP_TV;
    if (tfac) rk2 = tab;   // the factor table takes the 1/k^2 table's place
    // FP32 with the factors pre-rounded: read them as FP32 (the same values)
    const bool f32tab = sizeof(T) == 4 && tfac && tabf != nullptr;
    VT* buf = bufs + (size_t)g * d.M;

    const VT* col = S + (size_t)(active ? kx : 0) * d.ldS;
    const double* rcol = rk2 + (size_t)(active ? kx : 0) * d.ldS;
    const float* fcol = f32tab ? tabf + (size_t)(active ? kx : 0) * d.ldS : nullptr;
    // M = kElemsPerThread * Tg: a fixed trip count lets every load of the
    // column be in flight at once (the loads are latency-bound)
#pragma unroll
    for (int i = 0; i < kElemsPerThread; ++i) {
        const int n = lane + i * d.Tg;
        VT val = mk<VT>((T)0, (T)0);
        int jc = -1, ky = 0;
        if (n <= d.K) {
            jc = n;
            ky = n;
        } else if (n >= d.M - d.K) {
            ky = n - d.M;
            jc = ky + d.KY;
        }
        if (active && jc >= 0) {
            if (f32tab) {   // i f w, as scale_by forms it from the FP64 factor
                const VT w = __ldcg(&col[jc]);
                const T fv = (T)fcol[jc];
                val = mk<VT>(-fv * w.y, fv * w.x);
            } else {
                val = apply_op(op, __ldcg(&col[jc]), kx, ky, rcol[jc]);
            }
        }
        buf[n] = val;
    }
    fft_run<true>(buf, d, lane, tw);

    VT* out = reinterpret_cast<VT*>(outp);
    const int gtot = min(G, d.KX - kx0);
    if (G == 1) {   // no integer division per element (it competes with the FP64 pipe)
        for (int y = threadIdx.x; y < d.M; y += blockDim.x) out[(size_t)y * d.ldI + kx0] = bufs[y];
    } else {
        const DivBy byG(G);
        for (int idx = threadIdx.x; idx < d.M * G; idx += blockDim.x) {
            const int y = byG(idx);
            const int gg = idx - y * G;
            if (gg < gtot) out[(size_t)y * d.ldI + kx0 + gg] = bufs[(size_t)gg * d.M + y];
        }
    }
}

// Hermitian extension of two half-spectrum rows X, Y (kx in [0,K]) packed as
// Z = X + iY over the full length M; the kx=0 entries contribute their real
// parts only (the c2r convention of FFTW, used by src/Spectral.F90:780).
template <typename VT>
__device__ __forceinline__ void build_pair(VT* buf, const VT* __restrict__ X, const VT* __restrict__ Y,
                                           const Dims& d, int lane, bool active) {
    using T = decltype(buf[0].x);
    // M = kElemsPerThread * Tg; all loads in flight for FP32 (FP64 K2 would
    // spill at its 80-register budget)
#pragma unroll(sizeof(T) == 8 ? 1 : kElemsPerThread)
    for (int i = 0; i < kElemsPerThread; ++i) {
        const int n = lane + i * d.Tg;
        VT z = mk<VT>((T)0, (T)0);
        if (active) {
            if (n == 0) {
                z = mk<VT>(__ldcg(&X[0]).x, __ldcg(&Y[0]).x);
            } else if (n <= d.K) {
                const VT a = __ldcg(&X[n]), b = __ldcg(&Y[n]);
                z = mk<VT>(a.x - b.y, a.y + b.x);
            } else if (n >= d.M - d.K) {
                const VT a = __ldcg(&X[d.M - n]), b = __ldcg(&Y[d.M - n]);
                z = mk<VT>(a.x + b.y, b.x - a.y);
            }
        }
        buf[n] = z;
    }
}

// Split the forward FFT P of p = a + i b (a, b real rows) into the half
// spectra A(k) = (P(k) + conj P(M-k))/2 and B(k) = (P(k) - conj P(M-k))/(2i),
// k in [0, K], times scale.
template <typename VT>
__device__ __forceinline__ void extract_pair(const VT* buf, VT* A, VT* B, const Dims& d, int lane,
                                             bool active, decltype(buf[0].x) scale) {
    if (!active) return;
    if (scale == (decltype(scale))1) {   // products of prescaled u, v: no multiply
        for (int k = lane; k <= d.K; k += d.Tg) {
            const VT p = buf[k];
            const VT q = buf[k == 0 ? 0 : d.M - k];
            A[k] = mk<VT>(p.x + q.x, p.y - q.y);
            B[k] = mk<VT>(p.y + q.y, q.x - p.x);
        }
        return;
    }
    for (int k = lane; k <= d.K; k += d.Tg) {
        const VT p = buf[k];
        const VT q = buf[k == 0 ? 0 : d.M - k];
        A[k] = mk<VT>((p.x + q.x) * scale, (p.y - q.y) * scale);
        B[k] = mk<VT>((p.y + q.y) * scale, (q.x - p.x) * scale);
    }
}

// ------------------------------------------------------------------------
// K2 (Basdevant form): one physical row per transform, rows [blk*G, blk*G+G).
// z = u + i v from one inverse FFT, then p = u v + i (v^2 - u^2), one forward
// FFT, split into the normalised half spectra of u v (-> Iu row) and
// v^2 - u^2 (-> Iv row).  Two complex FFTs per row.
// ------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void xpass_bas_body(const Dims& d, typename Vec<T>::t* Iu, typename Vec<T>::t* Iv,
                                               const typename Vec<T>::t* __restrict__ tw, int G, T scale,
                                               int blk, typename Vec<T>::t* bufs) {
    using VT = typename Vec<T>::t;
    const int g = threadIdx.x / d.Tg;
    const int lane = threadIdx.x - g * d.Tg;
    const int y = blk * G + g;
    const bool active = y < d.rows && g < G;
    VT* Z = bufs + (size_t)g * d.M;
    VT* urow = Iu + (size_t)(active ? y : 0) * d.ldI;
    VT* vrow = Iv + (size_t)(active ? y : 0) * d.ldI;
    build_pair(Z, urow, vrow, d, lane, active);
    fft_run<true>(Z, d, lane, tw);
    for (int n = lane; n < d.M; n += d.Tg) {
        const VT z = Z[n];
        Z[n] = mk<VT>(z.x * z.y, z.y * z.y - z.x * z.x);
    }
    fft_run<false>(Z, d, lane, tw);
    extract_pair(Z, urow, vrow, d, lane, active, scale);
}

// a b + c with one rounding, and a b alone rounded (never fused into a
// neighbouring add): the epilogue's arithmetic fixed operation by operation,
// so that every kernel that inlines it -- the single-run stage kernels and
// the batch -- rounds the same way whatever the compiler would contract.
__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double mul_t(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_t(float a, float b) { return __fmul_rn(a, b); }

// One mode (kx, jc) of the K3 epilogue: dW from the two transformed products
// nx, ny, then the stage update below, Truncate (|k|^2 > K^2 -> 0) and the
// non-finite check.  Returns true for a non-finite result.  kxl is the
// mode's column in the arrays given (kx = kxl + d.kx0).
template <typename T>
__device__ __forceinline__ bool stage_point(const Dims& d, typename Vec<T>::t nx, typename Vec<T>::t ny, int kxl,
                                            int jc, typename Vec<T>::t* S0, typename Vec<T>::t* S1,
                                            typename Vec<T>::t* Sdw, const typename Vec<T>::t* __restrict__ src,
                                            int stage, double dt, const Phys& ph, const T* fac = nullptr) {
    using VT = typename Vec<T>::t;
    const T tdt = (T)dt;
    const T c34 = (T)0.75, c14 = (T)0.25, c13 = (T)(1.0 / 3.0), c23 = (T)(2.0 / 3.0);
    // 2 dt / 3 as dt times the rounded 2/3, like the 1/3 above: a division
    // here would be one FP64 division per mode in the one-mode-per-thread
    // stage kernel (its stage-3 launch took 107 instead of 76 us at 2048^2)
    const T dt4 = (T)(0.25 * dt), dt23 = (T)(dt * (2.0 / 3.0));
    const T tnu = (T)ph.nu, talpha = (T)ph.alpha;
    const int kx = kxl + d.kx0;
    const int ky = ky_of_jc(d, jc);
    const size_t off = (size_t)kxl * d.ldS + jc;
    const int kk = kx * kx + ky * ky;
    bool bad = false;
    VT out;
    if (kk > d.K * d.K) {
        out = mk<VT>((T)0, (T)0);
    } else {
        const VT w0 = S0[off];
        const VT win = (stage <= 1) ? w0 : S1[off];
        const T fkx = (T)kx, fky = (T)ky;
        // fac (Basdevant): kx^2 - ky^2, kx ky, nu k^2 of this mode from tables
        // (the same values, exact or the same product)
        const T visc = fac ? fac[2] : tnu * (T)kk;
        T dwx, dwy;
        if (ph.form == S2D_NL_BASDEVANT) {
            // dW = (kx^2-ky^2) F[uv] + kx ky F[v^2-u^2] - nu k^2 w
            const T c1 = fac ? fac[0] : (T)(kx * kx - ky * ky), c2 = fac ? fac[1] : (T)(kx * ky);
            dwx = fma_t(c1, nx.x, fma_t(c2, ny.x, -mul_t(visc, win.x)));
            dwy = fma_t(c1, nx.y, fma_t(c2, ny.y, -mul_t(visc, win.y)));
        } else {
            // dW = -i kx F[uw] - i ky F[vw] - nu k^2 w  (src/Spectral.F90:464-479)
            dwx = fma_t(fkx, nx.y, fma_t(fky, ny.y, -mul_t(visc, win.x)));
            dwy = fma_t(-fkx, nx.x, fma_t(-fky, ny.x, -mul_t(visc, win.y)));
        }
        if (talpha != (T)0) {
            dwx = fma_t(-talpha, win.x, dwx);
            dwy = fma_t(-talpha, win.y, dwy);
        }
        if (ph.fk != 0 && kx == 0 && (ky == ph.fk || ky == -ph.fk)) {
            dwx += (T)ph.f_re;
            dwy += (ky > 0) ? (T)ph.f_im : (T)(-ph.f_im);
        }
        if (src) {
            const VT e = src[off];
            dwx += e.x;
            dwy += e.y;
        }
        if (stage == 0) {
            out = mk<VT>(dwx, dwy);
        } else if (stage == 1) {
            out = mk<VT>(fma_t(tdt, dwx, w0.x), fma_t(tdt, dwy, w0.y));
        } else if (stage == 2) {
            out = mk<VT>(fma_t(dt4, dwx, fma_t(c14, win.x, mul_t(c34, w0.x))),
                         fma_t(dt4, dwy, fma_t(c14, win.y, mul_t(c34, w0.y))));
        } else {
            out = mk<VT>(fma_t(dt23, dwx, fma_t(c23, win.x, mul_t(c13, w0.x))),
                         fma_t(dt23, dwy, fma_t(c23, win.y, mul_t(c13, w0.y))));
        }
        bad = bits_nonfinite(out.x) | bits_nonfinite(out.y);
    }
    if (stage == 0) Sdw[off] = out;
    else if (stage == 3) S0[off] = out;
    else S1[off] = out;
    return bad;
}

// Columns kx0 .. kx0+G-1 of the half-spectral rows of one or two fields
// (X, then Y) into bufs[(field * G + gg) * M + y], zero past gtot; n =
// G * M elements of X alone, 2 G M of both.  One element per row is a
// strided gather, so each thread keeps kU loads in flight before it
// stores them.
template <typename T>
__device__ __forceinline__ void gather_columns(const Dims& d, const typename Vec<T>::t* __restrict__ X,
                                               const typename Vec<T>::t* __restrict__ Y, int G, int gtot, int kx0,
                                               int n, typename Vec<T>::t* bufs) {
    using VT = typename Vec<T>::t;
    constexpr int kU = sizeof(T) == 8 ? 4 : 8;
    const DivBy byG(G), byM(d.M);
    for (int base = threadIdx.x; base < n; base += kU * blockDim.x) {
        VT v[kU];
        int dst[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const int idx = base + u * blockDim.x;
            v[u] = mk<VT>((T)0, (T)0);
            dst[u] = -1;
            if (idx < n) {
                int gg = 0, y, fld;
                if (G == 1) {
                    fld = idx >= d.M;
                    y = idx - fld * d.M;
                } else {
                    const int rest = byG(idx);
                    gg = idx - rest * G;
                    fld = byM(rest);
                    y = rest - fld * d.M;
                }
                dst[u] = (fld * G + gg) * d.M + y;
                if (gg < gtot) v[u] = __ldcg(&(fld ? Y : X)[(size_t)y * d.ldI + kx0 + gg]);
            }
        }
#pragma unroll
        for (int u = 0; u < kU; ++u)
            if (dst[u] >= 0) bufs[dst[u]] = v[u];
    }
}

// K3 split in two for a third CTA per SM (the single-run FP64 path): the
// forward y-FFT of one field's columns, its retained rows stored in the
// compact layout (Out[kx][jc])...
template <typename T>
__device__ __forceinline__ void yfwd_col_body(const Dims& d, const typename Vec<T>::t* __restrict__ Iu,
                                              const typename Vec<T>::t* __restrict__ Iv, typename Vec<T>::t* OutU,
                                              typename Vec<T>::t* OutV, const typename Vec<T>::t* __restrict__ tw,
                                              int G, int blk, typename Vec<T>::t* bufs) {
    using VT = typename Vec<T>::t;
    const int g = threadIdx.x / d.Tg;
    const int lane = threadIdx.x - g * d.Tg;
    const int ncg = (d.KX + G - 1) / G;
    const int f = blk / ncg;
    const int kx0 = (blk - f * ncg) * G;
    const int gtot = min(G, d.KX - kx0);
    const VT* I = f ? Iv : Iu;
    VT* Out = f ? OutV : OutU;
    gather_columns<T>(d, I, I, G, gtot, kx0, G * d.M, bufs);
    fft_run<false>(bufs + (size_t)g * d.M, d, lane, tw);
    __syncthreads();
    const DivBy byKY(d.KY);
    for (int idx = threadIdx.x; idx < gtot * d.KY; idx += blockDim.x) {
        const int gg = gtot == 1 ? 0 : byKY(idx);
        const int jc = idx - gg * d.KY;
        const int n = jc <= d.K ? jc : ky_of_jc(d, jc) + d.M;
        Out[(size_t)(kx0 + gg) * d.ldS + jc] = bufs[(size_t)gg * d.M + n];
    }
}

// ... and the epilogue of every mode from the two compact arrays: column kx
// = blockIdx.y, rows jc = blockIdx.x * blockDim.x + threadIdx.x.
template <typename T>
__device__ __forceinline__ bool stage_body(const Dims& d, const typename Vec<T>::t* __restrict__ Fu,
                                           const typename Vec<T>::t* __restrict__ Fv, typename Vec<T>::t* S0,
                                           typename Vec<T>::t* S1, typename Vec<T>::t* Sdw,
                                           const typename Vec<T>::t* __restrict__ src, int stage, double dt,
                                           const Phys& ph, const double2* __restrict__ cc,
                                           const double* __restrict__ vk) {
    const int kx = blockIdx.y;
    const int jc = blockIdx.x * blockDim.x + threadIdx.x;
    if (kx >= d.KX || jc >= d.KY) return false;
    const size_t off = (size_t)kx * d.ldS + jc;
    if (cc) {   // the mode's factors from tables: no integer-to-FP64 conversions or nu k^2 product
        const double2 c = __ldg(&cc[off]);
        const T fac[3] = {(T)c.x, (T)c.y, (T)__ldg(&vk[off])};
        return stage_point<T>(d, __ldcg(&Fu[off]), __ldcg(&Fv[off]), kx, jc, S0, S1, Sdw, src, stage, dt, ph, fac);
    }
    return stage_point<T>(d, __ldcg(&Fu[off]), __ldcg(&Fv[off]), kx, jc, S0, S1, Sdw, src, stage, dt, ph);
}

// ------------------------------------------------------------------------
// K3: forward y-pass of the two products + RK3 stage epilogue on columns
// [blk*G, blk*G+G): 2G transforms (G columns x two product fields: {u v,
// v^2 - u^2} in the Basdevant form, {u w, v w} in the conservative form),
// run blockDim/Tg at a time.
//   stage 1: S1 = S0 + dt dW                    (w_in = S0)
//   stage 2: S1 = 3/4 S0 + 1/4 S1 + dt/4 dW      (w_in = S1)
//   stage 3: S0 = S0/3 + 2/3 S1 + 2dt/3 dW       (w_in = S1)
//   stage 0: Sdw = dW of w_in = S0 (ComputeRHS alone)
// followed by Truncate (|k|^2 > K^2 -> 0).  Division by 3 is a multiply by
// the rounded reciprocal (a <= 1 ulp difference from
// src/TimeIntegration.F90:198-200).  src, when not null, is an additive
// spectral source in the compact layout (added to dW).
// ------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ bool yfwd_body(const Dims& d, const typename Vec<T>::t* __restrict__ Iu,
                                          const typename Vec<T>::t* __restrict__ Iv, typename Vec<T>::t* S0,
                                          typename Vec<T>::t* S1, typename Vec<T>::t* Sdw,
                                          const typename Vec<T>::t* __restrict__ src, int stage, double dt,
                                          const Phys& ph, const typename Vec<T>::t* __restrict__ tw, int G,
                                          int blk, typename Vec<T>::t* bufs) {
    using VT = typename Vec<T>::t;
    const int t = threadIdx.x / d.Tg;
    const int lane = threadIdx.x - t * d.Tg;
    const int kx0 = blk * G;
    const int gtot = min(G, d.KX - kx0);

    gather_columns<T>(d, Iu, Iv, G, gtot, kx0, 2 * G * d.M, bufs);
    const int nconc = blockDim.x / d.Tg;
    for (int t0 = 0; t0 < 2 * G; t0 += nconc) fft_run<false>(bufs + (size_t)(t0 + t) * d.M, d, lane, tw);
    __syncthreads();

    bool bad = false;
    const DivBy byKY(d.KY);
    for (int idx = threadIdx.x; idx < gtot * d.KY; idx += blockDim.x) {
        const int gg = gtot == 1 ? 0 : byKY(idx);
        const int jc = idx - gg * d.KY;
        const int ky = ky_of_jc(d, jc);
        const int n = jc <= d.K ? jc : ky + d.M;
        bad |= stage_point<T>(d, bufs[(size_t)gg * d.M + n], bufs[(size_t)(G + gg) * d.M + n], kx0 + gg, jc, S0, S1,
                              Sdw, src, stage, dt, ph);
    }
    return bad;
}

}  // namespace s2d
