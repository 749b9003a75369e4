// s2d_kernels.cu -- sm_103a kernels of the Spectral2D time step.
//
// One right-hand side (src/Spectral.F90:396-482) is three kernels:
//
//   K1 yinv      compact omega columns -> psi, u, v derived on the fly
//                (ComputePsi :508-560, ComputeVelocity :576-610) -> inverse
//                y-FFT of each kx column (the y half of TransformC2R :772-781,
//                pruned to the N/2+1 non-zero columns) -> half-spectral rows.
//   K2 xpass     per physical row (Basdevant form, the default): one inverse
//                x-FFT of u + i v, the products u v and v^2 - u^2, one
//                forward x-FFT and the real/imaginary split (the x halves of
//                TransformC2R / TransformR2C :749-781, normalisation folded
//                in).  The reference's conservative form (k_xpass_rhs) works
//                on row pairs: inverse FFTs of (u, v) and omega, the products
//                u w and v w (:442-447), forward FFTs.  Physical fields never
//                touch HBM.
//   K3 yfwd_rk3  forward y-FFT of each kx column of the two products, then
//                Truncate (:457-458), the derivatives -- (kx^2 - ky^2) and
//                kx ky (Basdevant) or i kx / i ky (:464-465) -- the viscous
//                term (:479), drag, forcing and an optional source, and the
//                TVD-RK3 stage combination with ComputePsi and Truncate
//                (src/TimeIntegration.F90:156-209) in one epilogue.
//
// omega is not round-tripped through physical space (the reference does at
// :435/:453); that changes omega by round-off only.
#include "s2d_step.cuh"

#include <cuda_runtime.h>

namespace s2d {

// ------------------------------------------------------------------------
// K1, K2, K3 of one simulation: one tile per CTA (bodies in s2d_step.cuh).
// K1, K2 and the split K3 come in register budgets B, chosen from the CTA
// size by budget<T>():
//   B = 1: CTAs of at most 256 threads, FP64 three per SM (80 registers: a
//          third CTA fills the barrier phases of the other two), FP32 four
//          (64 registers);
//   B = 2: FP32 CTAs of at most 512 threads (M = 6144), two per SM (64
//          registers);
//   B = 0: one CTA of up to 512 threads per SM.
// (Wider FP32 column tiles -- 2 or 4 columns per CTA of 512 or 1024 threads,
// so that the half-spectral rows are written and gathered a sector at a
// time -- measured slower at 2048^2: 0.81 / 0.82 against 0.774 ms per step.)
// ------------------------------------------------------------------------
template <int B>
constexpr int kMaxThreads = B == 1 ? 256 : 512;
template <typename T, int B>
constexpr int kMinBlocks = B == 1 ? (sizeof(T) == 8 ? 3 : 4) : (B == 2 ? 2 : 1);
template <typename T>
int budget(int threads) {
    return threads <= 256 ? 1 : (sizeof(T) == 4 ? 2 : 0);
}

template <typename T, int B>
__global__ void __launch_bounds__(kMaxThreads<B>, (kMinBlocks<T, B>)) k_yinv(Dims d, const typename Vec<T>::t* __restrict__ S,
                                               const double* __restrict__ rk2, FieldSet fs,
                                               const typename Vec<T>::t* __restrict__ tw, int G) {
    using VT = typename Vec<T>::t;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    pdl_enter();
    yinv_body<T>(d, S, rk2, fs, tw, G, blockIdx.x, reinterpret_cast<VT*>(smem_raw));
}

template <typename T, int B>
__global__ void __launch_bounds__(kMaxThreads<B>, (kMinBlocks<T, B>)) k_xpass_bas(Dims d, typename Vec<T>::t* Iu, typename Vec<T>::t* Iv,
                                                    const typename Vec<T>::t* __restrict__ tw, int G,
                                                    T scale) {
    using VT = typename Vec<T>::t;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    pdl_enter();
    xpass_bas_body<T>(d, Iu, Iv, tw, G, scale, blockIdx.x, reinterpret_cast<VT*>(smem_raw));
}

// The FP32 x-pass of M = 3072 rows (s2d_xpass32.cuh): one row per 256-thread
// CTA, three CTAs per SM (the radix-16 passes hold 16 complex values per
// thread; inlined into k_xpass_bas at its four-per-SM budget of 64 registers
// they spilled).
__global__ void __launch_bounds__(256, 4) k_xpass32(Dims d, float2* Iu, float2* Iv, const float2* __restrict__ tw) {
    __shared__ float2 sb[kX32Buf];
    pdl_enter();
    xpass32_m3072_row(d, Iu, Iv, tw, blockIdx.x, (int)blockIdx.x < d.rows, threadIdx.x, sb);
}

template <typename T, int B>
__global__ void __launch_bounds__(kMaxThreads<B>, (kMinBlocks<T, B>)) k_yfwd_rk3(Dims d, const typename Vec<T>::t* __restrict__ Iu,
                                                   const typename Vec<T>::t* __restrict__ Iv,
                                                   typename Vec<T>::t* S0, typename Vec<T>::t* S1,
                                                   typename Vec<T>::t* Sdw,
                                                   const typename Vec<T>::t* __restrict__ src, int stage,
                                                   double dt, Phys ph, const typename Vec<T>::t* __restrict__ tw,
                                                   int G, unsigned int* flags) {
    using VT = typename Vec<T>::t;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    pdl_enter();
    const bool bad = yfwd_body<T>(d, Iu, Iv, S0, S1, Sdw, src, stage, dt, ph, tw, G, blockIdx.x,
                                  reinterpret_cast<VT*>(smem_raw));
    if (bad && flags) atomicOr(flags, 1u);   // flags may be null: no non-finite report
}

// K3 split in two (FP64 single runs): forward y-FFT of one field's columns
// into a compact array, then the epilogue of every mode.
template <typename T, int B>
__global__ void __launch_bounds__(kMaxThreads<B>, (kMinBlocks<T, B>))
    k_yfwd_col(Dims d, const typename Vec<T>::t* __restrict__ Iu, const typename Vec<T>::t* __restrict__ Iv,
               typename Vec<T>::t* Fu, typename Vec<T>::t* Fv, const typename Vec<T>::t* __restrict__ tw, int G) {
    using VT = typename Vec<T>::t;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    pdl_enter();
    yfwd_col_body<T>(d, Iu, Iv, Fu, Fv, tw, G, blockIdx.x, reinterpret_cast<VT*>(smem_raw));
}

template <typename T>
__global__ void __launch_bounds__(256) k_stage(Dims d, const typename Vec<T>::t* __restrict__ Fu,
                                               const typename Vec<T>::t* __restrict__ Fv, typename Vec<T>::t* S0,
                                               typename Vec<T>::t* S1, typename Vec<T>::t* Sdw,
                                               const typename Vec<T>::t* __restrict__ src, int stage, double dt,
                                               Phys ph, unsigned int* flags, const double2* __restrict__ cc,
                                               const double* __restrict__ vk) {
    pdl_enter();
    if (stage_body<T>(d, Fu, Fv, S0, S1, Sdw, src, stage, dt, ph, cc, vk)) atomicOr(flags, 1u);
}

// ------------------------------------------------------------------------
// K2 in the conservative form (the reference's): row pairs (y1, y2) =
// (2p, 2p+1).  Per group two buffers: W holds omega of both rows (w1 = Re,
// w2 = Im after the inverse FFT), Z holds u + i v of one row, then
// u*w + i v*w, then its spectrum.  On exit rows y of Iu / Iv hold the
// normalised half spectra of u*w / v*w.
// ------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(512) k_xpass_rhs(Dims d, typename Vec<T>::t* Iu, typename Vec<T>::t* Iv,
                                                    const typename Vec<T>::t* __restrict__ Iw,
                                                    const typename Vec<T>::t* __restrict__ tw, int G,
                                                    T scale) {
    using VT = typename Vec<T>::t;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    pdl_enter();
    VT* bufs = reinterpret_cast<VT*>(smem_raw);
    const int g = threadIdx.x / d.Tg;
    const int lane = threadIdx.x - g * d.Tg;
    const int p = blockIdx.x * G + g;
    const bool active = p < d.M / 2;
    const int y1 = active ? 2 * p : 0;
    const int y2 = y1 + 1;
    VT* W = bufs + (size_t)(2 * g) * d.M;
    VT* Z = W + d.M;

    build_pair(W, Iw + (size_t)y1 * d.ldI, Iw + (size_t)y2 * d.ldI, d, lane, active);
    fft_run<true>(W, d, lane, tw);

#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
        const int yy = h ? y2 : y1;
        VT* urow = Iu + (size_t)yy * d.ldI;
        VT* vrow = Iv + (size_t)yy * d.ldI;
        build_pair(Z, urow, vrow, d, lane, active);
        fft_run<true>(Z, d, lane, tw);
        for (int n = lane; n < d.M; n += d.Tg) {
            const VT z = Z[n];
            const T s = h ? W[n].y : W[n].x;
            Z[n] = mk<VT>(z.x * s, z.y * s);
        }
        fft_run<false>(Z, d, lane, tw);
        extract_pair(Z, urow, vrow, d, lane, active, scale);
        __syncthreads();
    }
}

// ------------------------------------------------------------------------
// Layout conversion between the reference's (cISize, nyG) complex128 array
// and the compact state.
// ------------------------------------------------------------------------
template <typename T>
__global__ void k_ref_to_compact(Dims d, const double2* __restrict__ ref, int C, typename Vec<T>::t* S) {
    using VT = typename Vec<T>::t;
    const int total = d.KX * d.KY;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        const int kx = idx / d.KY;
        const int jc = idx - kx * d.KY;
        const int ky = ky_of_jc(d, jc);
        const int n = ky >= 0 ? ky : ky + d.M;
        VT v = mk<VT>((T)0, (T)0);
        if (kx * kx + ky * ky <= d.K * d.K) {
            const double2 r = ref[(size_t)n * C + kx];
            v = mk<VT>((T)r.x, (T)r.y);
        }
        S[(size_t)kx * d.ldS + jc] = v;
    }
}

// psi = w / (kx^2 + ky^2), psi(0,0) = 0 (src/Spectral.F90:508-560), written
// with the state into full reference arrays (zeros outside the rectangle).
template <typename T>
__global__ void k_compact_to_ref(Dims d, const typename Vec<T>::t* __restrict__ S, int C, double2* refW,
                                 double2* refPsi) {
    const long total = (long)d.M * C;
    for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
        const int n = (int)(idx / C);
        const int kx = (int)(idx - (long)n * C);
        const int ky = n <= d.M / 2 ? n : n - d.M;
        double2 w = make_double2(0.0, 0.0);
        if (kx <= d.K && ky >= -d.K && ky <= d.K) {
            const int jc = ky >= 0 ? ky : ky + d.KY;
            const auto v = S[(size_t)kx * d.ldS + jc];
            w = make_double2((double)v.x, (double)v.y);
        }
        if (refW) refW[idx] = w;
        if (refPsi) {
            const double k2 = (double)kx * kx + (double)ky * ky;
            refPsi[idx] = (k2 == 0.0) ? make_double2(0.0, 0.0) : make_double2(w.x / k2, w.y / k2);
        }
    }
}

// ------------------------------------------------------------------------
// Host-array I/O of the retained rectangle (kx <= K, |ky| <= K; row n = ky
// mod M, pitch C) through 32 x 32 tiles in shared memory, so that both the
// compact columns and the reference rows are read and written in 512-byte
// runs.  ref may be the caller's host array itself (page-locked, or pageable
// memory reached through the host page tables), where scattered 16-byte
// accesses would each cost a transaction on the host link.
// ------------------------------------------------------------------------
constexpr int kIoTile = 32;

template <typename T>
__global__ void __launch_bounds__(256) k_rect_to_compact(Dims d, const double2* __restrict__ ref, int C,
                                                         typename Vec<T>::t* __restrict__ S) {
    using VT = typename Vec<T>::t;
    __shared__ double2 tile[kIoTile][kIoTile + 1];
    const int kx0 = blockIdx.x * kIoTile, jc0 = blockIdx.y * kIoTile;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int i = ty; i < kIoTile; i += 8) {
        const int jc = jc0 + i, kx = kx0 + tx;
        double2 v = make_double2(0.0, 0.0);
        if (jc < d.KY && kx < d.KX) {
            const int ky = ky_of_jc(d, jc), kxt = kx + d.kx0;
            if (kxt * kxt + ky * ky <= d.K * d.K) v = ref[(size_t)(ky >= 0 ? ky : ky + d.M) * C + kx];
        }
        tile[i][tx] = v;
    }
    __syncthreads();
    for (int i = ty; i < kIoTile; i += 8) {
        const int kx = kx0 + i, jc = jc0 + tx;
        if (kx < d.KX && jc < d.KY) {
            const double2 v = tile[tx][i];
            S[(size_t)kx * d.ldS + jc] = mk<VT>((T)v.x, (T)v.y);
        }
    }
}

// omega and psi = omega / (kx^2 + ky^2), psi(0,0) = 0 (src/Spectral.F90:508-560)
// on the rectangle; either output may be null.
template <typename T>
__global__ void __launch_bounds__(256) k_compact_to_rect(Dims d, const typename Vec<T>::t* __restrict__ S, int C,
                                                         double2* refW, double2* refPsi) {
    __shared__ double2 tile[kIoTile][kIoTile + 1];
    const int kx0 = blockIdx.x * kIoTile, jc0 = blockIdx.y * kIoTile;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int i = ty; i < kIoTile; i += 8) {
        const int kx = kx0 + i, jc = jc0 + tx;
        double2 v = make_double2(0.0, 0.0);
        if (kx < d.KX && jc < d.KY) {
            const auto s = S[(size_t)kx * d.ldS + jc];
            v = make_double2((double)s.x, (double)s.y);
        }
        tile[i][tx] = v;
    }
    __syncthreads();
    for (int i = ty; i < kIoTile; i += 8) {
        const int jc = jc0 + i, kx = kx0 + tx;
        if (jc < d.KY && kx < d.KX) {
            const int ky = ky_of_jc(d, jc);
            const size_t o = (size_t)(ky >= 0 ? ky : ky + d.M) * C + kx;
            const double2 w = tile[tx][i];
            if (refW) refW[o] = w;
            if (refPsi) {
                const double kxt = (double)(kx + d.kx0);
                const double k2 = kxt * kxt + (double)ky * ky;
                refPsi[o] = (k2 == 0.0) ? make_double2(0.0, 0.0) : make_double2(w.x / k2, w.y / k2);
            }
        }
    }
}

// Zeros of the truncated part of a reference array (blockIdx.y selects a or
// b): columns kx > K of the rectangle's rows, then rows K+1..M-K-1 whole.
__global__ void __launch_bounds__(256) k_zero_truncated(Dims d, int C, double2* a, double2* b) {
    double2* p = blockIdx.y == 0 ? a : b;
    if (!p) return;
    const int w = C - d.KX;
    const long strip = (long)d.KY * w;
    const long total = strip + (long)(d.M - d.KY) * C;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        size_t o;
        if (i < strip) {
            const int r = (int)i / w, c = (int)i - ((int)i / w) * w;
            o = (size_t)(r <= d.K ? r : r - d.KY + d.M) * C + d.KX + c;
        } else {
            o = (size_t)(d.K + 1) * C + (size_t)(i - strip);
        }
        p[o] = make_double2(0.0, 0.0);
    }
}

cudaError_t launch_zero_truncated(const Dims& d, int C, double* a, double* b, int blocks, cudaStream_t st) {
    k_zero_truncated<<<dim3(blocks, 2), 256, 0, st>>>(d, C, (double2*)a, (double2*)b);
    return cudaGetLastError();
}

// ------------------------------------------------------------------------
// Diagnostics
// ------------------------------------------------------------------------
__device__ __forceinline__ int isqrt_floor(int c) {
    int r = (int)sqrtf((float)c);
    while (r > 0 && r * r > c) --r;
    while ((r + 1) * (r + 1) <= c) ++r;
    return r;
}

// One warp per spectrum bin b: modes with round(|k|) == b, i.e.
// b^2 - b + 1 <= kx^2 + ky^2 <= b^2 + b (the bins of BinarySearch with the
// edges of src/Analysis.F90:358-362).  Energy per mode |u|^2 + |v|^2 with
// u = i ky psi, v = -i kx psi and weight 1/2 on kx = 0 (:380-395).  Bins
// above K hold no retained mode and are written as zero.
template <typename T>
__global__ void k_spectrum(Dims d, const typename Vec<T>::t* __restrict__ S, double* Ek, int nbins) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int b = warp;
    if (b >= nbins) return;
    double sum = 0.0;
    if (b <= d.K) {
        const int lo = b == 0 ? 0 : b * b - b + 1;
        const int hi = min(b == 0 ? 0 : b * b + b, d.K * d.K);
        for (int kx = lane; kx <= min(b, d.K); kx += 32) {
            const int kx2 = kx * kx;
            const int c = hi - kx2;
            if (c < 0) continue;
            const int a = max(lo - kx2, 0);
            int kylo = isqrt_floor(a);
            if (kylo * kylo < a) ++kylo;
            const int kyhi = isqrt_floor(c);
            for (int aky = kylo; aky <= kyhi; ++aky) {
                for (int sgn = 0; sgn < (aky == 0 ? 1 : 2); ++sgn) {
                    const int ky = sgn ? -aky : aky;
                    const int jc = ky >= 0 ? ky : ky + d.KY;
                    const auto v = S[(size_t)kx * d.ldS + jc];
                    const double k2 = (double)kx2 + (double)ky * ky;
                    double px = 0.0, py = 0.0;
                    if (k2 != 0.0) {
                        px = (double)v.x / k2;
                        py = (double)v.y / k2;
                    }
                    const double ux = -(double)ky * py, uy = (double)ky * px;
                    const double vx = (double)kx * py, vy = -(double)kx * px;
                    const double e = ux * ux + uy * uy + vx * vx + vy * vy;
                    sum += (kx == 0) ? 0.5 * e : e;
                }
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) Ek[b] = sum;
}

// Partial sums of weight*|w|^2 per block (deterministic order).
template <typename T>
__global__ void k_enstrophy_partial(Dims d, const typename Vec<T>::t* __restrict__ S, double* part) {
    __shared__ double red[256];
    double s = 0.0;
    const int total = d.KX * d.KY;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        const int kx = idx / d.KY;
        const int jc = idx - kx * d.KY;
        const auto v = S[(size_t)kx * d.ldS + jc];
        const double e = (double)v.x * v.x + (double)v.y * v.y;
        s += (kx == 0) ? e : 2.0 * e;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// out[0] = max|w|, out[1] = min|w|, out[2] = max|psi|, out[3] = min|psi| as
// the bit patterns of non-negative doubles (ordered like unsigned integers).
template <typename T>
__global__ void k_minmax(Dims d, const typename Vec<T>::t* __restrict__ S, unsigned long long* out) {
    double mxw = 0.0, mnw = 1.0e308, mxp = 0.0, mnp = 1.0e308;
    const int total = d.KX * d.KY;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        const int kx = idx / d.KY;
        const int jc = idx - kx * d.KY;
        const int ky = ky_of_jc(d, jc);
        const auto v = S[(size_t)kx * d.ldS + jc];
        const double aw = hypot((double)v.x, (double)v.y);
        const double k2 = (double)kx * kx + (double)ky * ky;
        const double ap = (k2 == 0.0) ? 0.0 : hypot((double)v.x / k2, (double)v.y / k2);
        mxw = fmax(mxw, aw);
        mnw = fmin(mnw, aw);
        mxp = fmax(mxp, ap);
        mnp = fmin(mnp, ap);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mxw = fmax(mxw, __shfl_xor_sync(0xffffffffu, mxw, o));
        mnw = fmin(mnw, __shfl_xor_sync(0xffffffffu, mnw, o));
        mxp = fmax(mxp, __shfl_xor_sync(0xffffffffu, mxp, o));
        mnp = fmin(mnp, __shfl_xor_sync(0xffffffffu, mnp, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&out[0], (unsigned long long)__double_as_longlong(mxw));
        atomicMin(&out[1], (unsigned long long)__double_as_longlong(mnw));
        atomicMax(&out[2], (unsigned long long)__double_as_longlong(mxp));
        atomicMin(&out[3], (unsigned long long)__double_as_longlong(mnp));
    }
}

// Physical u, v of each row (one complex inverse FFT of u + i v), then
// max(|u|/dx + |v|/dy) with dx = dy = 2 pi / M.
template <typename T>
__global__ void __launch_bounds__(512) k_xinv_cfl(Dims d, const typename Vec<T>::t* __restrict__ Iu,
                                                   const typename Vec<T>::t* __restrict__ Iv,
                                                   const typename Vec<T>::t* __restrict__ tw, int G,
                                                   unsigned long long* maxbits) {
    using VT = typename Vec<T>::t;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    VT* bufs = reinterpret_cast<VT*>(smem_raw);
    __shared__ double red[32];
    const int g = threadIdx.x / d.Tg;
    const int lane = threadIdx.x - g * d.Tg;
    const int y = blockIdx.x * G + g;
    const bool active = y < d.M;
    VT* Z = bufs + (size_t)g * d.M;
    const int yy = active ? y : 0;
    build_pair(Z, Iu + (size_t)yy * d.ldI, Iv + (size_t)yy * d.ldI, d, lane, active);
    fft_run<true>(Z, d, lane, tw);
    const double inv_dx = (double)d.M / (2.0 * 3.14159265358979323846);
    double m = 0.0;
    if (active)
        for (int n = lane; n < d.M; n += d.Tg) {
            const VT z = Z[n];
            m = fmax(m, fabs((double)z.x) * inv_dx + fabs((double)z.y) * inv_dx);
        }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x + 31) / 32 ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (threadIdx.x == 0) atomicMax(maxbits, (unsigned long long)__double_as_longlong(v));
    }
}

// Skewness moments of two physical fields a (real part) and b (imaginary
// part) of one inverse FFT per row: out[row] = (sum a b^2, sum a^2, sum b^2)
// (src/Analysis.F90:157-163, :203-209), summed over rows later in order.
template <typename T>
__global__ void __launch_bounds__(512) k_xinv_moments(Dims d, const typename Vec<T>::t* __restrict__ Ia,
                                                      const typename Vec<T>::t* __restrict__ Ib,
                                                      const typename Vec<T>::t* __restrict__ tw, int G,
                                                      double* out) {
    using VT = typename Vec<T>::t;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    VT* bufs = reinterpret_cast<VT*>(smem_raw);
    const int g = threadIdx.x / d.Tg;
    const int lane = threadIdx.x - g * d.Tg;
    const int y = blockIdx.x * G + g;
    const bool active = y < d.M;
    VT* Z = bufs + (size_t)g * d.M;
    const int yy = active ? y : 0;
    build_pair(Z, Ia + (size_t)yy * d.ldI, Ib + (size_t)yy * d.ldI, d, lane, active);
    fft_run<true>(Z, d, lane, tw);
    // one row per group; the group's threads reduce in a fixed order
    double s1 = 0.0, s2 = 0.0, s3 = 0.0;
    for (int n = lane; n < d.M; n += d.Tg) {
        const double a = (double)Z[n].x, b = (double)Z[n].y;
        s1 += a * b * b;
        s2 += a * a;
        s3 += b * b;
    }
    __syncthreads();
    double* scratch = reinterpret_cast<double*>(bufs);   // reuse: 3 x blockDim doubles
    scratch[3 * threadIdx.x] = s1;
    scratch[3 * threadIdx.x + 1] = s2;
    scratch[3 * threadIdx.x + 2] = s3;
    __syncthreads();
    if (lane == 0 && active) {
        double t1 = 0.0, t2 = 0.0, t3 = 0.0;
        for (int i = 0; i < d.Tg; ++i) {
            const int k = g * d.Tg + i;
            t1 += scratch[3 * k];
            t2 += scratch[3 * k + 1];
            t3 += scratch[3 * k + 2];
        }
        out[3 * y] = t1;
        out[3 * y + 1] = t2;
        out[3 * y + 2] = t3;
    }
}

// Taylor-Green vorticity on the physical grid, 2 sin(x_i) sin(y_j) with the
// 1-based coordinates of src/SetIC.F90:88-96 (sx, sy precomputed on the host
// with the same FP64 sin as the reference).
template <typename T>
__global__ void k_fill_tg(Dims d, const double* __restrict__ sx, const double* __restrict__ sy, T* phys) {
    const long total = (long)d.M * d.M;
    for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
        const int j = (int)(idx / d.M);
        const int i = (int)(idx - (long)j * d.M);
        phys[idx] = (T)((2.0 * sx[i]) * sy[j]);
    }
}

// Forward x-transform of physical rows (pitch M) in pairs: one complex FFT
// of r1 + i r2, split into two normalised half spectra (kx in [0,K]).
template <typename T>
__global__ void __launch_bounds__(512) k_xfwd_phys(Dims d, const T* __restrict__ phys,
                                                    typename Vec<T>::t* Iout,
                                                    const typename Vec<T>::t* __restrict__ tw, int G,
                                                    T scale) {
    using VT = typename Vec<T>::t;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    VT* bufs = reinterpret_cast<VT*>(smem_raw);
    const int g = threadIdx.x / d.Tg;
    const int lane = threadIdx.x - g * d.Tg;
    const int p = blockIdx.x * G + g;
    const bool active = p < d.M / 2;
    const int y1 = active ? 2 * p : 0;
    VT* Z = bufs + (size_t)g * d.M;
    const T* r1 = phys + (size_t)y1 * d.M;
    const T* r2 = r1 + d.M;
    for (int n = lane; n < d.M; n += d.Tg) Z[n] = active ? mk<VT>(r1[n], r2[n]) : mk<VT>((T)0, (T)0);
    fft_run<false>(Z, d, lane, tw);
    extract_pair(Z, Iout + (size_t)y1 * d.ldI, Iout + (size_t)(y1 + 1) * d.ldI, d, lane, active, scale);
}

// Forward y-transform of half-spectral columns into the compact state, with
// Truncate.
template <typename T>
__global__ void __launch_bounds__(512) k_yfwd_store(Dims d, const typename Vec<T>::t* __restrict__ I,
                                                     typename Vec<T>::t* S,
                                                     const typename Vec<T>::t* __restrict__ tw, int G) {
    using VT = typename Vec<T>::t;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    VT* bufs = reinterpret_cast<VT*>(smem_raw);
    const int g = threadIdx.x / d.Tg;
    const int lane = threadIdx.x - g * d.Tg;
    const int kx0 = blockIdx.x * G;
    const int gtot = min(G, d.KX - kx0);
    for (int idx = threadIdx.x; idx < G * d.M; idx += blockDim.x) {
        const int gg = idx % G;
        const int y = idx / G;
        bufs[(size_t)gg * d.M + y] = gg < gtot ? I[(size_t)y * d.ldI + kx0 + gg] : mk<VT>((T)0, (T)0);
    }
    fft_run<false>(bufs + (size_t)g * d.M, d, lane, tw);
    __syncthreads();
    for (int idx = threadIdx.x; idx < gtot * d.KY; idx += blockDim.x) {
        const int gg = idx / d.KY;
        const int jc = idx - gg * d.KY;
        const int kx = kx0 + gg;
        const int ky = ky_of_jc(d, jc);
        const int n = jc <= d.K ? jc : ky + d.M;
        VT v = bufs[(size_t)gg * d.M + n];
        if (kx * kx + ky * ky > d.K * d.K) v = mk<VT>((T)0, (T)0);
        S[(size_t)kx * d.ldS + jc] = v;
    }
}

// 1/(kx^2+ky^2) per compact mode, 0 at the mean mode (FP64 in every variant).
__global__ void k_init_rk2(Dims d, double* rk2, double factor) {
    const int total = d.KX * d.KY;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        const int kx = idx / d.KY;
        const int jc = idx - kx * d.KY;
        const int ky = ky_of_jc(d, jc);
        const double k2 = (double)kx * kx + (double)ky * ky;
        rk2[(size_t)kx * d.ldS + jc] = (k2 == 0.0) ? 0.0 : factor / k2;
    }
}

__global__ void k_init_uv_factors(Dims d, const double* __restrict__ rk2, double* fu, double* fv) {
    const int total = d.KX * d.KY;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        const int kx = idx / d.KY;
        const int jc = idx - kx * d.KY;
        const int ky = ky_of_jc(d, jc);
        const size_t off = (size_t)kx * d.ldS + jc;
        // the expressions of apply_op's OP_U and OP_V
        fu[off] = (double)ky * rk2[off];
        fv[off] = -(double)kx * rk2[off];
    }
}

// The Basdevant stage factors of every retained mode: cc = (kx^2 - ky^2,
// kx ky), exact; vk = nu k^2, the product stage_point forms.
__global__ void k_init_stage_factors(Dims d, double nu, double2* cc, double* vk) {
    const int total = d.KX * d.KY;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        const int kx = idx / d.KY;
        const int jc = idx - kx * d.KY;
        const int ky = ky_of_jc(d, jc);
        const size_t off = (size_t)kx * d.ldS + jc;
        cc[off] = make_double2((double)(kx * kx - ky * ky), (double)(kx * ky));
        vk[off] = nu * (double)(kx * kx + ky * ky);
    }
}

// FP64 throughput probe: 8 independent FMA chains per thread.
__global__ void k_fp64_probe(double* sink, int iters) {
    double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-9, a2 = a0 + 2e-9, a3 = a0 + 3e-9;
    double a4 = a0 + 4e-9, a5 = a0 + 5e-9, a6 = a0 + 6e-9, a7 = a0 + 7e-9;
    const double b = 0.999999, c = 1e-7;
    for (int i = 0; i < iters; ++i) {
        a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
        a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
    }
    const double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == 12345.678) sink[threadIdx.x] = s;
}

// ------------------------------------------------------------------------
// Host-side launchers
// ------------------------------------------------------------------------
static int grid_for(long work, int threads) {
    long b = (work + threads - 1) / threads;
    if (b > 152L * 32) b = 152L * 32;
    if (b < 1) b = 1;
    return (int)b;
}

template <typename T>
cudaError_t Kern<T>::yinv(const Dims& d, const void* S, const double* rk2, const FieldSet& fs, const void* tw,
                          cudaStream_t st, const Launch& L) {
    using VT = typename Vec<T>::t;
    const int ncg = (d.KX + L.G - 1) / L.G;
    const int nb = ncg * fs.nf;
    const VT* s = (const VT*)S;
    const VT* t = (const VT*)tw;
    switch (budget<T>(L.threads)) {
        case 1: return launch_k(k_yinv<T, 1>, nb, L.threads, L.smem, st, L.pdl, d, s, rk2, fs, t, L.G);
        case 2:
            if constexpr (sizeof(T) == 4)
                return launch_k(k_yinv<T, 2>, nb, L.threads, L.smem, st, L.pdl, d, s, rk2, fs, t, L.G);
            return cudaErrorInvalidConfiguration;
        default: return launch_k(k_yinv<T, 0>, nb, L.threads, L.smem, st, L.pdl, d, s, rk2, fs, t, L.G);
    }
}

template <typename T>
cudaError_t Kern<T>::xpass_rhs(const Dims& d, void* Iu, void* Iv, const void* Iw, const void* tw,
                               cudaStream_t st, const Launch& L) {
    using VT = typename Vec<T>::t;
    const int pairs = d.M / 2;
    const T scale = (T)(0.5 / ((double)d.M * (double)d.M));
    return launch_k(k_xpass_rhs<T>, (pairs + L.G - 1) / L.G, L.threads, L.smem, st, L.pdl, d, (VT*)Iu, (VT*)Iv,
                    (const VT*)Iw, (const VT*)tw, L.G, scale);
}

template <typename T>
cudaError_t Kern<T>::xpass_bas(const Dims& d, void* Iu, void* Iv, const void* tw, cudaStream_t st,
                               const Launch& L, bool prescaled) {
    using VT = typename Vec<T>::t;
    const T scale = prescaled ? (T)1 : (T)(0.5 / ((double)d.M * (double)d.M));
    const int nb = (d.rows + L.G - 1) / L.G;
    VT* u = (VT*)Iu;
    VT* v = (VT*)Iv;
    const VT* t = (const VT*)tw;
    if constexpr (sizeof(T) == 4)
        if (d.M == kX32M && prescaled && !d.xgen)
            return launch_k(k_xpass32, d.rows, 256, 0, st, L.pdl, d, (float2*)Iu, (float2*)Iv, (const float2*)tw);
    switch (budget<T>(L.threads)) {
        case 1: return launch_k(k_xpass_bas<T, 1>, nb, L.threads, L.smem, st, L.pdl, d, u, v, t, L.G, scale);
        case 2:
            if constexpr (sizeof(T) == 4)
                return launch_k(k_xpass_bas<T, 2>, nb, L.threads, L.smem, st, L.pdl, d, u, v, t, L.G, scale);
            return cudaErrorInvalidConfiguration;
        default: return launch_k(k_xpass_bas<T, 0>, nb, L.threads, L.smem, st, L.pdl, d, u, v, t, L.G, scale);
    }
}

template <typename T>
cudaError_t Kern<T>::yfwd_rk3(const Dims& d, const void* Iu, const void* Iv, void* S0, void* S1, void* Sdw,
                              const void* src, int stage, double dt, const Phys& ph, const void* tw,
                              unsigned int* flags, cudaStream_t st, const Launch& L) {
    using VT = typename Vec<T>::t;
    const int nb = (d.KX + L.G - 1) / L.G;
    // FP32 CTAs of up to 256 threads at 64 registers, four per SM (at 80
    // registers, three per SM: 0.244 against 0.219 ms of K3 per 2048^2 step)
    if constexpr (sizeof(T) == 4)
        if (L.threads <= 256)
            return launch_k(k_yfwd_rk3<T, 1>, nb, L.threads, L.smem, st, L.pdl, d, (const VT*)Iu, (const VT*)Iv,
                            (VT*)S0, (VT*)S1, (VT*)Sdw, (const VT*)src, stage, dt, ph, (const VT*)tw, L.G, flags);
    return launch_k(k_yfwd_rk3<T, 0>, nb, L.threads, L.smem, st, L.pdl, d, (const VT*)Iu, (const VT*)Iv, (VT*)S0,
                    (VT*)S1, (VT*)Sdw, (const VT*)src, stage, dt, ph, (const VT*)tw, L.G, flags);
}

template <typename T>
cudaError_t Kern<T>::yfwd_col(const Dims& d, const void* Iu, const void* Iv, void* Fu, void* Fv, const void* tw,
                              cudaStream_t st, const Launch& L) {
    using VT = typename Vec<T>::t;
    const int ncg = (d.KX + L.G - 1) / L.G;
    const VT* u = (const VT*)Iu;
    const VT* v = (const VT*)Iv;
    const VT* t = (const VT*)tw;
    switch (budget<T>(L.threads)) {
        case 1:
            return launch_k(k_yfwd_col<T, 1>, 2 * ncg, L.threads, L.smem, st, L.pdl, d, u, v, (VT*)Fu, (VT*)Fv, t,
                            L.G);
        case 2:
            if constexpr (sizeof(T) == 4)
                return launch_k(k_yfwd_col<T, 2>, 2 * ncg, L.threads, L.smem, st, L.pdl, d, u, v, (VT*)Fu,
                                (VT*)Fv, t, L.G);
            return cudaErrorInvalidConfiguration;
        default:
            return launch_k(k_yfwd_col<T, 0>, 2 * ncg, L.threads, L.smem, st, L.pdl, d, u, v, (VT*)Fu, (VT*)Fv, t,
                            L.G);
    }
}

template <typename T>
cudaError_t Kern<T>::stage(const Dims& d, const void* Fu, const void* Fv, void* S0, void* S1, void* Sdw,
                           const void* src, int stage, double dt, const Phys& ph, unsigned int* flags,
                           cudaStream_t st, bool pdl, const double* cc, const double* vk) {
    using VT = typename Vec<T>::t;
    return launch_k(k_stage<T>, dim3((d.KY + 255) / 256, d.KX), dim3(256), 0, st, pdl, d, (const VT*)Fu,
                    (const VT*)Fv, (VT*)S0, (VT*)S1, (VT*)Sdw, (const VT*)src, stage, dt, ph, flags,
                    (const double2*)cc, vk);
}

template <typename T>
cudaError_t Kern<T>::ref_to_compact(const Dims& d, const double* ref, int C, void* S, cudaStream_t st) {
    using VT = typename Vec<T>::t;
    k_ref_to_compact<T><<<grid_for((long)d.KX * d.KY, 256), 256, 0, st>>>(d, (const double2*)ref, C, (VT*)S);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Kern<T>::rect_to_compact(const Dims& d, const double* ref, int C, void* S, cudaStream_t st) {
    using VT = typename Vec<T>::t;
    const dim3 grid((d.KX + kIoTile - 1) / kIoTile, (d.KY + kIoTile - 1) / kIoTile);
    k_rect_to_compact<T><<<grid, 256, 0, st>>>(d, (const double2*)ref, C, (VT*)S);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Kern<T>::compact_to_rect(const Dims& d, const void* S, int C, double* refW, double* refPsi,
                                     cudaStream_t st) {
    using VT = typename Vec<T>::t;
    const dim3 grid((d.KX + kIoTile - 1) / kIoTile, (d.KY + kIoTile - 1) / kIoTile);
    k_compact_to_rect<T><<<grid, 256, 0, st>>>(d, (const VT*)S, C, (double2*)refW, (double2*)refPsi);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Kern<T>::compact_to_ref(const Dims& d, const void* S, int C, double* refW, double* refPsi,
                                    cudaStream_t st) {
    using VT = typename Vec<T>::t;
    k_compact_to_ref<T><<<grid_for((long)d.M * C, 256), 256, 0, st>>>(d, (const VT*)S, C, (double2*)refW,
                                                                     (double2*)refPsi);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Kern<T>::spectrum(const Dims& d, const void* S, double* Ek, cudaStream_t st) {
    using VT = typename Vec<T>::t;
    // bins 0..K get a warp each; the caller zeroes the rest
    const int nb = d.K + 1;
    k_spectrum<T><<<(nb * 32 + 255) / 256, 256, 0, st>>>(d, (const VT*)S, Ek, nb);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Kern<T>::enstrophy_partial(const Dims& d, const void* S, double* part, int nblocks,
                                       cudaStream_t st) {
    using VT = typename Vec<T>::t;
    k_enstrophy_partial<T><<<nblocks, 256, 0, st>>>(d, (const VT*)S, part);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Kern<T>::minmax(const Dims& d, const void* S, unsigned long long* out4, cudaStream_t st) {
    using VT = typename Vec<T>::t;
    k_minmax<T><<<grid_for((long)d.KX * d.KY, 256), 256, 0, st>>>(d, (const VT*)S, out4);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Kern<T>::xinv_cfl(const Dims& d, const void* Iu, const void* Iv, const void* tw,
                              unsigned long long* maxbits, cudaStream_t st, const Launch& L) {
    using VT = typename Vec<T>::t;
    k_xinv_cfl<T><<<(d.M + L.G - 1) / L.G, L.threads, L.smem, st>>>(d, (const VT*)Iu, (const VT*)Iv,
                                                                     (const VT*)tw, L.G, maxbits);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Kern<T>::xinv_moments(const Dims& d, const void* Ia, const void* Ib, const void* tw, double* out,
                                  cudaStream_t st, const Launch& L) {
    using VT = typename Vec<T>::t;
    k_xinv_moments<T><<<(d.M + L.G - 1) / L.G, L.threads, L.smem, st>>>(d, (const VT*)Ia, (const VT*)Ib,
                                                                         (const VT*)tw, L.G, out);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Kern<T>::fill_tg(const Dims& d, const double* sx, const double* sy, void* phys, cudaStream_t st) {
    k_fill_tg<T><<<grid_for((long)d.M * d.M, 256), 256, 0, st>>>(d, sx, sy, (T*)phys);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Kern<T>::xfwd_phys(const Dims& d, const void* phys, void* Iout, const void* tw, cudaStream_t st,
                               const Launch& L) {
    using VT = typename Vec<T>::t;
    const T scale = (T)(0.5 / ((double)d.M * (double)d.M));
    k_xfwd_phys<T><<<(d.M / 2 + L.G - 1) / L.G, L.threads, L.smem, st>>>(d, (const T*)phys, (VT*)Iout,
                                                                         (const VT*)tw, L.G, scale);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Kern<T>::yfwd_store(const Dims& d, const void* I, void* S, const void* tw, cudaStream_t st,
                                const Launch& L) {
    using VT = typename Vec<T>::t;
    k_yfwd_store<T><<<(d.KX + L.G - 1) / L.G, L.threads, L.smem, st>>>(d, (const VT*)I, (VT*)S,
                                                                       (const VT*)tw, L.G);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Kern<T>::init_rk2(const Dims& d, double* rk2, cudaStream_t st, double factor) {
    k_init_rk2<<<grid_for((long)d.KX * d.KY, 256), 256, 0, st>>>(d, rk2, factor);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Kern<T>::init_uv_factors(const Dims& d, const double* rk2, double* fu, double* fv, cudaStream_t st) {
    k_init_uv_factors<<<grid_for((long)d.KX * d.KY, 256), 256, 0, st>>>(d, rk2, fu, fv);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Kern<T>::init_stage_factors(const Dims& d, double nu, double* cc, double* vk, cudaStream_t st) {
    k_init_stage_factors<<<grid_for((long)d.KX * d.KY, 256), 256, 0, st>>>(d, nu, (double2*)cc, vk);
    return cudaGetLastError();
}

template <typename T>
size_t Kern<T>::smem_limit_yinv() {
    return 0;
}

template struct Kern<double>;
template struct Kern<float>;

template <typename K>
static cudaError_t set_smem(K kernel, int bytes) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

cudaError_t configure_kernels(int max_smem_optin) {
    cudaError_t e = cudaSuccess;
#define S2D_SET(k)                                          \
    do {                                                    \
        cudaError_t e2 = set_smem(k, max_smem_optin);       \
        if (e2 != cudaSuccess && e == cudaSuccess) e = e2;  \
    } while (0)
    S2D_SET((k_yinv<double, 1>));
    S2D_SET((k_yinv<double, 0>));
    S2D_SET((k_yinv<float, 1>));
    S2D_SET((k_yinv<float, 2>));
    S2D_SET((k_yinv<float, 0>));
    S2D_SET(k_xpass_rhs<double>);
    S2D_SET(k_xpass_rhs<float>);
    S2D_SET((k_xpass_bas<double, 1>));
    S2D_SET((k_xpass_bas<double, 0>));
    S2D_SET((k_xpass_bas<float, 1>));
    S2D_SET((k_xpass_bas<float, 2>));
    S2D_SET((k_xpass_bas<float, 0>));
    S2D_SET((k_yfwd_col<double, 1>));
    S2D_SET((k_yfwd_col<double, 0>));
    S2D_SET((k_yfwd_col<float, 1>));
    S2D_SET((k_yfwd_col<float, 2>));
    S2D_SET((k_yfwd_col<float, 0>));
    S2D_SET((k_yfwd_rk3<double, 0>));
    S2D_SET((k_yfwd_rk3<float, 0>));
    S2D_SET((k_yfwd_rk3<float, 1>));
    S2D_SET(k_xinv_cfl<double>);
    S2D_SET(k_xinv_moments<double>);
    S2D_SET(k_xinv_moments<float>);
    S2D_SET(k_xinv_cfl<float>);
    S2D_SET(k_xfwd_phys<double>);
    S2D_SET(k_xfwd_phys<float>);
    S2D_SET(k_yfwd_store<double>);
    S2D_SET(k_yfwd_store<float>);
#undef S2D_SET
    return e;
}

cudaError_t launch_fp64_probe(double* sink, int blocks, int threads, int iters, cudaStream_t st) {
    k_fp64_probe<<<blocks, threads, 0, st>>>(sink, iters);
    return cudaGetLastError();
}

}  // namespace s2d
