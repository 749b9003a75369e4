// s2d_fft.cuh -- block-level mixed-radix Stockham FFT in shared memory.
//
// One transform of length M is owned by Tg = M/12 consecutive threads; a CTA
// runs several transforms of the same length side by side.  Each pass with
// radix R is the self-sorting Stockham step (Govindaraju et al., SC'08):
// butterfly j (0 <= j < M/R) reads x[j + r*M/R], multiplies by the twiddle
// w^(r*(j mod Ns)*M/(Ns*R)) with w = exp(-2 pi i/M), does a radix-R DFT and
// writes x[(j/Ns)*Ns*R + j mod Ns + r*Ns], Ns being the product of the
// earlier radices.  The pass is done in place: every thread first loads all
// 12 of its elements into registers, the CTA synchronises, then every thread
// writes its results.
//
// FP64 on GB300 has a small fraction of the FP32 issue rate, so the code is
// written to minimise FP64 instructions: twiddles come from a table (a load,
// not a sincos), twiddled radix-4/2 passes use the FMA form (TwEnt), and the
// radix-3 and radix-4 butterflies use only additions and FMAs.
//
// FP32 runs the same passes; with 64x the FP64 rate, its cost is the
// shared-memory traffic and the barriers of the in-place passes.
#pragma once

#include "s2d_internal.h"

namespace s2d {

template <typename T>
struct Vec;
template <>
struct Vec<double> {
    using t = double2;
};
template <>
struct Vec<float> {
    using t = float2;
};

template <typename VT, typename T>
__device__ __forceinline__ VT mk(T x, T y) {
    VT r;
    r.x = x;
    r.y = y;
    return r;
}

// a * w (forward) or a * conj(w) (inverse)
template <bool INV, typename VT>
__device__ __forceinline__ VT twmul(VT a, VT w) {
    VT r;
    if (!INV) {
        r.x = a.x * w.x - a.y * w.y;
        r.y = a.x * w.y + a.y * w.x;
    } else {
        r.x = a.x * w.x + a.y * w.y;
        r.y = a.y * w.x - a.x * w.y;
    }
    return r;
}

template <bool INV, typename VT>
__device__ __forceinline__ void bf2(VT* v) {
    VT a = v[0], b = v[1];
    v[0].x = a.x + b.x;
    v[0].y = a.y + b.y;
    v[1].x = a.x - b.x;
    v[1].y = a.y - b.y;
}

// Radix-3 DFT: y1 = a - (b+c)/2 -/+ i sin(2pi/3) (b-c) (forward/inverse).
template <bool INV, typename VT>
__device__ __forceinline__ void bf3(VT* v) {
    using T = decltype(v[0].x);
    const T s = (T)0.86602540378443864676;
    const T h = (T)0.5;
    VT a = v[0], b = v[1], c = v[2];
    T t1x = b.x + c.x, t1y = b.y + c.y;
    T t2x = b.x - c.x, t2y = b.y - c.y;
    T mx = a.x - h * t1x, my = a.y - h * t1y;
    v[0].x = a.x + t1x;
    v[0].y = a.y + t1y;
    if (!INV) {
        v[1].x = mx + s * t2y;
        v[1].y = my - s * t2x;
        v[2].x = mx - s * t2y;
        v[2].y = my + s * t2x;
    } else {
        v[1].x = mx - s * t2y;
        v[1].y = my + s * t2x;
        v[2].x = mx + s * t2y;
        v[2].y = my - s * t2x;
    }
}

template <bool INV, typename VT>
__device__ __forceinline__ void bf4(VT* v) {
    VT a = v[0], b = v[1], c = v[2], d = v[3];
    auto t0x = a.x + c.x, t0y = a.y + c.y;
    auto t1x = a.x - c.x, t1y = a.y - c.y;
    auto t2x = b.x + d.x, t2y = b.y + d.y;
    auto t3x = b.x - d.x, t3y = b.y - d.y;
    v[0].x = t0x + t2x;
    v[0].y = t0y + t2y;
    v[2].x = t0x - t2x;
    v[2].y = t0y - t2y;
    if (!INV) {  // y1 = t1 - i t3, y3 = t1 + i t3
        v[1].x = t1x + t3y;
        v[1].y = t1y - t3x;
        v[3].x = t1x - t3y;
        v[3].y = t1y + t3x;
    } else {
        v[1].x = t1x - t3y;
        v[1].y = t1y + t3x;
        v[3].x = t1x + t3y;
        v[3].y = t1y - t3x;
    }
}

template <int R, bool INV, typename VT>
__device__ __forceinline__ void butterfly(VT* v) {
    if constexpr (R == 2) bf2<INV>(v);
    else if constexpr (R == 3) bf3<INV>(v);
    else bf4<INV>(v);
}

// j mod Ns by a multiply-high: q = floor(j mg / 2^32) with mg = ceil(2^32 /
// Ns) (Dims::mg, set on the host) is floor(j / Ns) exactly while
// j (mg Ns - 2^32) < 2^32, i.e. for every j < 2^32 / Ns (here j < M <= 6144).
// No integer division on the device: on GB300 it competes with the FP64
// pipe (the FP64 step ran 3 % faster without one per butterfly).
struct ModNs {
    int Ns;
    unsigned mg;
    __device__ __forceinline__ ModNs(int ns, unsigned m) : Ns(ns), mg(m) {}
    __device__ __forceinline__ int operator()(int j) const {
        return Ns == 1 ? 0 : j - (int)__umulhi((unsigned)j, mg) * Ns;
    }
};

// floor(n / d) by the same multiply-high with m = ceil(2^32 / d), built once
// per thread (one division) and used per element: exact while
// n (m d - 2^32) < 2^32, which holds for the index splits of the column
// gathers and stores (n < 2^17, d < 2^14).  Small plans take G > 1
// transforms per CTA, and a division per element there was a third of the
// instructions of their latency-bound column kernels.
struct DivBy {
    int d;
    unsigned m;
    __device__ __forceinline__ explicit DivBy(int dd) : d(dd), m(dd > 1 ? 0xFFFFFFFFu / (unsigned)dd + 1u : 0u) {}
    __device__ __forceinline__ int operator()(int n) const { return d == 1 ? n : (int)__umulhi((unsigned)n, m); }
};

// One in-place Stockham pass of radix R over the transform in buf.
template <int R, bool INV, typename VT>
__device__ __forceinline__ void fft_pass(VT* buf, int M, int Ns, unsigned mg, int tstep, int lane, int Tg,
                                         const VT* __restrict__ tw) {
    constexpr int NB = kElemsPerThread / R;
    VT v[NB][R];
    const int stride = M / R;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = lane + b * Tg;
#pragma unroll
        for (int r = 0; r < R; ++r) v[b][r] = buf[j + r * stride];
    }
    __syncthreads();
    const ModNs mod(Ns, mg);
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = lane + b * Tg;
        const int k = mod(j);
        if (Ns > 1) {
            const int ts = k * tstep;
#pragma unroll
            for (int r = 1; r < R; ++r) v[b][r] = twmul<INV>(v[b][r], __ldg(&tw[r * ts]));
        }
        butterfly<R, INV>(v[b]);
        const int base = (j - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) buf[base + r * Ns] = v[b][r];
    }
    __syncthreads();
}

// Radix-3 DFT of (a, 0, c): 8 instead of 12 floating-point instructions.
template <bool INV, typename VT>
__device__ __forceinline__ void bf3_bzero(VT* v) {
    using T = decltype(v[0].x);
    const T s = (T)0.86602540378443864676;
    const T h = (T)0.5;
    const VT a = v[0], c = v[2];
    const T mx = a.x - h * c.x, my = a.y - h * c.y;
    v[0].x = a.x + c.x;
    v[0].y = a.y + c.y;
    if (!INV) {  // y1 = m + i s c, y2 = m - i s c
        v[1].x = mx - s * c.y;
        v[1].y = my + s * c.x;
        v[2].x = mx + s * c.y;
        v[2].y = my - s * c.x;
    } else {
        v[1].x = mx + s * c.y;
        v[1].y = my - s * c.x;
        v[2].x = mx - s * c.y;
        v[2].y = my + s * c.x;
    }
}

// First pass of an inverse transform whose input is zero in the middle third
// except at index M/3 -- every inverse transform here: the spectra are
// truncated to |k| <= K = M/3, so index n is non-zero only for n <= K or
// n >= M - K.  Butterfly j reads (x[j], x[j + M/3], x[j + 2M/3]); its middle
// input is zero for j > 0.
template <bool INV, typename VT>
__device__ __forceinline__ void fft_pass3_midzero(VT* buf, int M, int lane, int Tg) {
    constexpr int NB = kElemsPerThread / 3;
    VT v[NB][3];
    const int stride = M / 3;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = lane + b * Tg;
        v[b][0] = buf[j];
        v[b][1] = buf[j + stride];
        v[b][2] = buf[j + 2 * stride];
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = lane + b * Tg;
        if (j == 0) bf3<INV>(v[b]);
        else bf3_bzero<INV>(v[b]);
        buf[j * 3] = v[b][0];
        buf[j * 3 + 1] = v[b][1];
        buf[j * 3 + 2] = v[b][2];
    }
    __syncthreads();
}

__device__ __forceinline__ double ffma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float ffma(float a, float b, float c) { return fmaf(a, b, c); }

__device__ __forceinline__ double neg_if(double v, int cond) {
    return __longlong_as_double(__double_as_longlong(v) ^ ((long long)(cond != 0) << 63));
}
__device__ __forceinline__ float neg_if(float v, int cond) {
    return __int_as_float(__float_as_int(v) ^ ((cond != 0) << 31));
}

// x * i^q by register moves and sign flips only (integer operations).
template <typename VT>
__device__ __forceinline__ VT rot_iq(VT x, int q) {
    VT r;
    r.x = (q & 1) ? x.y : x.x;
    r.y = (q & 1) ? x.x : x.y;
    r.x = neg_if(r.x, (q + 1) & 2);
    r.y = neg_if(r.y, q & 2);
    return r;
}

// (x * i^q) * (1 + i t): two FMAs; the inverse uses conj(w) = i^-q c (1 - i t).
template <bool INV, typename VT, typename T>
__device__ __forceinline__ VT tw_fma(VT x, T t, int q) {
    const VT y = rot_iq(x, INV ? ((4 - q) & 3) : q);
    const T tt = INV ? -t : t;
    VT r;
    r.x = ffma(-tt, y.y, y.x);
    r.y = ffma(tt, y.x, y.y);
    return r;
}

// Radix-4 Stockham pass with FMA-form twiddles (Ns > 1): 22 FP64
// instructions per butterfly instead of 12 (3 complex products) + 16.
template <bool INV, typename VT, typename T>
__device__ __forceinline__ void fft_pass4_fma(VT* buf, int M, int Ns, unsigned mg, int lane, int Tg,
                                              const TwEnt<T>* __restrict__ tab) {
    constexpr int NB = kElemsPerThread / 4;
    VT v[NB][4];
    const int stride = M / 4;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = lane + b * Tg;
#pragma unroll
        for (int r = 0; r < 4; ++r) v[b][r] = buf[j + r * stride];
    }
    __syncthreads();
    const ModNs mod(Ns, mg);
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = lane + b * Tg;
        const int k = mod(j);
        const TwEnt<T> e = tab[k];
        const VT a = v[b][0];
        const VT B = tw_fma<INV>(v[b][1], e.t1, e.q & 3);
        const VT Cc = tw_fma<INV>(v[b][2], e.t2, (e.q >> 2) & 3);
        const VT D = tw_fma<INV>(v[b][3], e.t3, (e.q >> 4) & 3);
        // t0,1 = a +- c2 C ; E,F = B +- (c3/c1) D ; y = t +- c1 E, t -+ i c1 F
        const T t0x = ffma(e.c2, Cc.x, a.x), t0y = ffma(e.c2, Cc.y, a.y);
        const T t1x = ffma(-e.c2, Cc.x, a.x), t1y = ffma(-e.c2, Cc.y, a.y);
        const T Ex = ffma(e.r31, D.x, B.x), Ey = ffma(e.r31, D.y, B.y);
        const T Fx = ffma(-e.r31, D.x, B.x), Fy = ffma(-e.r31, D.y, B.y);
        VT y0, y1, y2, y3;
        y0.x = ffma(e.c1, Ex, t0x);
        y0.y = ffma(e.c1, Ey, t0y);
        y2.x = ffma(-e.c1, Ex, t0x);
        y2.y = ffma(-e.c1, Ey, t0y);
        if (!INV) {  // y1 = t1 - i c1 F, y3 = t1 + i c1 F
            y1.x = ffma(e.c1, Fy, t1x);
            y1.y = ffma(-e.c1, Fx, t1y);
            y3.x = ffma(-e.c1, Fy, t1x);
            y3.y = ffma(e.c1, Fx, t1y);
        } else {
            y1.x = ffma(-e.c1, Fy, t1x);
            y1.y = ffma(e.c1, Fx, t1y);
            y3.x = ffma(e.c1, Fy, t1x);
            y3.y = ffma(-e.c1, Fx, t1y);
        }
        const int base = (j - k) * 4 + k;
        buf[base] = y0;
        buf[base + Ns] = y1;
        buf[base + 2 * Ns] = y2;
        buf[base + 3 * Ns] = y3;
    }
    __syncthreads();
}

// Radix-2 Stockham pass with an FMA-form twiddle (Ns > 1): y = a +- c1 B.
template <bool INV, typename VT, typename T>
__device__ __forceinline__ void fft_pass2_fma(VT* buf, int M, int Ns, unsigned mg, int lane, int Tg,
                                              const TwEnt<T>* __restrict__ tab) {
    constexpr int NB = kElemsPerThread / 2;
    VT v[NB][2];
    const int stride = M / 2;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = lane + b * Tg;
        v[b][0] = buf[j];
        v[b][1] = buf[j + stride];
    }
    __syncthreads();
    const ModNs mod(Ns, mg);
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = lane + b * Tg;
        const int k = mod(j);
        const T t1 = tab[k].t1, c1 = tab[k].c1;
        const int q = tab[k].q;
        const VT a = v[b][0];
        const VT B = tw_fma<INV>(v[b][1], t1, q & 3);
        const int base = (j - k) * 2 + k;
        VT y0, y1;
        y0.x = ffma(c1, B.x, a.x);
        y0.y = ffma(c1, B.y, a.y);
        y1.x = ffma(-c1, B.x, a.x);
        y1.y = ffma(-c1, B.y, a.y);
        buf[base] = y0;
        buf[base + Ns] = y1;
    }
    __syncthreads();
}

// Full transform: unnormalised, sign -1 (forward) or +1 (INV).  Every thread
// of the CTA must call it (it synchronises the CTA); starts with a barrier so
// that callers may fill buf just before.  tw points at the complex table
// (M entries) followed, d.tab_bytes later, by the TwEnt table.  Inverse
// transforms of truncated spectra (input zero for K < n < M - K, K = M/3: the
// inverse transforms of this library) take the pruned first radix-3 pass.
template <bool INV, typename VT>
__device__ __forceinline__ void fft_run(VT* buf, const Dims& d, int lane, const VT* __restrict__ tw) {
    using T = decltype(buf[0].x);
    const TwEnt<T>* tab = reinterpret_cast<const TwEnt<T>*>(reinterpret_cast<const char*>(tw) + d.tab_bytes);
    __syncthreads();
    int Ns = 1;
    for (int p = 0; p < d.npass; ++p) {
        const int R = d.radix[p];
        const int off = d.twoff[p];
        const unsigned mg = d.mg[p];
        if (INV && p == 0 && R == 3 && 3 * d.K == d.M) {
            fft_pass3_midzero<INV>(buf, d.M, lane, d.Tg);
        } else if (R == 4) {
            if (off >= 0) fft_pass4_fma<INV>(buf, d.M, Ns, mg, lane, d.Tg, tab + off);
            else fft_pass<4, INV>(buf, d.M, Ns, mg, d.tstep[p], lane, d.Tg, tw);
        } else if (R == 2) {
            if (off >= 0) fft_pass2_fma<INV>(buf, d.M, Ns, mg, lane, d.Tg, tab + off);
            else fft_pass<2, INV>(buf, d.M, Ns, mg, d.tstep[p], lane, d.Tg, tw);
        } else {
            fft_pass<3, INV>(buf, d.M, Ns, mg, d.tstep[p], lane, d.Tg, tw);
        }
        Ns *= R;
    }
}

}  // namespace s2d
