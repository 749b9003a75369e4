// s2d_xpass32.cuh -- the FP32 x-pass of the Basdevant form for M = 3072
// (the 2048^2 grid) with register-resident radix-12 and radix-16 passes.
//
// The generic engine (s2d_fft.cuh) runs six radix-3/4 passes per transform,
// each a full round trip of the row through shared memory; in FP32 that
// traffic is the bound of the x-pass (L1/shared ~91 % busy).  Here each
// thread keeps 12 or 16 elements in registers and does a whole radix-12 or
// radix-16 DFT on them (itself 3 x 4 or 4 x 4 with constant internal
// twiddles), so a 3072-point transform is three Stockham passes -- 12, 16,
// 16 for the inverse and 16, 16, 12 for the forward -- with two exchanges
// through shared memory each:
//
//   inverse pass 1 (radix 12, 256 threads) reads u + i v straight from the
//     half-spectral rows (Hermitian extension on the fly) -- no staging;
//   inverse pass 3 (radix 16, 192 threads) ends with element t + 192 q of
//     the physical row in register slot 4 (q % 4) + q / 4 of thread t, and the
//     forward pass 1 (radix 16, Stockham stride M/16 = 192) reads exactly
//     those elements: the products u v and v^2 - u^2 are formed in place and
//     transformed by a 16-point DFT that takes its input in that order, with
//     no exchange in between;
//   forward pass 3 (radix 12, 256 threads) ends with P[t + 256 q] in
//     thread t; the split into the two half spectra needs P[M - k], which
//     one small exchange of the upper registers provides.
//
// Per element and row that is about 10 shared-memory accesses against
// about 29 for the generic engine, each exchange with a buffer index free
// of bank conflicts (x32_i1, x32_i2).  Twiddles between passes come from the handle's
// complex table tw[e] = exp(-2 pi i e / M) (conjugated for the inverse).
#pragma once

#include "s2d_internal.h"

namespace s2d {

// Buffer index of element i in each of the five exchanges of a row, chosen
// so that both the stores and the loads of that exchange are free of bank
// conflicts in the half-warp phases of 8-byte accesses (counted on the host
// for every access pattern; one padding per 32 elements for all five left
// the stores 1.7x over the conflict-free wavefront count, as ncu showed):
//   X1 inverse 1 -> 2, X2 inverse 2 -> 3, X3 forward 1 -> 2,
//   X4 forward 2 -> 3, X5 the split's partners.
__device__ __forceinline__ int x32_i1(int i) { return i ^ ((i >> 4) & 3); }
__device__ __forceinline__ int x32_i2(int i) { return i + (i >> 4); }

__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return f2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return f2(a.x - b.x, a.y - b.y); }
// a * w (S = -1, forward) or a * conj(w) (S = +1, inverse) for w from the
// forward table
template <int S>
__device__ __forceinline__ float2 f2tw(float2 a, float2 w) {
    return S < 0 ? f2(a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x) : f2(a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y);
}
// a * (c + i S s)
template <int S>
__device__ __forceinline__ float2 f2rot(float2 a, float c, float s) {
    const float ss = S > 0 ? s : -s;
    return f2(a.x * c - a.y * ss, a.x * ss + a.y * c);
}
// a * (S i)
template <int S>
__device__ __forceinline__ float2 f2i(float2 a) {
    return S > 0 ? f2(-a.y, a.x) : f2(a.y, -a.x);
}

// In-place 4-point DFT with kernel exp(S 2 pi i n k / 4).
template <int S>
__device__ __forceinline__ void x32_dft4(float2& a, float2& b, float2& c, float2& d) {
    const float2 t0 = f2add(a, c), t1 = f2sub(a, c), t2 = f2add(b, d), t3 = f2i<S>(f2sub(b, d));
    a = f2add(t0, t2);
    c = f2sub(t0, t2);
    b = f2add(t1, t3);
    d = f2sub(t1, t3);
}

// In-place 3-point DFT with kernel exp(S 2 pi i n k / 3).
template <int S>
__device__ __forceinline__ void x32_dft3(float2& a, float2& b, float2& c) {
    const float h = 0.5f, s3 = 0.86602540378443864676f;
    const float2 t1 = f2add(b, c), t2 = f2sub(b, c);
    const float2 m = f2(a.x - h * t1.x, a.y - h * t1.y);
    const float2 r = f2i<S>(f2(s3 * t2.x, s3 * t2.y));
    a = f2add(a, t1);
    b = f2add(m, r);
    c = f2sub(m, r);
}

// 16-point DFT (kernel exp(S 2 pi i n k / 16)) of x[0..15]; X[k] is left in
// x[4 (k % 4) + k / 4].  n = 4 n1 + n2, k = k1 + 4 k2: 4-point DFTs over n1,
// internal twiddles exp(S 2 pi i n2 k1 / 16), 4-point DFTs over n2.
template <int S>
__device__ __forceinline__ void x32_dft16(float2* x) {
    const float c1 = 0.92387953251128675613f, s1 = 0.38268343236508977173f;   // 2 pi / 16
    const float c2 = 0.70710678118654752440f;                                 // 2 pi 2 / 16
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) x32_dft4<S>(x[n2], x[n2 + 4], x[n2 + 8], x[n2 + 12]);
    // slot n2 + 4 k1 holds Y[n2][k1]; twiddle by W16^(n2 k1)
    x[1 + 4] = f2rot<S>(x[1 + 4], c1, s1);        // n2=1,k1=1: W^1
    x[1 + 8] = f2rot<S>(x[1 + 8], c2, c2);        // n2=1,k1=2: W^2
    x[1 + 12] = f2rot<S>(x[1 + 12], s1, c1);      // n2=1,k1=3: W^3
    x[2 + 4] = f2rot<S>(x[2 + 4], c2, c2);        // n2=2,k1=1: W^2
    x[2 + 8] = f2i<S>(x[2 + 8]);                  // n2=2,k1=2: W^4 = S i
    x[2 + 12] = f2rot<S>(x[2 + 12], -c2, c2);     // n2=2,k1=3: W^6
    x[3 + 4] = f2rot<S>(x[3 + 4], s1, c1);        // n2=3,k1=1: W^3
    x[3 + 8] = f2rot<S>(x[3 + 8], -c2, c2);       // n2=3,k1=2: W^6
    x[3 + 12] = f2rot<S>(x[3 + 12], -c1, -s1);    // n2=3,k1=3: W^9
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) x32_dft4<S>(x[4 * k1], x[4 * k1 + 1], x[4 * k1 + 2], x[4 * k1 + 3]);
}

// The same 16-point DFT taking its input in that permuted order (x[n] in
// slot 4 (n % 4) + n / 4) and leaving X[k] in slot k: 4-point DFTs over n1
// on contiguous slots 4 n2 + n1, twiddles, 4-point DFTs over n2.
template <int S>
__device__ __forceinline__ void x32_dft16t(float2* x) {
    const float c1 = 0.92387953251128675613f, s1 = 0.38268343236508977173f;
    const float c2 = 0.70710678118654752440f;
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) x32_dft4<S>(x[4 * n2], x[4 * n2 + 1], x[4 * n2 + 2], x[4 * n2 + 3]);
    // slot 4 n2 + k1 holds Y[n2][k1]
    x[4 + 1] = f2rot<S>(x[4 + 1], c1, s1);        // n2=1,k1=1: W^1
    x[4 + 2] = f2rot<S>(x[4 + 2], c2, c2);        // n2=1,k1=2: W^2
    x[4 + 3] = f2rot<S>(x[4 + 3], s1, c1);        // n2=1,k1=3: W^3
    x[8 + 1] = f2rot<S>(x[8 + 1], c2, c2);        // n2=2,k1=1: W^2
    x[8 + 2] = f2i<S>(x[8 + 2]);                  // n2=2,k1=2: W^4
    x[8 + 3] = f2rot<S>(x[8 + 3], -c2, c2);       // n2=2,k1=3: W^6
    x[12 + 1] = f2rot<S>(x[12 + 1], s1, c1);      // n2=3,k1=1: W^3
    x[12 + 2] = f2rot<S>(x[12 + 2], -c2, c2);     // n2=3,k1=2: W^6
    x[12 + 3] = f2rot<S>(x[12 + 3], -c1, -s1);    // n2=3,k1=3: W^9
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) x32_dft4<S>(x[k1], x[k1 + 4], x[k1 + 8], x[k1 + 12]);
}

// 12-point DFT of x[0..11]; X[k] is left in x[3 (k % 4) + k / 4].
// n = 3 n1 + n2, k = k1 + 4 k2: 4-point DFTs over n1, twiddles
// exp(S 2 pi i n2 k1 / 12), 3-point DFTs over n2.
template <int S>
__device__ __forceinline__ void x32_dft12(float2* x) {
    const float c1 = 0.86602540378443864676f, s1 = 0.5f;   // 2 pi / 12
#pragma unroll
    for (int n2 = 0; n2 < 3; ++n2) x32_dft4<S>(x[n2], x[n2 + 3], x[n2 + 6], x[n2 + 9]);
    // slot n2 + 3 k1 holds Y[n2][k1]; twiddle by W12^(n2 k1)
    x[1 + 3] = f2rot<S>(x[1 + 3], c1, s1);       // W^1
    x[1 + 6] = f2rot<S>(x[1 + 6], s1, c1);       // W^2
    x[1 + 9] = f2i<S>(x[1 + 9]);                 // W^3
    x[2 + 3] = f2rot<S>(x[2 + 3], s1, c1);       // W^2
    x[2 + 6] = f2rot<S>(x[2 + 6], -s1, c1);      // W^4
    x[2 + 9] = f2(-x[2 + 9].x, -x[2 + 9].y);     // W^6
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) x32_dft3<S>(x[3 * k1], x[3 * k1 + 1], x[3 * k1 + 2]);
}

// The x-pass of one group of 256 threads on row y (active: y < d.rows):
// u + i v from the half-spectral rows Iu[y], Iv[y] (kx in [0, K]) -> inverse
// FFT -> (u v, v^2 - u^2) -> forward FFT -> the two half spectra written
// back to the rows (their 1/(2 M^2) is carried by the prescaled u, v).
// Every thread of the CTA calls it (it synchronises the CTA); sb is the
// group's kX32Buf-element buffer.
__device__ __forceinline__ void xpass32_m3072_row(const Dims& d, float2* Iu, float2* Iv,
                                                  const float2* __restrict__ tw, int y, bool active, int t,
                                                  float2* sb) {
    constexpr int M = kX32M;
    const int K = d.K;
    float2* urow = Iu + (size_t)(active ? y : 0) * d.ldI;
    float2* vrow = Iv + (size_t)(active ? y : 0) * d.ldI;
    float2 x[16];
    // ---- inverse pass 1: radix 12, Ns = 1; z[t + 256 r] built from the rows
#pragma unroll
    for (int r = 0; r < 12; ++r) {
        const int n = t + 256 * r;
        float2 z = f2(0.f, 0.f);
        if (active) {
            if (n == 0) {
                z = f2(__ldcg(&urow[0]).x, __ldcg(&vrow[0]).x);
            } else if (n <= K) {
                const float2 a = __ldcg(&urow[n]), b = __ldcg(&vrow[n]);
                z = f2(a.x - b.y, a.y + b.x);
            } else if (n >= M - K) {
                const float2 a = __ldcg(&urow[M - n]), b = __ldcg(&vrow[M - n]);
                z = f2(a.x + b.y, b.x - a.y);
            }
        }
        x[r] = z;
    }
    x32_dft12<+1>(x);
#pragma unroll
    for (int q = 0; q < 12; ++q) sb[x32_i1(12 * t + q)] = x[3 * (q % 4) + q / 4];
    __syncthreads();
    // ---- inverse pass 2: radix 16, Ns = 12 (threads < 192)
    const bool r16 = t < 192;
    const int k12 = t % 12;
    if (r16) {
#pragma unroll
        for (int r = 0; r < 16; ++r) x[r] = sb[x32_i1(t + 192 * r)];
#pragma unroll
        for (int r = 1; r < 16; ++r) x[r] = f2tw<+1>(x[r], __ldg(&tw[16 * r * k12]));
        x32_dft16<+1>(x);
    }
    __syncthreads();
    if (r16) {
#pragma unroll
        for (int q = 0; q < 16; ++q) sb[x32_i2((t - k12) * 16 + k12 + 12 * q)] = x[4 * (q % 4) + q / 4];
    }
    __syncthreads();
    // ---- inverse pass 3: radix 16, Ns = 192 -> z[t + 192 q]; products;
    //      forward pass 1: radix 16, Ns = 1 on p[t + 192 r] in registers
    if (r16) {
#pragma unroll
        for (int r = 0; r < 16; ++r) x[r] = sb[x32_i2(t + 192 * r)];
#pragma unroll
        for (int r = 1; r < 16; ++r) x[r] = f2tw<+1>(x[r], __ldg(&tw[r * t]));
        x32_dft16<+1>(x);   // z[t + 192 q] in slot 4 (q % 4) + q / 4
#pragma unroll
        for (int s = 0; s < 16; ++s) {
            const float2 z = x[s];
            x[s] = f2(z.x * z.y, z.y * z.y - z.x * z.x);
        }
        x32_dft16t<-1>(x);  // input in that order, output q in slot q
    }
    __syncthreads();
    if (r16) {
#pragma unroll
        for (int q = 0; q < 16; ++q) sb[x32_i2(16 * t + q)] = x[q];
    }
    __syncthreads();
    // ---- forward pass 2: radix 16, Ns = 16
    const int k16 = t % 16;
    if (r16) {
#pragma unroll
        for (int r = 0; r < 16; ++r) x[r] = sb[x32_i2(t + 192 * r)];
#pragma unroll
        for (int r = 1; r < 16; ++r) x[r] = f2tw<-1>(x[r], __ldg(&tw[12 * r * k16]));
        x32_dft16<-1>(x);
    }
    __syncthreads();
    if (r16) {
#pragma unroll
        for (int q = 0; q < 16; ++q) sb[x32_i2((t - k16) * 16 + k16 + 16 * q)] = x[4 * (q % 4) + q / 4];
    }
    __syncthreads();
    // ---- forward pass 3: radix 12, Ns = 256 -> P[t + 256 q]
#pragma unroll
    for (int r = 0; r < 12; ++r) x[r] = sb[x32_i2(t + 256 * r)];
#pragma unroll
    for (int r = 1; r < 12; ++r) x[r] = f2tw<-1>(x[r], __ldg(&tw[r * t]));
    x32_dft12<-1>(x);
    __syncthreads();
    // P[2048 .. 3071] (q = 8..11) through shared memory for the partners
    // P[M - k] of the outputs k in [1, K]
#pragma unroll
    for (int q = 8; q < 12; ++q) sb[t + 256 * q] = x[3 * (q % 4) + q / 4];
    __syncthreads();
    if (active) {
#pragma unroll
        for (int r = 0; r < 5; ++r) {
            const int k = t + 256 * r;
            if (k <= K) {
                const float2 p = x[3 * (r % 4) + r / 4];
                const float2 q = k == 0 ? p : sb[M - k];
                urow[k] = f2(p.x + q.x, p.y - q.y);
                vrow[k] = f2(p.y + q.y, q.x - p.x);
            }
        }
    }
}

}  // namespace s2d
