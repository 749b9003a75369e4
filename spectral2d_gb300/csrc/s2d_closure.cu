// s2d_closure.cu -- learned subgrid closure for coarse LES (no counterpart in
// the reference).
//
// Data: the DNS state is sharp-spectrally filtered to the LES's retained
// modes |k| <= nx_les/2 (a Truncate-style mask with a smaller radius,
// src/Spectral.F90:788-802), and the subgrid vorticity flux
//     Pi^ = T[N_dns(w)] - N_les(T w),   N(w) = F[u . grad w] (dealiased),
// is formed in spectral space from the two solvers' right-hand sides
// (N = -(dW + nu k^2 w)).  Fields go to the LES collocation grid (3/2 rule,
// M = 3 nx_les / 2) for the network.
//
// Network: 6 circular 3x3 convolutions, 2 -> 32 -> 32 -> 32 -> 32 -> 32 -> 1
// channels, GELU (erf) after the first five; activations and working weights
// in BF16, accumulation FP32, FP32 master weights, Adam.  Convolutions are
// implicit GEMMs (pixels x out-channels x 9*in-channels): the forward pass and
// the data gradient on the tcgen05 tensor cores (BF16 operands from shared
// memory, FP32 accumulator in tensor memory), the weight gradient on the
// tensor cores too (k_wgrad_tc: a contraction over pixels with MN-major
// operands) with a deterministic two-stage reduction over CTAs.  Channel counts are padded to multiples of 16
// (input 2 -> 16, output 1 -> 16) with zero weights.
//
// LES with closure: each step the network maps (w, psi) of the LES state to
// Pi on the collocation grid; -Pi^ (truncated) is added to dW in all three
// RK3 stages of the step.
#include "s2d.h"
#include "s2d_internal.h"
#include "s2d_step.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace s2d {

constexpr int kLayers = 6;
constexpr int kCinP[kLayers] = {16, 32, 32, 32, 32, 32};
constexpr int kCoutP[kLayers] = {32, 32, 32, 32, 32, 16};
constexpr int kCin[kLayers] = {2, 32, 32, 32, 32, 32};
constexpr int kCout[kLayers] = {32, 32, 32, 32, 32, 1};

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }
__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}
__device__ __forceinline__ float2 unpack_bf16(uint32_t u) {
    __nv_bfloat162 h = *reinterpret_cast<__nv_bfloat162*>(&u);
    return __bfloat1622float2(h);
}
// GELU (erf form) with erf from Abramowitz & Stegun 7.1.26 (Hastings): for
// z >= 0, 1 - erf(z) = t (a1 + t (a2 + t (a3 + t (a4 + t a5)))) exp(-z^2) with
// t = 1 / (1 + p z), |error| <= 1.5e-7 (3.3e-7 for gelu in FP32 arithmetic),
// far below the BF16 resolution of the activations, in about a third of the
// instructions of erff.  With z = |x| / sqrt(2), q = 1 - erf(z) and e =
// exp(-x^2 / 2): gelu(x) = x (1 - q/2) for x >= 0, x q / 2 for x < 0, and
// gelu'(x) = Phi(x) + x e / sqrt(2 pi) with Phi(x) = 1 - q/2 or q/2.
struct GeluQE {
    float q, e;
};
__device__ __forceinline__ GeluQE gelu_qe(float x) {
    const float z = fabsf(x) * 0.70710678118654752f;
    const float t = __fdividef(1.0f, fmaf(0.3275911f, z, 1.0f));
    const float pt = fmaf(fmaf(fmaf(fmaf(1.061405429f, t, -1.453152027f), t, 1.421413741f), t, -0.284496736f), t,
                          0.254829592f);
    const float e = __expf(-0.5f * x * x);
    return {t * pt * e, e};
}
__device__ __forceinline__ float gelu_f(float x) {
    const float hq = 0.5f * gelu_qe(x).q;
    return x >= 0.0f ? x - x * hq : x * hq;
}
__device__ __forceinline__ float gelu_grad_f(float x) {
    const GeluQE g = gelu_qe(x);
    const float cdf = x >= 0.0f ? 1.0f - 0.5f * g.q : 0.5f * g.q;
    return cdf + x * 0.39894228040143268f * g.e;
}

// ---- tcgen05 (5th-generation tensor core) helpers -----------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor, no swizzle, K-major operand stored as
// 8-row x 16-byte core matrices: lbo = byte step between core matrices along
// K, sbo = byte step between 8-row groups along M (or N).
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;   // descriptor version of the sm_100 family; base offset 0, no swizzle
    return d;
}

// Instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

constexpr int kMbarSpinLimit = 1 << 22;

// Shared-memory matrix descriptor of a K-major operand stored with the
// 32- or 64-byte swizzle (rows of ROWB = 32 or 64 bytes, 8-row atoms of
// 8 * ROWB bytes, 16-byte chunk c of row r stored at chunk c ^ ((r >> s) & m)
// with s = 2, m = 1 for 32 B and s = 1, m = 3 for 64 B -- the layout TMA
// writes with CU_TENSOR_MAP_SWIZZLE_32B / _64B): sbo = the atom stride; a K
// offset within a row is added to the start address.
template <int ROWB>
__device__ __forceinline__ uint64_t umma_desc_sw(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;                                    // leading offset: unused for this layout
    d |= (uint64_t)(((8u * ROWB) >> 4) & 0x3FFFu) << 32;       // stride offset: one 8-row atom
    d |= (uint64_t)1 << 46;                                    // descriptor version of the sm_100 family
    d |= (uint64_t)(ROWB == 64 ? 4 : 6) << 61;                 // 64-byte or 32-byte swizzle
    return d;
}

// TMA: one box of a 4-D tensor map into shared memory, its bytes counted on
// the mbarrier bar (which the issuing thread armed with expect_tx).
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];\n" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}

// Bounded wait of one thread on an mbarrier phase.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
    for (int it = 0; it < kMbarSpinLimit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Implicit-GEMM 3x3 circular convolution on the tcgen05 tensor cores.
// A CTA (8 warps) owns an output tile of 8 rows x 14 columns of one image at
// a time (persistent: tiles blockIdx.x, + gridDim.x, ...).  Its halo, image
// rows ty0 - 1 .. ty0 + 8 and columns tx0 - 1 .. tx0 + 14, is one TMA box of
// 10 x 16 pixels, a pixel's KC channels (32 or 64 bytes) per box row,
// swizzled (32 or 64 B) as the tensor core reads K-major operands.  The
// three column taps sit side by side in the MMA's N dimension:
//   D[128 box pixels, (dx, n)] += A_dy[128, KC] B_dy[KC, 3 NC]
// over the three rows of taps dy and the K steps of 16 channels (3 KC / 16
// MMAs of N = 3 NC per tile), A_dy being box rows dy .. dy + 7 (a whole
// number of 8-pixel atoms: a descriptor into the box) and B_dy the weights
// of row dy, column group (dx, 8 output channels), K-major, no swizzle,
// staged once.  Output pixel (r, c) of the box (columns 1 .. 14 are the
// tile's) sums tap dx evaluated at box pixel (r, c + dx - 1): the epilogue
// adds the three column blocks with shuffles inside the 16 lanes of a box
// row.  The tensor map zero-fills what lies outside the image; for tiles at
// an edge those positions are rewritten with the circularly wrapped pixels
// once the box has landed.
// Thread 0 issues the TMA load and the MMAs, commits them to an mbarrier and
// waits for it (every wait bounded); once the MMAs have read the box it
// loads the next tile's box into the same slot, so that it flies while this
// tile's epilogue runs.  The 8 warps read the accumulator for the epilogue,
// warp w lanes 32 (w % 4) .. + 31 (tcgen05.ld reaches the lane quarter
// w % 4) and, of each column block, channels 16 (w / 4) .. + 15:
//   EPI 0: + bias, store z (unless z is null: no backward follows) and
//   gelu(z) (BF16); 1: + bias, channel 0 as FP32;
//   2: multiply by gelu'(zprev), store BF16.
//   FWD (SIGN = +1): out[p, n] = sum_{t,k} in[p + off_t, k] W[n, t, k]
//   data gradient (SIGN = -1): out[q, n] = sum_{t,k} in[q - off_t, k] W^T[n, t, k]
// A wait that exceeds its iteration limit sets bit 4 of *err and skips the
// rest (the kernel waits, bounded, for its loads and MMAs in flight, frees
// its tensor memory and returns).
constexpr int kConvTY = 8;    // output rows of a tile
constexpr int kConvTX = 16;   // box width in pixels
constexpr int kConvOW = 14;   // output columns of a tile (box columns 1 .. 14)

template <int KC, int NC>
struct ConvTile {
    static constexpr int KG = KC / 8;                      // 8-channel groups
    static constexpr int HR = kConvTY + 2;                 // halo rows
    static constexpr int CORE = 128;                       // bytes of one no-swizzle core matrix
    static constexpr int ROWB = KC * 2;                    // bytes of one pixel (one swizzled row)
    static constexpr int BOX = HR * kConvTX * ROWB;        // one TMA box: 10 rows x 16 pixels
    static constexpr int N = 3 * NC;                       // MMA columns: (dx, output channel)
    static constexpr int NG = N / 8;                       // 8-column groups
    static constexpr int WGROUP = KG * CORE;               // weights of 8 columns, all input channels
    static constexpr int WBYTES = 3 * NG * WGROUP;         // weights of all taps
    static constexpr int TMEM_COLS = N <= 64 ? 64 : 128;   // power of two >= N
    static constexpr size_t SMEM = BOX + WBYTES + 1024;    // + slack to align the base to 1024 B
    static_assert(BOX % 1024 == 0, "boxes stay aligned to the swizzle pattern");
    static_assert(N % 16 == 0 && N <= 256, "M = 128 MMA shape");
};

constexpr int kConvThreads = 256;

template <int KC, int NC, int SIGN, int EPI>
__global__ void __launch_bounds__(kConvThreads, 4) k_conv_tc(const __grid_constant__ CUtensorMap tin,
                                                 const __nv_bfloat16* __restrict__ in,
                                                 const __nv_bfloat16* __restrict__ W,
                                                 const float* __restrict__ bias,
                                                 const __nv_bfloat16* __restrict__ zprev, __nv_bfloat16* z,
                                                 __nv_bfloat16* a, float* yout, int B, int H, int Wd,
                                                 unsigned int* err) {
    using TL = ConvTile<KC, NC>;
    constexpr int KG = TL::KG;
    constexpr int ROWB = TL::ROWB;
    constexpr int NG = TL::NG;
    constexpr int TMEM_COLS = TL::TMEM_COLS;
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    const uint32_t sraw = smem_u32(tc_smem);
    const uint32_t sbase = (sraw + 1023u) & ~1023u;        // the halo box, then the weights
    unsigned char* gbase = tc_smem + (sbase - sraw);
    const uint32_t bw = sbase + TL::BOX;
    __shared__ __align__(8) uint64_t mbar_mma;
    __shared__ __align__(8) uint64_t mbar_full;
    __shared__ uint32_t tmem_base;
    __shared__ int s_ok;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tiles_x = (Wd + kConvOW - 1) / kConvOW;
    const int tiles_img = tiles_x * ((H + kConvTY - 1) / kConvTY);
    const int ntiles = tiles_img * B;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    const uint32_t bar_mma = smem_u32(&mbar_mma);
    const uint32_t bar_full = smem_u32(&mbar_full);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar_mma) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar_full) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        s_ok = 1;
    }
    // weights (once per CTA): row of taps dyi, column group g = (dxi, 8
    // output channels), channels [8 kg, 8 kg + 8).  Block (dyi, dxi) meets
    // the input at offset (dyi - 1, dxi - 1): tap (dyi, dxi) of W forward,
    // the mirrored tap of W^T for the data gradient.
    for (int i = tid; i < 3 * TL::N * KG; i += blockDim.x) {
        const int nl = i % 8;
        const int kg = (i / 8) % KG;
        const int g = (i / (8 * KG)) % NG;
        const int dyi = i / (8 * KG * NG);
        const int dxi = g / (NC / 8);
        const int n = (g % (NC / 8)) * 8 + nl;
        const int t = (SIGN * (dyi - 1) + 1) * 3 + (SIGN * (dxi - 1) + 1);
        const uint4 v = *reinterpret_cast<const uint4*>(W + ((long)n * 9 + t) * KC + kg * 8);
        const int off = ((dyi * NG + g) * KG + kg) * TL::CORE + nl * 16;
        *reinterpret_cast<uint4*>(gbase + TL::BOX + off) = v;
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = tmem_base;
    // Launched as a programmatic dependent (the closure's inference chain
    // only, where the weights do not change), the prologue above -- TMEM
    // columns, barriers, the layer's weights -- overlaps the previous kernel;
    // the input activations and the outputs are touched only after this.  A
    // CTA waiting for its TMEM columns waits only on CTAs (of this launch or
    // the one before) that run to completion without waiting on it.
    pdl_enter();

    // thread 0's bookkeeping: the parity to wait for on each barrier and what
    // is in flight
    uint32_t ph_mma = 0, ph_full = 0;
    bool pend = false, mma_pend = false;
    auto issue_load = [&](int tile) {
        const int b = tile / tiles_img;
        const int tl = tile - b * tiles_img;
        const int tx0 = (tl % tiles_x) * kConvOW;
        const int ty0 = (tl / tiles_x) * kConvTY;
        mbar_expect_tx(bar_full, (uint32_t)TL::BOX);
        tma_load_4d(sbase, &tin, 0, tx0 - 1, ty0 - 1, b, bar_full);
        pend = true;
    };
    if (tid == 0 && (int)blockIdx.x < ntiles) issue_load(blockIdx.x);

    int it = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
        const int b = tile / tiles_img;
        const int tl = tile - b * tiles_img;
        const int tx0 = (tl % tiles_x) * kConvOW;
        const int ty0 = (tl / tiles_x) * kConvTY;
        const long img = (long)b * H * Wd;

        if (tid == 0) {
            if (mbar_wait_bounded(bar_full, ph_full)) {
                ph_full ^= 1u;
                pend = false;
            } else {
                s_ok = 0;
            }
        }
        __syncthreads();
        if (!s_ok) break;

        // circular wrap at the image edges: rewrite the zero-filled positions
        // (box columns tx0 - 1 .. tx0 + 14, rows ty0 - 1 .. ty0 + 8)
        if (tx0 == 0 || ty0 == 0 || tx0 + kConvOW >= Wd || ty0 + kConvTY >= H) {
            // each writer observes the completed phase itself (the k-th load
            // has parity k & 1), so its stores follow the box's fill
            (void)mbar_try_wait(bar_full, (uint32_t)it & 1u);
            for (int i = tid; i < TL::HR * kConvTX * KG; i += blockDim.x) {
                const int q = i % KG;   // 16-byte chunk of the pixel
                const int r = i / KG;
                const int c = r % kConvTX;
                const int hr = r / kConvTX;
                int yy = ty0 + hr - 1, xx = tx0 + c - 1;
                if (yy >= 0 && yy < H && xx >= 0 && xx < Wd) continue;
                // yy in [-1, H + 8), xx in [-1, Wd + 14): at most two wraps (grid >= 8)
                yy += yy < 0 ? H : 0;
                yy -= yy >= H ? H : 0;
                yy -= yy >= H ? H : 0;
                xx += xx < 0 ? Wd : 0;
                xx -= xx >= Wd ? Wd : 0;
                xx -= xx >= Wd ? Wd : 0;
                const uint4 v = *reinterpret_cast<const uint4*>(in + (img + (long)yy * Wd + xx) * KC + q * 8);
                const int pq = ROWB == 64 ? (q ^ ((r >> 1) & 3)) : (q ^ ((r >> 2) & 1));
                *reinterpret_cast<uint4*>(gbase + r * ROWB + pq * 16) = v;
            }
        }
        // the rewritten positions must be visible to the tensor core (async proxy)
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");

        if (tid == 0) {
            constexpr uint32_t idesc = umma_idesc_bf16(128, TL::N);
            const uint64_t ad0 = umma_desc_sw<ROWB>(sbase);
            const uint64_t bd0 = umma_desc(bw, TL::CORE, TL::WGROUP);
#pragma unroll
            for (int dyi = 0; dyi < 3; ++dyi) {
#pragma unroll
                for (int j = 0; j < KC / 16; ++j) {
                    // start addresses advance in 16-byte units in the low field
                    const uint64_t ad = ad0 + (uint64_t)((dyi * kConvTX * ROWB + j * 32) >> 4);
                    const uint64_t bd = bd0 + (uint64_t)((dyi * NG * TL::WGROUP + j * 2 * TL::CORE) >> 4);
                    asm volatile(
                        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                        "l"(ad), "l"(bd), "r"(idesc), "r"((dyi | j) ? 1u : 0u)
                        : "memory");
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar_mma)
                         : "memory");
            mma_pend = true;
            if (mbar_wait_bounded(bar_mma, ph_mma)) {
                ph_mma ^= 1u;
                mma_pend = false;
                // the MMAs have read the box: the next tile's box loads
                // while this tile's epilogue runs
                if (tile + (int)gridDim.x < ntiles) issue_load(tile + gridDim.x);
            } else {
                s_ok = 0;
            }
        }
        __syncthreads();
        if (!s_ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");

        // warp w reads accumulator lanes 32 (w % 4) .. + 31 (box pixels m:
        // row m / 16, column m % 16) and, of each column block dx, channels
        // 16 (w / 4) .. + 15; pixel m sums block dx at box pixel m + dx - 1
        const int quarter = warp & 3, half = warp >> 2;
        const bool cols = half * 16 < NC;   // warp-uniform
        float s[16];
        if (cols) {
            const uint32_t trow = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(half * 16);
#pragma unroll
            for (int e = 0; e < 16; ++e) s[e] = 0.0f;
#pragma unroll
            for (int dxi = 0; dxi < 3; ++dxi) {
                if constexpr (EPI == 1) {   // channel 0 only
                    uint32_t r0;
                    asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];\n"
                                 : "=r"(r0)
                                 : "r"(trow + (uint32_t)(dxi * NC)));
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                    const float v = __uint_as_float(r0);
                    s[0] += dxi == 0   ? __shfl_up_sync(0xffffffffu, v, 1, kConvTX)
                            : dxi == 1 ? v
                                       : __shfl_down_sync(0xffffffffu, v, 1, kConvTX);
                    continue;
                }
                uint32_t r[16];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                    "[%16];\n"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                      "=r"(r[15])
                    : "r"(trow + (uint32_t)(dxi * NC)));
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
                for (int e = 0; e < 16; ++e) {
                    const float v = __uint_as_float(r[e]);
                    s[e] += dxi == 0   ? __shfl_up_sync(0xffffffffu, v, 1, kConvTX)
                            : dxi == 1 ? v
                                       : __shfl_down_sync(0xffffffffu, v, 1, kConvTX);
                }
            }
        }
        // the next tile's MMAs may overwrite the accumulator only after every
        // warp has read it
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();

        const int m = quarter * 32 + lane;
        const int c = m % kConvTX;
        const int y = ty0 + m / kConvTX, x = tx0 - 1 + c;
        if (cols && c >= 1 && c <= kConvOW && y < H && x < Wd) {
            const long p = img + (long)y * Wd + x;
            if (EPI == 1) {
                if (half == 0) yout[p] = s[0] + bias[0];
            } else {
#pragma unroll
                for (int qq = 0; qq < 2; ++qq) {
                    const int q = half * 2 + qq;   // 8-channel group of the output
                    uint32_t zz[4], aa[4];
                    uint4 zp = make_uint4(0, 0, 0, 0);
                    if (EPI == 2) zp = *reinterpret_cast<const uint4*>(zprev + p * NC + q * 8);
                    const uint32_t zpv[4] = {zp.x, zp.y, zp.z, zp.w};
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int n = q * 8 + 2 * e;
                        float v0 = s[qq * 8 + 2 * e], v1 = s[qq * 8 + 2 * e + 1];
                        if (EPI == 0) {
                            v0 += bias[n];
                            v1 += bias[n + 1];
                            zz[e] = pack_bf16(v0, v1);
                            aa[e] = pack_bf16(gelu_f(v0), gelu_f(v1));
                        } else {
                            const float2 g = unpack_bf16(zpv[e]);
                            zz[e] = pack_bf16(v0 * gelu_grad_f(g.x), v1 * gelu_grad_f(g.y));
                        }
                    }
                    if (EPI != 0 || z)
                        *reinterpret_cast<uint4*>(z + p * NC + q * 8) = make_uint4(zz[0], zz[1], zz[2], zz[3]);
                    if (EPI == 0)
                        *reinterpret_cast<uint4*>(a + p * NC + q * 8) = make_uint4(aa[0], aa[1], aa[2], aa[3]);
                }
            }
        }
    }
    if (!s_ok && tid == 0) {
        atomicOr(err, 4u);
        // give the MMAs and the loads in flight a second bounded chance to
        // finish before the memory goes
        if (mma_pend) mbar_wait_bounded(bar_mma, ph_mma);
        if (pend) mbar_wait_bounded(bar_full, ph_full);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS)
                     : "memory");
}

// cuTensorMapEncodeTiled from the driver, through the runtime (no link
// dependency on the driver library).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// Tensor map of B activation images [B][H][Wd][KC] (BF16, channels
// innermost) as the 4-D array {KC, Wd, H, B}, boxes of 16 pixels x `rows`
// rows (10: a tile and its halo) with the 32- (KC = 16) or 64-byte (KC = 32)
// swizzle.
template <int KC>
cudaError_t conv_tensor_map(CUtensorMap* map, const __nv_bfloat16* act, int B, int H, int Wd,
                            int rows = kConvTY + 2) {
    const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return cudaErrorNotSupported;
    const cuuint64_t dims[4] = {(cuuint64_t)KC, (cuuint64_t)Wd, (cuuint64_t)H, (cuuint64_t)B};
    const cuuint64_t strides[3] = {(cuuint64_t)KC * 2, (cuuint64_t)Wd * KC * 2, (cuuint64_t)H * Wd * KC * 2};
    const cuuint32_t box[4] = {(cuuint32_t)KC, kConvTX, (cuuint32_t)rows, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<__nv_bfloat16*>(act), dims, strides,
                           box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           KC == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// Launch k_conv_tc over B images of H x Wd: a persistent grid of up to four
// CTAs of 256 threads per SM (29 KB of shared memory each at KC = 32), each
// looping over 8 x 14-pixel output tiles.
template <int KC, int NC, int SIGN, int EPI>
cudaError_t launch_conv(const __nv_bfloat16* in, const __nv_bfloat16* W, const float* bias,
                        const __nv_bfloat16* zprev, __nv_bfloat16* z, __nv_bfloat16* a, float* yout, int B, int H,
                        int Wd, unsigned int* err, int sms, cudaStream_t st, bool pdl = false) {
    CUtensorMap map;
    const cudaError_t e = conv_tensor_map<KC>(&map, in, B, H, Wd);
    if (e != cudaSuccess) return e;
    const long ntiles = (long)((Wd + kConvOW - 1) / kConvOW) * ((H + kConvTY - 1) / kConvTY) * B;
    const int grid = (int)std::min<long>(ntiles, 4L * sms);
    return launch_k(k_conv_tc<KC, NC, SIGN, EPI>, grid, kConvThreads, ConvTile<KC, NC>::SMEM, st, pdl, map, in, W,
                    bias, zprev, z, a, yout, B, H, Wd, err);
}

// ---- the fused inference forward -----------------------------------------
// All six layers of the network in one persistent launch, for the forward
// passes that keep no pre-activations (the LES closure term, inference).
//
// Images carry a one-pixel circular frame: [B][H + 2][Wd + 2][KC], pixel
// (y, x) at (y + 1, x + 1), frame row 0 = image row H - 1, frame row H + 1 =
// image row 0, likewise the columns and the corners.  A layer's epilogue
// writes each border pixel into the frame as well (up to four copies), so
// the next layer's TMA boxes read the circular neighbourhood as it is, with
// no fix-up pass.  Activations ping-pong between two framed images; between
// layers the CTAs meet at a grid barrier (the launch is cooperative, so all
// of them are resident).
//
// The three column taps dx of a row of taps dy go side by side into the
// MMA's N dimension: for a box of 10 x 16 pixels (one TMA box, the tile's
// 8 x 14 outputs and their halo) D[m, (dx, n)] = sum over dy and channels of
// box pixel m + 16 (dy + 1) times W[n, (dy, dx), :], so a tile is 3 KC / 16
// MMAs of N = 3 NC (not 9 KC / 16 of N = NC, each of which streams the same
// 4 KB of activations from shared memory for only 32 columns), and output
// pixel m takes column block dx at pixel m + dx - 1, a warp shuffle.
// One CTA per SM (the cooperative limit): warp 17 issues the TMA loads of
// the boxes into four slots, warp 16 the MMAs of a tile into one of four
// tensor-memory accumulators (descriptors precomputed per slot: a row of
// taps is an offset of the start address), and two groups of eight warps
// take alternate tiles: read the accumulator, release it (mbarrier), sum the
// taps, apply bias and GELU and store, while the MMAs of the following tiles
// run.  The roles meet only at mbarriers: full (slot landed), mmad (its MMAs
// done: the accumulator ready, the slot free), accfree (accumulator read).
// Every wait is bounded: a wait that runs out sets bit 4 of *err and
// the abort flag, the CTA skips the rest (after bounded waits for its copies
// and MMAs in flight) and frees its tensor memory.
constexpr int kNetGroups = 2;                    // epilogue groups of 8 warps (tile i: group i % 2)
// Accumulators = box slots: tile i uses slot and accumulator i % 4, and one
// commit per tile (mmad) tells the epilogue the accumulator is ready and the
// producer the slot is free (a tcgen05.commit costs the tensor pipe about as
// much as three of these MMAs, so there is one per tile, not two).
constexpr int kNetAcc = 4;
constexpr int kNetEpiWarps = 8 * kNetGroups;     // warps 0-15
constexpr int kNetMmaWarp = kNetEpiWarps;        // warp 16
constexpr int kNetProdWarp = kNetEpiWarps + 1;   // warp 17
constexpr int kNetThreads = 32 * (kNetEpiWarps + 2);
constexpr int kNetAccCols = 128;                 // 3 * 32 columns used
constexpr int kNetTmemCols = kNetAccCols * kNetAcc;
constexpr int kNetOutH = 8, kNetOutW = 14;       // output tile
constexpr int kNetBoxRows = kNetOutH + 2, kNetBoxW = kNetOutW + 2;   // its halo box: M = 8 x 16 = 128 pixels
constexpr int kNetSlots = kNetAcc;
constexpr int kNetSlotBytes = kNetBoxRows * kNetBoxW * 64;   // one box of 32-channel pixels
constexpr int kNetWBytes = 3 * 96 * 4 * 16;                  // B operands of the three rows of taps
constexpr size_t kNetSmem = (size_t)kNetSlots * kNetSlotBytes + kNetWBytes + 1024;

struct NetArgs {
    const __nv_bfloat16* W[kLayers];   // BF16 working weights W[n][t][k]
    const float* bias[kLayers];
    __nv_bfloat16* act[2];             // framed 32-channel images
    float* y;                          // output channel 0, [B][H][Wd]
    unsigned int* bar;                 // grid barrier: arrivals of this launch
    unsigned int* err;
    int B, H, Wd;
    int stall;                         // fault injection: CTA 0 skips its first grid-barrier arrival
};

struct NetShared {
    uint64_t full[kNetSlots];   // the boxes of a slot have landed
    uint64_t mmad[kNetAcc];     // the MMAs of the tile in slot / accumulator are complete
    uint64_t accfree[kNetAcc];  // the 8 warps of its epilogue group have read an accumulator
    uint32_t tmem;
    int abort;
    float bias[32];
};

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
}

// Bounded wait that also gives up once another role of the CTA has aborted.
__device__ __forceinline__ bool net_wait(uint32_t bar, uint32_t parity, const volatile int* abort) {
    for (int it = 0; it < kMbarSpinLimit; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 255) == 255 && *abort) return false;
    }
    return false;
}

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    return t;
}

// Grid barrier of one thread per CTA (the CTA synchronised before and
// after): *bar counts the arrivals of the launch (zeroed before it), the
// j-th barrier opens at j * gridDim.x.  Bounded: false after a second.
__device__ __forceinline__ bool net_grid_sync(unsigned int* bar, unsigned int target) {
    __threadfence();
    atomicAdd(bar, 1u);
    const unsigned long long t0 = globaltimer_ns();
    while (ld_acquire_u32(bar) < target) {
        if (globaltimer_ns() - t0 > 1000000000ull) return false;
        __nanosleep(64);
    }
    return true;
}

// One layer over this CTA's tiles (tile blockIdx.x + k gridDim.x); irun is
// the CTA's running tile count over all layers, which fixes every slot,
// accumulator and barrier phase.
template <int KC, int NC, bool LAST>
__device__ __forceinline__ void net_layer(const CUtensorMap* tin, const __nv_bfloat16* __restrict__ W,
                                          const float* __restrict__ bias, __nv_bfloat16* out, float* yout,
                                          const NetArgs& a, NetShared& sh, unsigned char* gbase, uint32_t sbase,
                                          int& irun) {
    constexpr int KG = KC / 8;                 // 8-channel groups of a pixel
    constexpr int ROWB = KC * 2;               // bytes of one pixel
    constexpr int BOX = kNetBoxRows * kNetBoxW * ROWB;
    constexpr int N = 3 * NC;                  // the MMA's columns: (dx, output channel)
    constexpr int NG = N / 8;                  // 8-column groups
    constexpr int CORE = 128;
    constexpr int WGROUP = KG * CORE;          // 8 columns x all input channels
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int H = a.H, Wd = a.Wd;
    const int tiles_x = (Wd + kNetOutW - 1) / kNetOutW;
    const int tiles_img = tiles_x * ((H + kNetOutH - 1) / kNetOutH);
    const int ntiles = tiles_img * a.B;
    const int nk = (int)blockIdx.x < ntiles ? (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x : 0;
    const uint32_t bw = sbase + kNetSlots * kNetSlotBytes;
    volatile int* abort = &sh.abort;

    // the layer's weights as the B operands of the three rows of taps: for
    // row dy, column group g = (dx, 8 output channels), the input channels
    // K-major in core matrices (the previous layer's MMAs are all complete)
    for (int i = tid; i < 3 * N * KG; i += blockDim.x) {
        const int nl = i % 8;
        const int kg = (i / 8) % KG;
        const int g = (i / (8 * KG)) % NG;
        const int dyi = i / (8 * KG * NG);
        const int dxi = g / (NC / 8);
        const int n = (g % (NC / 8)) * 8 + nl;
        const int t = dyi * 3 + dxi;
        const uint4 v = *reinterpret_cast<const uint4*>(W + ((long)n * 9 + t) * KC + kg * 8);
        const int off = ((dyi * NG + g) * KG + kg) * CORE + nl * 16;
        *reinterpret_cast<uint4*>(gbase + kNetSlots * kNetSlotBytes + off) = v;
    }
    if (tid < NC) sh.bias[tid] = bias[tid];
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");

    // tile k: output rows [oy0, oy0 + 8), columns [ox0, ox0 + 14); its box is
    // image rows oy0 - 1 .. oy0 + 8 and columns ox0 - 1 .. ox0 + 14, at
    // framed coordinates (ox0, oy0)
    auto tile_xy = [&](int k, int& b, int& ox0, int& oy0) {
        const int tile = (int)blockIdx.x + k * (int)gridDim.x;
        b = tile / tiles_img;
        const int tl = tile - b * tiles_img;
        ox0 = (tl % tiles_x) * kNetOutW;
        oy0 = (tl / tiles_x) * kNetOutH;
    };
    const int i0 = irun;
    auto fail = [&]() {
        *abort = 1;
        atomicOr(a.err, 4u);
    };

    if (warp == kNetProdWarp) {
        // ---- TMA producer (one thread): one box per tile into slot
        // i % kNetSlots once the MMAs of tile i - kNetSlots have read it
        // (their commit on mmad, the slot's accumulator)
        if (lane == 0 && !*abort) {
            asm volatile("fence.proxy.async.global;\n" ::: "memory");
            int kl = 0;
            bool ok = true;
            for (; kl < nk; ++kl) {
                const int i = i0 + kl, s = i % kNetSlots;
                if (i >= kNetSlots &&
                    !(ok = net_wait(smem_u32(&sh.mmad[s]), (uint32_t)(i / kNetSlots - 1) & 1u, abort)))
                    break;
                int b, ox0, oy0;
                tile_xy(kl, b, ox0, oy0);
                const uint32_t bar = smem_u32(&sh.full[s]);
                mbar_expect_tx(bar, (uint32_t)BOX);
                tma_load_4d(sbase + s * kNetSlotBytes, tin, 0, ox0, oy0, b, bar);
            }
            if (!ok) {
                fail();
                // the loads that may still be in flight land before the memory goes
                for (int k = kl - kNetSlots < 0 ? 0 : kl - kNetSlots; k < kl; ++k) {
                    const int i = i0 + k;
                    mbar_wait_bounded(smem_u32(&sh.full[i % kNetSlots]), (uint32_t)(i / kNetSlots) & 1u);
                }
            }
        }
    } else if (warp == kNetMmaWarp) {
        // ---- MMA issuer (one thread): per tile 3 * KC / 16 MMAs of
        // M = 128 box pixels, N = 3 NC (the three column taps side by side),
        // K = 16 channels, one per row of taps dy and channel step, into
        // accumulator i % 4; one commit to mmad (epilogue and producer)
        if (lane == 0 && !*abort) {
            const uint64_t bd0 = umma_desc(bw, CORE, WGROUP);
            constexpr uint32_t idesc = umma_idesc_bf16(128, N);
            int km = -1;
            bool ok = true;
            for (int k = 0; k < nk; ++k) {
                const int i = i0 + k, s = i % kNetSlots, acc = i % kNetAcc;
                if (!(ok = net_wait(smem_u32(&sh.full[s]), (uint32_t)(i / kNetSlots) & 1u, abort))) break;
                if (i >= kNetAcc &&
                    !(ok = net_wait(smem_u32(&sh.accfree[acc]), (uint32_t)(i / kNetAcc - 1) & 1u, abort)))
                    break;
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint64_t ad0 = umma_desc_sw<ROWB>(sbase + s * kNetSlotBytes);
                const uint32_t dacc = sh.tmem + (uint32_t)(acc * kNetAccCols);
#pragma unroll
                for (int dyi = 0; dyi < 3; ++dyi) {
#pragma unroll
                    for (int j = 0; j < KC / 16; ++j) {
                        // box rows dyi .. dyi + 7 (whole 8-pixel atoms); start
                        // addresses advance in 16-byte units in the low field
                        const uint64_t ad = ad0 + (uint64_t)((dyi * kNetBoxW * ROWB + j * 32) >> 4);
                        const uint64_t bd = bd0 + (uint64_t)((dyi * NG * WGROUP + j * 2 * CORE) >> 4);
                        asm volatile(
                            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dacc),
                            "l"(ad), "l"(bd), "r"(idesc), "r"((dyi | j) ? 1u : 0u)
                            : "memory");
                    }
                }
                asm volatile(
                    "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                        smem_u32(&sh.mmad[acc]))
                    : "memory");
                km = k;
            }
            if (!ok) {
                fail();
                if (km >= 0) {
                    const int i = i0 + km;
                    mbar_wait_bounded(smem_u32(&sh.mmad[i % kNetAcc]), (uint32_t)(i / kNetAcc) & 1u);
                }
            }
        }
    } else {
        // ---- epilogue warps: group g = w / 8 takes the tiles with i % 2 == g;
        // warp w reads accumulator lanes 32 (w % 4) .. + 31 (box pixels m: row
        // m / 16, column m % 16) and, of each tap column dx, the output
        // channels 16 ((w % 8) / 4) .. + 15.  Output pixel m sums tap dx
        // evaluated at box pixel m + dx: a shuffle within the 16 lanes of its
        // row; box columns 1 .. 14 are the tile's outputs.
        const int grp = warp >> 3, quarter = warp & 3, half = (warp >> 2) & 1;
        const bool cols = half * 16 < NC;   // warp-uniform
        const long fw = Wd + 2;
        // this thread's 16 biases in registers (shared-memory reads per tile
        // would compete with the tensor core's operand reads)
        float bv[16];
#pragma unroll
        for (int e = 0; e < 16; ++e) bv[e] = cols ? sh.bias[half * 16 + e] : 0.0f;
        for (int k = (grp - (i0 & 1) + 2) & 1; k < nk; k += kNetGroups) {
            const int i = i0 + k, acc = i % kNetAcc;
            if (!net_wait(smem_u32(&sh.mmad[acc]), (uint32_t)(i / kNetAcc) & 1u, abort)) {
                fail();
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            uint32_t r[3][16];
            if (cols) {
#pragma unroll
                for (int dxi = 0; dxi < 3; ++dxi) {
                    const uint32_t taddr = sh.tmem + ((uint32_t)(quarter * 32) << 16) +
                                           (uint32_t)(acc * kNetAccCols + dxi * NC + half * 16);
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
                        "%15}, [%16];\n"
                        : "=r"(r[dxi][0]), "=r"(r[dxi][1]), "=r"(r[dxi][2]), "=r"(r[dxi][3]), "=r"(r[dxi][4]),
                          "=r"(r[dxi][5]), "=r"(r[dxi][6]), "=r"(r[dxi][7]), "=r"(r[dxi][8]), "=r"(r[dxi][9]),
                          "=r"(r[dxi][10]), "=r"(r[dxi][11]), "=r"(r[dxi][12]), "=r"(r[dxi][13]), "=r"(r[dxi][14]),
                          "=r"(r[dxi][15])
                        : "r"(taddr));
                }
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&sh.accfree[acc]));
            if (!cols) continue;

            int b, ox0, oy0;
            tile_xy(k, b, ox0, oy0);
            const int m = quarter * 32 + lane;
            const int c = m % kNetBoxW;
            const int y = oy0 + m / kNetBoxW, x = ox0 - 1 + c;
            const bool valid = c >= 1 && c <= kNetOutW && y < H && x < Wd;
            float z[16];
#pragma unroll
            for (int e = 0; e < 16; ++e)
                z[e] = __shfl_up_sync(0xffffffffu, __uint_as_float(r[0][e]), 1, kNetBoxW) +
                       __uint_as_float(r[1][e]) +
                       __shfl_down_sync(0xffffffffu, __uint_as_float(r[2][e]), 1, kNetBoxW);
            if (!valid) continue;
            if (LAST) {
                if (half == 0) yout[((long)b * H + y) * Wd + x] = z[0] + bv[0];
            } else {
                uint32_t v[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) v[e] = pack_bf16(gelu_f(z[2 * e] + bv[2 * e]), gelu_f(z[2 * e + 1] + bv[2 * e + 1]));
                const uint4 lo = make_uint4(v[0], v[1], v[2], v[3]), hi = make_uint4(v[4], v[5], v[6], v[7]);
                // the pixel and its copies in the frame
                const long img = (long)b * (H + 2) * fw;
                const int wy = y == 0 ? H + 1 : (y == H - 1 ? 0 : -1);
                const int wx = x == 0 ? Wd + 1 : (x == Wd - 1 ? 0 : -1);
                auto put = [&](int fy, int fx) {
                    uint4* p = reinterpret_cast<uint4*>(out + (img + fy * fw + fx) * 32 + half * 16);
                    p[0] = lo;
                    p[1] = hi;
                };
                put(y + 1, x + 1);
                if (wy >= 0) put(wy, x + 1);
                if (wx >= 0) put(y + 1, wx);
                if (wy >= 0 && wx >= 0) put(wy, wx);
            }
        }
        // this layer's stores are read by the next layer's TMA (async proxy)
        asm volatile("fence.proxy.async.global;\n" ::: "memory");
    }
    irun = i0 + nk;
}

__global__ void __launch_bounds__(kNetThreads, 1) k_net_fwd(const __grid_constant__ CUtensorMap m_in,
                                                          const __grid_constant__ CUtensorMap m_a0,
                                                          const __grid_constant__ CUtensorMap m_a1, NetArgs a) {
    extern __shared__ __align__(1024) unsigned char net_smem[];
    __shared__ NetShared sh;
    const uint32_t sraw = smem_u32(net_smem);
    const uint32_t sbase = (sraw + 1023u) & ~1023u;
    unsigned char* gbase = net_smem + (sbase - sraw);
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == kNetMmaWarp) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&sh.tmem)),
                     "r"(kNetTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < kNetSlots; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&sh.full[s])) : "memory");
        }
        for (int s = 0; s < kNetAcc; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&sh.mmad[s])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(&sh.accfree[s])),
                         "r"(kNetEpiWarps / kNetGroups)
                         : "memory");
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        sh.abort = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");

    int irun = 0, nbar = 0;
    auto barrier = [&]() {
        __syncthreads();
        ++nbar;
        const bool skip = a.stall && nbar == 1 && blockIdx.x == 0;   // host-injected fault (tests)
        if (tid == 0 && !sh.abort && !skip && !net_grid_sync(a.bar, (unsigned int)nbar * gridDim.x)) {
            sh.abort = 1;
            atomicOr(a.err, 4u);
        }
        __syncthreads();
    };
    net_layer<16, 32, false>(&m_in, a.W[0], a.bias[0], a.act[0], nullptr, a, sh, gbase, sbase, irun);
    barrier();
    net_layer<32, 32, false>(&m_a0, a.W[1], a.bias[1], a.act[1], nullptr, a, sh, gbase, sbase, irun);
    barrier();
    net_layer<32, 32, false>(&m_a1, a.W[2], a.bias[2], a.act[0], nullptr, a, sh, gbase, sbase, irun);
    barrier();
    net_layer<32, 32, false>(&m_a0, a.W[3], a.bias[3], a.act[1], nullptr, a, sh, gbase, sbase, irun);
    barrier();
    net_layer<32, 32, false>(&m_a1, a.W[4], a.bias[4], a.act[0], nullptr, a, sh, gbase, sbase, irun);
    barrier();
    net_layer<32, 16, true>(&m_a0, a.W[5], a.bias[5], nullptr, a.y, a, sh, gbase, sbase, irun);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == kNetMmaWarp)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(sh.tmem), "r"(kNetTmemCols)
                     : "memory");
}

// Framed copy of B images [B][H][Wd][16] (the layer-1 input written
// unframed): one thread per framed pixel and 16-byte half.
__global__ void k_frame16(const __nv_bfloat16* __restrict__ x, int B, int H, int Wd, __nv_bfloat16* xf) {
    const long fw = Wd + 2, fh = H + 2;
    const long n = (long)B * fh * fw * 2;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int q = (int)(i & 1);
        long p = i >> 1;
        const int fx = (int)(p % fw);
        p /= fw;
        const int fy = (int)(p % fh);
        const long b = p / fh;
        const int yy = fy == 0 ? H - 1 : (fy == H + 1 ? 0 : fy - 1);
        const int xx = fx == 0 ? Wd - 1 : (fx == Wd + 1 ? 0 : fx - 1);
        reinterpret_cast<uint4*>(xf)[i] =
            reinterpret_cast<const uint4*>(x)[((b * H + yy) * Wd + xx) * 2 + q];
    }
}

// Weight and bias gradient of one layer on the FP32 pipes:
//   dW[co, t, ci] = sum_p dz[p, co] in[p + off_t, ci],   db[co] = sum_p dz[p, co].
// A CTA walks image rows, staging dz of the row and in of rows y-1, y, y+1 in
// shared memory; thread = (co, group of CI/8 input channels); partial sums per
// CTA go to part[blockIdx] and are summed by k_reduce_rows in a fixed order.
template <int CI, int CO>
__global__ void __launch_bounds__(256) k_conv_wgrad(const __nv_bfloat16* __restrict__ dz,
                                                    const __nv_bfloat16* __restrict__ in, float* part, int B,
                                                    int H, int Wd) {
    constexpr int CIG = CI / 8;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16* rows = reinterpret_cast<__nv_bfloat16*>(smem_raw);   // [3][Wd][CI]
    __nv_bfloat16* drow = rows + 3 * Wd * CI;                            // [Wd][CO]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int co = warp * 4 + (lane >> 3);
    const int ci0 = (lane & 7) * CIG;
    float acc[9][CIG];
    float accb = 0.f;
#pragma unroll
    for (int t = 0; t < 9; ++t)
#pragma unroll
        for (int c = 0; c < CIG; ++c) acc[t][c] = 0.f;
    const long HW = (long)H * Wd;
    for (int r = blockIdx.x; r < B * H; r += gridDim.x) {
        const int b = r / H, y = r - (r / H) * H;
        __syncthreads();
        for (int i = threadIdx.x; i < 3 * Wd * CI / 2; i += blockDim.x) {
            const int e = 2 * i;
            const int rr = e / (Wd * CI);
            const int rem = e - rr * Wd * CI;
            int yy = y + rr - 1;
            yy += (yy < 0) ? H : ((yy >= H) ? -H : 0);
            reinterpret_cast<uint32_t*>(rows)[i] = ld32(in + ((long)b * HW + (long)yy * Wd) * CI + rem);
        }
        for (int i = threadIdx.x; i < Wd * CO / 2; i += blockDim.x)
            reinterpret_cast<uint32_t*>(drow)[i] = ld32(dz + ((long)b * HW + (long)y * Wd) * CO + 2 * i);
        __syncthreads();
        for (int x = 0; x < Wd; ++x) {
            const float d = __bfloat162float(drow[x * CO + co]);
            accb += d;
#pragma unroll
            for (int t = 0; t < 9; ++t) {
                int xs = x + (t % 3) - 1;
                xs += (xs < 0) ? Wd : ((xs >= Wd) ? -Wd : 0);
                const __nv_bfloat16* v = rows + ((t / 3) * Wd + xs) * CI + ci0;
#pragma unroll
                for (int c = 0; c < CIG; c += 2) {
                    const float2 f = unpack_bf16(ld32(v + c));
                    acc[t][c] += d * f.x;
                    acc[t][c + 1] += d * f.y;
                }
            }
        }
    }
    const long stride = (long)CO * 9 * CI + CO;
    float* out = part + (long)blockIdx.x * stride;
#pragma unroll
    for (int t = 0; t < 9; ++t)
#pragma unroll
        for (int c = 0; c < CIG; ++c) out[((long)co * 9 + t) * CI + ci0 + c] = acc[t][c];
    if ((lane & 7) == 0) out[(long)CO * 9 * CI + co] = accb;
}

// Weight and bias gradient of one layer on the tcgen05 tensor cores:
//   dW[co, t, ci] = sum_p dz[p, co] in[p + off_t, ci],   db[co] = sum_p dz[p, co],
// a contraction over the pixels.  A persistent CTA accumulates, over its
// 128-pixel tiles (8 x 16), one FP32 matrix in tensor memory
//   D[(dy, co), (dx, ci | 1)] += sum over the tile's halo pixels q of
//                                 dz_tile[q - (dy, 0), co] * in[q + (0, dx), ci]
// with K = the 160 pixels of the 10 x 16 halo box (one MMA of K = 16 per box
// row).  Both operands are MN-major (channels contiguous, as the images are
// stored), read through 32/64-byte swizzled descriptors straight from TMA
// boxes:
//   A (M = 128): the tile's dz box in rows 2..9 of a zeroed 24-row buffer Z;
//     row block dy (32 or 16 channels wide) starts at Z row 1 - dy, so the
//     blocks dy = +1, 0, -1 are whole-row offsets (the rest of M is unused);
//     the zero rows keep every pixel outside the tile out of the sum.
//   B (N = 3 CI + 16): the three dx-shifted boxes of the input halo (the
//     boxes of k_conv_tc, circular edges rewritten the same way) side by
//     side, then a block of ones -- whose column gives db from the dy = 0 rows.
// Thread 0 keeps the boxes of the next two tiles loading into three slots
// while the MMAs of this one run; at the end the 4 warps read D (warp w: lanes 32 w ..)
// and write the CTA's partial sums in k_conv_wgrad's layout for k_reduce_rows.
// Every wait is bounded (bit 4 of *err, the partial sums are then zero).
template <int CI, int CO>
struct WgTile {
    static constexpr int ROWI = CI * 2;                       // bytes of an input pixel
    static constexpr int ROWD = CO * 2;                       // bytes of a dz pixel
    static constexpr int BOXI = (kConvTY + 2) * kConvTX * ROWI;   // one input box, 10 x 16
    static constexpr int BOXD = kConvTY * kConvTX * ROWD;         // the dz box, 8 x 16
    // rows of Z the MMAs read: M / CO row blocks (4 or 8) + 10 - 1
    static constexpr int ZROWS = CO == 32 ? 16 : 24;
    static constexpr int ZB = ZROWS * kConvTX * ROWD;
    static constexpr int SLOT = 4 * BOXI + ZB;                // 3 dx boxes, the ones block, Z
    static constexpr int NSLOT = 3;
    static constexpr int N = 3 * CI + 16;
    static constexpr size_t SMEM = NSLOT * (size_t)SLOT + 1024;
    static_assert(BOXI % 1024 == 0 && ZB % 1024 == 0, "operands stay aligned to the swizzle pattern");
};

// Shared-memory descriptor of an MN-major operand with the 32- or 64-byte
// swizzle (ROWB = the swizzle width): lbo = byte step between ROWB-wide
// blocks along M (or N), sbo = byte step between groups of 8 rows along K.
template <int ROWB>
__device__ __forceinline__ uint64_t umma_desc_mn(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)(ROWB == 64 ? 4 : 6) << 61;
    return d;
}

template <int CI, int CO>
__global__ void __launch_bounds__(128, 1) k_wgrad_tc(const __grid_constant__ CUtensorMap tin,
                                                     const __grid_constant__ CUtensorMap tdz,
                                                     const __nv_bfloat16* __restrict__ in, float* part, int B,
                                                     int H, int Wd, unsigned int* err) {
    using WT = WgTile<CI, CO>;
    constexpr int ROWI = WT::ROWI, ROWD = WT::ROWD, KGI = CI / 8;
    constexpr int TMEM_COLS = 128;
    extern __shared__ __align__(1024) unsigned char wg_smem[];
    const uint32_t sraw = smem_u32(wg_smem);
    const uint32_t sbase = (sraw + 1023u) & ~1023u;
    unsigned char* gbase = wg_smem + (sbase - sraw);
    constexpr int NS = WT::NSLOT;
    __shared__ __align__(8) uint64_t mbar_full[NS];
    __shared__ __align__(8) uint64_t mbar_mma[NS];
    __shared__ uint32_t tmem_base;
    __shared__ int s_ok;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tiles_x = (Wd + kConvTX - 1) / kConvTX;
    const int tiles_img = tiles_x * ((H + kConvTY - 1) / kConvTY);
    const int ntiles = tiles_img * B;
    const int nk = (int)blockIdx.x < ntiles ? (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x : 0;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    // zero the Z buffers, ones in the ones blocks (their layout does not matter)
    for (int s = 0; s < NS; ++s) {
        uint4* z = reinterpret_cast<uint4*>(gbase + s * WT::SLOT + 4 * WT::BOXI);
        for (int i = tid; i < WT::ZB / 16; i += blockDim.x) z[i] = make_uint4(0, 0, 0, 0);
        uint4* o = reinterpret_cast<uint4*>(gbase + s * WT::SLOT + 3 * WT::BOXI);
        const uint32_t one2 = 0x3F803F80u;   // two BF16 ones
        for (int i = tid; i < WT::BOXI / 16; i += blockDim.x) o[i] = make_uint4(one2, one2, one2, one2);
    }
    if (tid == 0) {
        for (int s = 0; s < NS; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar_full[s])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar_mma[s])) : "memory");
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        s_ok = 1;
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = tmem_base;

    auto tile_xy = [&](int k, int& b, int& tx0, int& ty0) {
        const int tile = (int)blockIdx.x + k * (int)gridDim.x;
        b = tile / tiles_img;
        const int tl = tile - b * tiles_img;
        tx0 = (tl % tiles_x) * kConvTX;
        ty0 = (tl / tiles_x) * kConvTY;
    };
    auto issue_loads = [&](int k) {
        const int s = k % NS;
        int b, tx0, ty0;
        tile_xy(k, b, tx0, ty0);
        const uint32_t slot = sbase + s * WT::SLOT;
        const uint32_t bar = smem_u32(&mbar_full[s]);   // slot s, (k / NS)-th use
        mbar_expect_tx(bar, (uint32_t)(3 * WT::BOXI + WT::BOXD));
#pragma unroll
        for (int d = 0; d < 3; ++d) tma_load_4d(slot + d * WT::BOXI, &tin, 0, tx0 + d - 1, ty0 - 1, b, bar);
        tma_load_4d(slot + 4 * WT::BOXI + 2 * kConvTX * ROWD, &tdz, 0, tx0, ty0, b, bar);
    };
    // thread 0's bookkeeping: loads issued up to tile kl, MMAs committed up to km
    int kl = 0, km = -1;
    if (tid == 0)
        while (kl < nk && kl < NS - 1) issue_loads(kl++);

    for (int k = 0; k < nk; ++k) {
        const int s = k % NS;
        const uint32_t par = (uint32_t)(k / NS) & 1u;
        int b, tx0, ty0;
        tile_xy(k, b, tx0, ty0);
        if (tid == 0 && !mbar_wait_bounded(smem_u32(&mbar_full[s]), par)) s_ok = 0;
        __syncthreads();
        if (!s_ok) break;
        // circular wrap at the image edges: rewrite the zero-filled positions
        // of the three input boxes (as k_conv_tc)
        if (tx0 == 0 || ty0 == 0 || tx0 + kConvTX >= Wd || ty0 + kConvTY >= H) {
            (void)mbar_try_wait(smem_u32(&mbar_full[s]), par);
            const long img = (long)b * H * Wd;
            unsigned char* slotp = gbase + s * WT::SLOT;
            for (int i = tid; i < 3 * (kConvTY + 2) * kConvTX * KGI; i += blockDim.x) {
                const int q = i % KGI;
                int r = i / KGI;
                const int c = r % kConvTX;
                r /= kConvTX;
                const int hr = r % (kConvTY + 2);
                const int d = r / (kConvTY + 2);
                int yy = ty0 + hr - 1, xx = tx0 + c + d - 1;
                if (yy >= 0 && yy < H && xx >= 0 && xx < Wd) continue;
                yy += yy < 0 ? H : 0;
                yy -= yy >= H ? H : 0;
                yy -= yy >= H ? H : 0;
                xx += xx < 0 ? Wd : 0;
                xx -= xx >= Wd ? Wd : 0;
                xx -= xx >= Wd ? Wd : 0;
                const uint4 v = *reinterpret_cast<const uint4*>(in + (img + (long)yy * Wd + xx) * CI + q * 8);
                const int row = hr * kConvTX + c;
                const int pq = ROWI == 64 ? (q ^ ((row >> 1) & 3)) : (q ^ ((row >> 2) & 1));
                *reinterpret_cast<uint4*>(slotp + d * WT::BOXI + row * ROWI + pq * 16) = v;
            }
        }
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        if (tid == 0) {
            constexpr uint32_t idesc = umma_idesc_bf16(128, WT::N) | (1u << 15) | (1u << 16);   // A, B MN-major
            const uint32_t slot = sbase + s * WT::SLOT;
            const uint32_t z = slot + 4 * WT::BOXI;
#pragma unroll 1
            for (int rho = 0; rho < kConvTY + 2; ++rho) {
                const uint64_t ad = umma_desc_mn<ROWD>(z + rho * kConvTX * ROWD, kConvTX * ROWD, 8 * ROWD);
                const uint64_t bd = umma_desc_mn<ROWI>(slot + rho * kConvTX * ROWI, WT::BOXI, 8 * ROWI);
                const uint32_t acc = (k > 0 || rho > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             smem_u32(&mbar_mma[s]))
                         : "memory");
            km = k;
            // tile k + NS - 1 goes to the slot of tile k - 1 once the MMAs
            // that read it are done
            if (kl < nk) {
                if (k >= 1 && !mbar_wait_bounded(smem_u32(&mbar_mma[(k - 1) % NS]), (uint32_t)((k - 1) / NS) & 1u))
                    s_ok = 0;
                else
                    issue_loads(kl++);
            }
        }
    }
    // every MMA complete before the accumulator is read
    if (tid == 0 && km >= 0 && !mbar_wait_bounded(smem_u32(&mbar_mma[km % NS]), (uint32_t)(km / NS) & 1u)) s_ok = 0;
    if (tid == 0 && !s_ok) {
        atomicOr(err, 4u);
        for (int k = km + 1; k < kl; ++k) mbar_wait_bounded(smem_u32(&mbar_full[k % NS]), (uint32_t)(k / NS) & 1u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");

    // D row m = (block i = m / CO: dy = 1 - i, channel co = m % CO); column
    // n = (dx + 1) CI + ci, the ones column 3 CI
    const long stride = (long)CO * 9 * CI + CO;
    float* out = part + (long)blockIdx.x * stride;
    const int m = warp * 32 + lane;
    const int blk = m / CO, co = m % CO;
    const bool ok = s_ok && nk > 0;
#pragma unroll 1
    for (int c0 = 0; c0 < WT::N; c0 += 16) {
        uint32_t r[16];
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        if (blk > 2) continue;
        const int dy = 1 - blk;
#pragma unroll
        for (int e = 0; e < 16; ++e) {
            const int n = c0 + e;
            const float v = ok ? __uint_as_float(r[e]) : 0.0f;
            if (n < 3 * CI) {
                const int dx = n / CI - 1, ci = n % CI;
                const int t = (dy + 1) * 3 + (dx + 1);
                out[((long)co * 9 + t) * CI + ci] = v;
            } else if (n == 3 * CI && dy == 0) {
                out[(long)CO * 9 * CI + co] = v;
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

// Launch k_wgrad_tc over B images with up to `grid` CTAs (one per SM); the
// partial sums of the CTAs launched go to part[0 .. returned count).
template <int CI, int CO>
cudaError_t launch_wgrad(const __nv_bfloat16* dz, const __nv_bfloat16* in, float* part, int B, int H, int Wd,
                         int grid, unsigned int* err, cudaStream_t st, int* nblk) {
    CUtensorMap mi, md;
    cudaError_t e = conv_tensor_map<CI>(&mi, in, B, H, Wd);
    if (e == cudaSuccess) e = conv_tensor_map<CO>(&md, dz, B, H, Wd, kConvTY);
    if (e != cudaSuccess) return e;
    const long ntiles = (long)((Wd + kConvTX - 1) / kConvTX) * ((H + kConvTY - 1) / kConvTY) * B;
    *nblk = (int)std::max<long>(1, std::min<long>(ntiles, grid));
    return launch_k(k_wgrad_tc<CI, CO>, *nblk, 128, WgTile<CI, CO>::SMEM, st, false, mi, md, in, part, B, H, Wd,
                    err);
}

// out[i] = sum_b part[b * n + i], b in order.
__global__ void k_reduce_rows(const float* __restrict__ part, int nblk, long n, float* out) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < nblk; ++b) s += part[(long)b * n + i];
        out[i] = s;
    }
}

// MSE loss: dz[p, 0] = 2 (y - t) / n, other channels 0; per-block loss sums.
__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ tgt, long P, float inv_n,
                      __nv_bfloat16* dz, int CO, double* part) {
    __shared__ double red[256];
    double s = 0.0;
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < P; p += (long)gridDim.x * blockDim.x) {
        const float e = y[p] - tgt[p];
        s += (double)e * e;
        dz[p * CO] = __float2bfloat16_rn(2.f * e * inv_n);
        for (int c = 1; c < CO; ++c) dz[p * CO + c] = __float2bfloat16_rn(0.f);
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// Adam (Kingma & Ba 2015) on the FP32 master parameters.
__global__ void k_adam(float* p, const float* __restrict__ g, float* m, float* v, long n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// BF16 working copies of one layer: W[co][t][ci] and W^T[ci][t][co].
__global__ void k_refresh(const float* __restrict__ Wm, int CO, int CI, __nv_bfloat16* W, __nv_bfloat16* WT) {
    const int n = CO * 9 * CI;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int co = i / (9 * CI), rem = i - co * 9 * CI, t = rem / CI, ci = rem - t * CI;
        const __nv_bfloat16 h = __float2bfloat16_rn(Wm[i]);
        W[i] = h;
        WT[((long)ci * 9 + t) * CO + co] = h;
    }
}

// Network input (channels 0, 1 = w / (a s0), psi / (a s1); 2..15 = 0) and
// target (Pi / (a^2 s2)) of a batch, from dataset samples idx[b] (FP32
// [HW][3]); a = amp[idx[b]] is the sample's rms vorticity (1 when amp is
// null).  Dividing by a and a^2 makes the closure equivariant to the
// amplitude of the flow: Pi is quadratic in w.
__global__ void k_pack(const float* __restrict__ data, const float* __restrict__ amp,
                       const int* __restrict__ idx, int B, long HW, float r0, float r1, float r2,
                       __nv_bfloat16* x, float* tgt) {
    const long P = (long)B * HW;
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < P; p += (long)gridDim.x * blockDim.x) {
        const long b = p / HW, q = p - b * HW;
        const float* s = data + ((long)idx[b] * HW + q) * 3;
        const float ia = amp ? 1.f / amp[idx[b]] : 1.f;
        uint32_t* xr = reinterpret_cast<uint32_t*>(x + p * 16);
        xr[0] = pack_bf16(s[0] * r0 * ia, s[1] * r1 * ia);
        for (int c = 1; c < 8; ++c) xr[c] = 0u;
        if (tgt) tgt[p] = s[2] * r2 * ia * ia;
    }
}

// sum of squares of n doubles, accumulated into *acc (zeroed by the caller)
template <typename T>
__global__ void k_sumsq(const T* __restrict__ v, long n, double* acc) {
    __shared__ double red[256];
    double s = 0.0;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        s += (double)v[i] * (double)v[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(acc, red[0]);
}

// amp[i] = sqrt(*acc / n)
__global__ void k_store_rms(const double* __restrict__ acc, long n, float* amp) { *amp = (float)sqrt(*acc / (double)n); }

// ---- LES-side kernels ---------------------------------------------------

// Sharp filter DNS -> LES (|k| <= K_les) of w (LES state in FP64 or FP32),
// and N_dns = -(dW + nu k^2 w) when dWd is given.
template <typename VTL>
__global__ void k_filter_gather(Dims dd, Dims dl, const double2* __restrict__ wd, const double2* __restrict__ dWd,
                                double nu_d, VTL* wl, double2* pil) {
    const int total = dl.KX * dl.KY;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int kx = i / dl.KY, jc = i - kx * dl.KY;
        const int ky = ky_of_jc(dl, jc);
        double2 w = make_double2(0.0, 0.0), nl = make_double2(0.0, 0.0);
        if (kx * kx + ky * ky <= dl.K * dl.K) {
            const int jd = ky >= 0 ? ky : ky + dd.KY;
            const size_t od = (size_t)kx * dd.ldS + jd;
            w = wd[od];
            if (dWd) {
                const double2 d = dWd[od];
                const double visc = nu_d * (double)(kx * kx + ky * ky);
                nl = make_double2(-(d.x + visc * w.x), -(d.y + visc * w.y));
            }
        }
        const size_t ol = (size_t)kx * dl.ldS + jc;
        wl[ol].x = w.x;
        wl[ol].y = w.y;
        if (pil) pil[ol] = nl;
    }
}

// Pi = N_dns_filtered - N_les with N_les = -(dW_les + nu k^2 w): pi += dW + nu k^2 w.
__global__ void k_pi_finish(Dims dl, const double2* __restrict__ w, const double2* __restrict__ dW, double nu,
                            double2* pi) {
    const int total = dl.KX * dl.KY;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int kx = i / dl.KY, jc = i - kx * dl.KY;
        const int ky = ky_of_jc(dl, jc);
        const size_t o = (size_t)kx * dl.ldS + jc;
        if (kx * kx + ky * ky > dl.K * dl.K) {
            pi[o] = make_double2(0.0, 0.0);
            continue;
        }
        const double visc = nu * (double)(kx * kx + ky * ky);
        const double2 a = pi[o], d = dW[o], ww = w[o];
        pi[o] = make_double2(a.x + d.x + visc * ww.x, a.y + d.y + visc * ww.y);
    }
}

// Physical rows of two spectral fields X, Y (half-spectral rows, Y may be
// null): one inverse FFT of X + iY per row, real part -> ox, imaginary -> oy.
template <typename T>
__global__ void __launch_bounds__(512) k_xinv_phys2(Dims d, const typename Vec<T>::t* __restrict__ X,
                                                    const typename Vec<T>::t* __restrict__ Y,
                                                    const typename Vec<T>::t* __restrict__ tw, int G, T* ox, T* oy) {
    using VT = typename Vec<T>::t;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    VT* bufs = reinterpret_cast<VT*>(smem_raw);
    const int g = threadIdx.x / d.Tg;
    const int lane = threadIdx.x - g * d.Tg;
    const int y = blockIdx.x * G + g;
    const bool active = y < d.M;
    VT* Z = bufs + (size_t)g * d.M;
    const int yy = active ? y : 0;
    if (Y) {
        build_pair(Z, X + (size_t)yy * d.ldI, Y + (size_t)yy * d.ldI, d, lane, active);
    } else {
        // X alone: Z = X Hermitian-extended
        for (int n = lane; n < d.M; n += d.Tg) {
            VT z = mk<VT>((T)0, (T)0);
            if (active) {
                const VT* Xr = X + (size_t)yy * d.ldI;
                if (n == 0) z = mk<VT>(__ldcg(&Xr[0]).x, (T)0);
                else if (n <= d.K) z = __ldcg(&Xr[n]);
                else if (n >= d.M - d.K) {
                    const VT a = __ldcg(&Xr[d.M - n]);
                    z = mk<VT>(a.x, -a.y);
                }
            }
            Z[n] = z;
        }
    }
    fft_run<true>(Z, d, lane, tw);
    if (active)
        for (int n = lane; n < d.M; n += d.Tg) {
            ox[(size_t)y * d.M + n] = Z[n].x;
            if (oy) oy[(size_t)y * d.M + n] = Z[n].y;
        }
}

// Dataset sample (FP32 [HW][3]) from physical w, psi, Pi (FP64).
__global__ void k_to_sample(const double* __restrict__ w, const double* __restrict__ p, const double* __restrict__ pi,
                            long HW, float* out) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < HW; i += (long)gridDim.x * blockDim.x) {
        out[3 * i] = (float)w[i];
        out[3 * i + 1] = (float)p[i];
        out[3 * i + 2] = (float)pi[i];
    }
}

// ---- closure terms of n LES runs of one grid (blockIdx.y = run) ----------
// Per-run pointers; the same layout for both precisions.
template <typename T>
struct LesRun {
    const typename Vec<T>::t* S0;
    typename Vec<T>::t* I0;
    typename Vec<T>::t* I1;
    typename Vec<T>::t* I2;
    typename Vec<T>::t* src;   // -Pi^ (compact layout)
    double* part;   // sums of |w^|^2 per column tile of k_cl_yinv; part[nparts]: their total
};

// Sum of the nparts partial sums by one warp in a fixed order (lane l adds
// part[l], part[l + 32], ... in turn, then an xor butterfly over the lanes):
// every lane returns the same value, on every call.
__device__ __forceinline__ double warp_ordered_sum(const double* __restrict__ part, int nparts, int lane) {
    double s = 0.0;
    for (int i = lane; i < nparts; i += 32) s += __ldcg(&part[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

// K1 of (w, psi): inverse y-pass of every run's state.  The CTAs of the w
// field also sum |w^|^2 over their columns (kx > 0 twice: the other half of
// the spectrum), which by Parseval is the mean of w^2 over the collocation
// grid (the inverse transform is unnormalised); per thread, then a fixed
// tree over the CTA, into part[column tile].
template <typename T>
__global__ void __launch_bounds__(512) k_cl_yinv(Dims d, const LesRun<T>* __restrict__ runs,
                                                  const double* __restrict__ rk2,
                                                  const typename Vec<T>::t* __restrict__ tw, int G) {
    using VT = typename Vec<T>::t;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    pdl_enter();
    const LesRun<T>& R = runs[blockIdx.y];
    FieldSet fs{};
    fs.nf = 2;
    fs.op[0] = OP_W;
    fs.op[1] = OP_PSI;
    fs.out[0] = R.I0;
    fs.out[1] = R.I1;
    yinv_body<T>(d, R.S0, rk2, fs, tw, G, blockIdx.x, reinterpret_cast<VT*>(smem_raw));
    const int ncg = (d.KX + G - 1) / G;
    if ((int)blockIdx.x >= ncg) return;   // the psi field's CTAs (uniform per CTA)
    const int kx0 = blockIdx.x * G;
    const int gtot = min(G, d.KX - kx0);
    const DivBy byKY(d.KY);
    double s = 0.0;
    for (int idx = threadIdx.x; idx < gtot * d.KY; idx += blockDim.x) {
        const int gg = byKY(idx);
        const int kx = kx0 + gg;
        const VT v = __ldcg(&R.S0[(size_t)kx * d.ldS + (idx - gg * d.KY)]);
        const double m = (double)v.x * (double)v.x + (double)v.y * (double)v.y;
        s += kx > 0 ? 2.0 * m : m;
    }
    // tree over the CTA in the (now free) FFT buffers: G*M*vsz >= 8 B per thread
    double* red = reinterpret_cast<double*>(smem_raw);
    __syncthreads();
    red[threadIdx.x] = s;
    __syncthreads();
    int w = 1;
    while (w < (int)blockDim.x) w <<= 1;
    for (w >>= 1; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w && threadIdx.x + w < blockDim.x) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) R.part[blockIdx.x] = red[0];
}

// Physical rows of w and psi (one inverse FFT of W + i PSI per row), written
// as the network input of every run: (w / (a s0), psi / (a s1)) in BF16, a =
// rms w of the run from the nparts sums of k_cl_yinv (their total, the mean
// of w^2, is kept in part[nparts] for k_cl_xfwd).  Only channels 0 and 1 of
// x are written: channels 2..15 of the input buffer are zero from its
// allocation on, and every writer of it keeps them so.  framed: x holds
// images with the one-pixel circular frame of the fused forward ([M + 2]^2
// pixels, pixel (y, n) at (y + 1, n + 1)), the border pixels written into the
// frame as well.
template <typename T>
__global__ void __launch_bounds__(512) k_cl_xinv(Dims d, const LesRun<T>* __restrict__ runs,
                                                  const typename Vec<T>::t* __restrict__ tw, int G, int nparts,
                                                  float r0, float r1, __nv_bfloat16* x, int framed) {
    using VT = typename Vec<T>::t;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double s_ia;
    pdl_enter();
    const LesRun<T>& R = runs[blockIdx.y];
    if (threadIdx.x < 32) {
        const double mean = warp_ordered_sum(R.part, nparts, threadIdx.x);
        if (threadIdx.x == 0) {
            s_ia = 1.0 / sqrt(mean);
            if (blockIdx.x == 0) R.part[nparts] = mean;
        }
    }
    VT* bufs = reinterpret_cast<VT*>(smem_raw);
    const int g = threadIdx.x / d.Tg;
    const int lane = threadIdx.x - g * d.Tg;
    const int y = blockIdx.x * G + g;
    const bool active = y < d.M;
    const int yy = active ? y : 0;
    VT* Z = bufs + (size_t)g * d.M;
    build_pair(Z, R.I0 + (size_t)yy * d.ldI, R.I1 + (size_t)yy * d.ldI, d, lane, active);
    fft_run<true>(Z, d, lane, tw);   // begins with a barrier: s_ia is visible after it
    const T a0 = (T)((double)r0 * s_ia), a1 = (T)((double)r1 * s_ia);
    if (active && !framed) {
        uint32_t* xr = reinterpret_cast<uint32_t*>(x + ((size_t)blockIdx.y * d.M + y) * (size_t)d.M * 16);
        for (int n = lane; n < d.M; n += d.Tg) {
            const VT z = Z[n];
            xr[(size_t)n * 8] = pack_bf16((float)(z.x * a0), (float)(z.y * a1));
        }
    } else if (active) {
        const size_t fw = (size_t)d.M + 2;
        const int wy = y == 0 ? d.M + 1 : (y == d.M - 1 ? 0 : -1);
        uint32_t* xr = reinterpret_cast<uint32_t*>(x + ((size_t)blockIdx.y * fw + y + 1) * fw * 16);
        uint32_t* xw = reinterpret_cast<uint32_t*>(x + ((size_t)blockIdx.y * fw + (wy < 0 ? 0 : wy)) * fw * 16);
        for (int n = lane; n < d.M; n += d.Tg) {
            const VT z = Z[n];
            const uint32_t v = pack_bf16((float)(z.x * a0), (float)(z.y * a1));
            const int wx = n == 0 ? d.M + 1 : (n == d.M - 1 ? 0 : -1);
            xr[(size_t)(n + 1) * 8] = v;
            if (wx >= 0) xr[(size_t)wx * 8] = v;
            if (wy >= 0) {
                xw[(size_t)(n + 1) * 8] = v;
                if (wx >= 0) xw[(size_t)wx * 8] = v;
            }
        }
    }
}

// Network output -> -Pi on the grid (scale a^2 y, scale = -s2), forward x-FFT
// of row pairs into the half-spectral rows I2.
template <typename T>
__global__ void __launch_bounds__(512) k_cl_xfwd(Dims d, const LesRun<T>* __restrict__ runs, int nparts,
                                                  const float* __restrict__ Y, double scale,
                                                  const typename Vec<T>::t* __restrict__ tw, int G, T xscale) {
    using VT = typename Vec<T>::t;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    pdl_enter();
    const LesRun<T>& R = runs[blockIdx.y];
    const long HW = (long)d.M * d.M;
    const T s = (T)(scale * __ldcg(&R.part[nparts]));
    VT* bufs = reinterpret_cast<VT*>(smem_raw);
    const int g = threadIdx.x / d.Tg;
    const int lane = threadIdx.x - g * d.Tg;
    const int p = blockIdx.x * G + g;
    const bool active = p < d.M / 2;
    const int y1 = active ? 2 * p : 0;
    VT* Z = bufs + (size_t)g * d.M;
    const float* r1 = Y + (size_t)blockIdx.y * HW + (size_t)y1 * d.M;
    const float* r2 = r1 + d.M;
    for (int n = lane; n < d.M; n += d.Tg)
        Z[n] = active ? mk<VT>(s * (T)r1[n], s * (T)r2[n]) : mk<VT>((T)0, (T)0);
    fft_run<false>(Z, d, lane, tw);
    extract_pair(Z, R.I2 + (size_t)y1 * d.ldI, R.I2 + (size_t)(y1 + 1) * d.ldI, d, lane, active, xscale);
}

// Forward y-FFT of the columns of I2 with Truncate into src; modes with
// |k|^2 < kmin2 (the closure's band) are zero.
template <typename T>
__global__ void __launch_bounds__(512) k_cl_ystore(Dims d, const LesRun<T>* __restrict__ runs,
                                                    const typename Vec<T>::t* __restrict__ tw, int G,
                                                    double kmin2) {
    using VT = typename Vec<T>::t;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    pdl_enter();
    const LesRun<T>& R = runs[blockIdx.y];
    VT* bufs = reinterpret_cast<VT*>(smem_raw);
    const int g = threadIdx.x / d.Tg;
    const int lane = threadIdx.x - g * d.Tg;
    const int kx0 = blockIdx.x * G;
    const int gtot = min(G, d.KX - kx0);
    const DivBy byG(G), byKY(d.KY);
    for (int idx = threadIdx.x; idx < G * d.M; idx += blockDim.x) {
        const int y = byG(idx);
        const int gg = idx - y * G;
        bufs[(size_t)gg * d.M + y] = gg < gtot ? __ldcg(&R.I2[(size_t)y * d.ldI + kx0 + gg]) : mk<VT>((T)0, (T)0);
    }
    fft_run<false>(bufs + (size_t)g * d.M, d, lane, tw);
    __syncthreads();
    for (int idx = threadIdx.x; idx < gtot * d.KY; idx += blockDim.x) {
        const int gg = byKY(idx);
        const int jc = idx - gg * d.KY;
        const int kx = kx0 + gg;
        const int ky = ky_of_jc(d, jc);
        const int n = jc <= d.K ? jc : ky + d.M;
        VT v = bufs[(size_t)gg * d.M + n];
        const int k2 = kx * kx + ky * ky;
        if (k2 > d.K * d.K || (double)k2 < kmin2) v = mk<VT>((T)0, (T)0);
        R.src[(size_t)kx * d.ldS + jc] = v;
    }
}

// Moments of the dataset after the per-sample amplitude normalisation:
// per-block sums of (w/a)^2, (psi/a)^2, (Pi/a^2)^2.
__global__ void k_moments(const float* __restrict__ data, const float* __restrict__ amp, long HW, long n,
                          double* part) {
    __shared__ double red[3][256];
    double s0 = 0, s1 = 0, s2 = 0;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double ia = 1.0 / (double)amp[i / HW];
        const double a = data[3 * i] * ia, b = data[3 * i + 1] * ia, c = data[3 * i + 2] * ia * ia;
        s0 += a * a;
        s1 += b * b;
        s2 += c * c;
    }
    red[0][threadIdx.x] = s0;
    red[1][threadIdx.x] = s1;
    red[2][threadIdx.x] = s2;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int c = 0; c < 3; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int c = 0; c < 3; ++c) part[3 * blockIdx.x + c] = red[c][0];
}

}  // namespace s2d

using namespace s2d;

struct s2d_cnn {
    int device = 0;
    int H = 0, Wd = 0, maxB = 0;
    cudaStream_t stream = nullptr;
    long poff[kLayers + 1];            // offsets of each layer's (W, b) in the padded FP32 arrays
    long nparam_pad = 0;
    float *master = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16 *Wb[kLayers] = {}, *WTb[kLayers] = {};
    __nv_bfloat16* X0 = nullptr;
    __nv_bfloat16 *Z[kLayers - 1] = {}, *A[kLayers - 1] = {};
    __nv_bfloat16 *dZ6 = nullptr, *dZa = nullptr, *dZb = nullptr;
    // s2d_cnn_keep_layer_grads: dL/dz of every hidden layer kept (else the
    // backward pass reuses two buffers)
    __nv_bfloat16* dZk[kLayers - 1] = {};
    bool keep = false;
    float *Y = nullptr, *tgt = nullptr;
    float* part = nullptr;
    long part_n = 0;
    int wg_blocks = 0;
    int sms = 152;                    // SMs of the device (persistent conv grid)
    double* lpart = nullptr;
    int* idx = nullptr;
    float* data = nullptr;
    float* amp = nullptr;       // per-sample rms vorticity
    double* sumsq = nullptr;    // scratch accumulator (rms of one state)
    unsigned int* cflags = nullptr;   // bit 4: a tensor-core wait gave up (S2D_ERR_TIMEOUT)
    int data_cap = 0, data_n = 0;
    double scale[3] = {1.0, 1.0, 1.0};
    double k_min = 0.0;         // the closure term is applied only where |k| >= k_min
    long step = 0;
    // the fused inference forward (k_net_fwd): framed layer-1 input and the
    // two framed activation images, the grid barrier's arrival count
    bool fused = true;
    bool net_stall = false;     // s2d_cnn_inject_stall
    int net_grid = 0;           // resident CTAs of k_net_fwd (cooperative launch)
    __nv_bfloat16* X0f = nullptr;
    __nv_bfloat16* F[2] = {};
    unsigned int* netbar = nullptr;
};

namespace {

int cerr(int code, const char* m) { return set_error(code, m); }

#define C_CUDA(call)                                                               \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) return cerr(S2D_ERR_CUDA, cudaGetErrorString(e_));  \
    } while (0)

int nblocks(long n, int threads) { return (int)std::min<long>((n + threads - 1) / threads, 152L * 16); }

int refresh_all(s2d_cnn* c) {
    for (int l = 0; l < kLayers; ++l) {
        const int n = kCoutP[l] * 9 * kCinP[l];
        k_refresh<<<nblocks(n, 256), 256, 0, c->stream>>>(c->master + c->poff[l], kCoutP[l], kCinP[l], c->Wb[l],
                                                           c->WTb[l]);
        C_CUDA(cudaGetLastError());
    }
    return S2D_OK;
}

int ensure_net_buffers(s2d_cnn* c) {
    if (c->netbar) return S2D_OK;
    const size_t fp = (size_t)c->maxB * (c->H + 2) * (c->Wd + 2);
    C_CUDA(cudaFuncSetAttribute(k_net_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kNetSmem));
    int occ = 0;
    C_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_net_fwd, kNetThreads, kNetSmem));
    if (occ < 1) return cerr(S2D_ERR_UNSUPPORTED, "the fused network kernel does not fit on an SM");
    occ = 1;   // one CTA per SM by design (its TMEM columns, the launch bound)
    c->net_grid = occ * c->sms;
    bool ok = cudaMalloc(&c->X0f, fp * 16 * sizeof(__nv_bfloat16)) == cudaSuccess &&
              cudaMemset(c->X0f, 0, fp * 16 * sizeof(__nv_bfloat16)) == cudaSuccess &&
              cudaMalloc(&c->F[0], fp * 32 * sizeof(__nv_bfloat16)) == cudaSuccess &&
              cudaMalloc(&c->F[1], fp * 32 * sizeof(__nv_bfloat16)) == cudaSuccess &&
              cudaMalloc(&c->netbar, 64) == cudaSuccess;
    if (!ok) {
        cudaFree(c->X0f);
        cudaFree(c->F[0]);
        cudaFree(c->F[1]);
        cudaFree(c->netbar);
        c->X0f = c->F[0] = c->F[1] = nullptr;
        c->netbar = nullptr;
        return cerr(S2D_ERR_NOMEM, "cudaMalloc failed (fused network buffers)");
    }
    return S2D_OK;
}

// Inference forward of B images in one launch (k_net_fwd); the layer-1 input
// is in X0f already framed (k_cl_xinv writes it so) or framed here from X0.
int forward_fused(s2d_cnn* c, int B, bool input_framed) {
    int r = ensure_net_buffers(c);
    if (r != S2D_OK) return r;
    const int H = c->H, Wd = c->Wd;
    if (!input_framed) {
        k_frame16<<<nblocks((long)B * (H + 2) * (Wd + 2) * 2, 256), 256, 0, c->stream>>>(c->X0, B, H, Wd, c->X0f);
        C_CUDA(cudaGetLastError());
    }
    CUtensorMap m_in, m_a0, m_a1;
    C_CUDA(conv_tensor_map<16>(&m_in, c->X0f, B, H + 2, Wd + 2));
    C_CUDA(conv_tensor_map<32>(&m_a0, c->F[0], B, H + 2, Wd + 2));
    C_CUDA(conv_tensor_map<32>(&m_a1, c->F[1], B, H + 2, Wd + 2));
    NetArgs a{};
    for (int l = 0; l < kLayers; ++l) {
        a.W[l] = c->Wb[l];
        a.bias[l] = c->master + c->poff[l] + (long)kCoutP[l] * 9 * kCinP[l];
    }
    a.act[0] = c->F[0];
    a.act[1] = c->F[1];
    a.y = c->Y;
    a.bar = c->netbar;
    a.err = c->cflags;
    a.B = B;
    a.H = H;
    a.Wd = Wd;
    a.stall = c->net_stall ? 1 : 0;
    const long ntiles = (long)((Wd + kNetOutW - 1) / kNetOutW) * ((H + kNetOutH - 1) / kNetOutH) * B;
    const int grid = (int)std::min<long>(ntiles, c->net_grid);
    C_CUDA(cudaMemsetAsync(c->netbar, 0, sizeof(unsigned int), c->stream));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kNetThreads);
    cfg.dynamicSmemBytes = kNetSmem;
    cfg.stream = c->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    C_CUDA(cudaLaunchKernelEx(&cfg, k_net_fwd, m_in, m_a0, m_a1, a));
    return S2D_OK;
}

// forward of the batch in X0 (B images); the pre-activations z are kept only
// when a backward pass follows.  Without them the fused kernel runs (unless
// switched off by s2d_cnn_set_fused).
int forward(s2d_cnn* c, int B, bool keep_z, bool pdl = false) {
    if (!keep_z && c->fused) return forward_fused(c, B, false);
    const float* bias[kLayers];
    for (int l = 0; l < kLayers; ++l) bias[l] = c->master + c->poff[l] + (long)kCoutP[l] * 9 * kCinP[l];
    C_CUDA((launch_conv<16, 32, 1, 0>(c->X0, c->Wb[0], bias[0], nullptr, keep_z ? c->Z[0] : nullptr, c->A[0],
                                      nullptr, B, c->H, c->Wd, c->cflags, c->sms, c->stream, pdl)));
    for (int l = 1; l < kLayers - 1; ++l)
        C_CUDA((launch_conv<32, 32, 1, 0>(c->A[l - 1], c->Wb[l], bias[l], nullptr, keep_z ? c->Z[l] : nullptr,
                                          c->A[l], nullptr, B, c->H, c->Wd, c->cflags, c->sms, c->stream, pdl)));
    C_CUDA((launch_conv<32, 16, 1, 1>(c->A[kLayers - 2], c->Wb[kLayers - 1], bias[kLayers - 1], nullptr, nullptr,
                                      nullptr, c->Y, B, c->H, c->Wd, c->cflags, c->sms, c->stream, pdl)));
    return S2D_OK;
}

// loss of the batch (targets in tgt) and, with grads, the full backward pass
int loss_backward(s2d_cnn* c, int B, bool grads, double* loss) {
    const long P = (long)B * c->H * c->Wd;
    const int lb = 256;
    k_mse<<<lb, 256, 0, c->stream>>>(c->Y, c->tgt, P, 1.0f / (float)P, c->dZ6, 16, c->lpart);
    C_CUDA(cudaGetLastError());
    std::vector<double> lp(lb);
    C_CUDA(cudaMemcpyAsync(lp.data(), c->lpart, sizeof(double) * lb, cudaMemcpyDeviceToHost, c->stream));
    if (grads) {
        // S2D_WGRAD_FP32=1: the weight gradient on the FP32 pipes (comparisons)
        const char* wv = std::getenv("S2D_WGRAD_FP32");
        const bool wgrad_fp32 = wv && wv[0] && wv[0] != '0';
        const __nv_bfloat16* dz = c->dZ6;
        __nv_bfloat16* bufs[2] = {c->dZa, c->dZb};
        for (int l = kLayers - 1; l >= 0; --l) {
            const __nv_bfloat16* in = l == 0 ? c->X0 : c->A[l - 1];
            const int CI = kCinP[l], CO = kCoutP[l];
            const long n = (long)CO * 9 * CI + CO;
            int nblk = c->wg_blocks;
            if (wgrad_fp32) {   // the FP32-pipe kernel, for comparisons
                const size_t sm = (size_t)(3 * c->Wd * CI + c->Wd * CO) * sizeof(__nv_bfloat16);
                if (CI == 16)
                    k_conv_wgrad<16, 32><<<nblk, 32 * 8, sm, c->stream>>>(dz, in, c->part, B, c->H, c->Wd);
                else if (CO == 16)
                    k_conv_wgrad<32, 16><<<nblk, 16 * 8, sm, c->stream>>>(dz, in, c->part, B, c->H, c->Wd);
                else
                    k_conv_wgrad<32, 32><<<nblk, 32 * 8, sm, c->stream>>>(dz, in, c->part, B, c->H, c->Wd);
                C_CUDA(cudaGetLastError());
            } else {
                const int g = std::min(c->wg_blocks, c->sms);
                if (CI == 16)
                    C_CUDA((launch_wgrad<16, 32>(dz, in, c->part, B, c->H, c->Wd, g, c->cflags, c->stream, &nblk)));
                else if (CO == 16)
                    C_CUDA((launch_wgrad<32, 16>(dz, in, c->part, B, c->H, c->Wd, g, c->cflags, c->stream, &nblk)));
                else
                    C_CUDA((launch_wgrad<32, 32>(dz, in, c->part, B, c->H, c->Wd, g, c->cflags, c->stream, &nblk)));
            }
            k_reduce_rows<<<nblocks(n, 256), 256, 0, c->stream>>>(c->part, nblk, n, c->grad + c->poff[l]);
            C_CUDA(cudaGetLastError());
            if (l > 0) {
                __nv_bfloat16* out = c->keep ? c->dZk[l - 1] : bufs[l & 1];
                if (CO == 16)
                    C_CUDA((launch_conv<16, 32, -1, 2>(dz, c->WTb[l], nullptr, c->Z[l - 1], out, nullptr, nullptr,
                                                       B, c->H, c->Wd, c->cflags, c->sms, c->stream)));
                else
                    C_CUDA((launch_conv<32, 32, -1, 2>(dz, c->WTb[l], nullptr, c->Z[l - 1], out, nullptr, nullptr,
                                                       B, c->H, c->Wd, c->cflags, c->sms, c->stream)));
                dz = out;
            }
        }
    }
    C_CUDA(cudaStreamSynchronize(c->stream));
    double s = 0.0;
    for (double x : lp) s += x;
    if (loss) *loss = s / (double)P;
    return S2D_OK;
}

int adam_step(s2d_cnn* c, double lr) {
    c->step += 1;
    const double b1 = 0.9, b2 = 0.999;
    const float c1 = (float)(1.0 - std::pow(b1, (double)c->step));
    const float c2 = (float)(1.0 - std::pow(b2, (double)c->step));
    k_adam<<<nblocks(c->nparam_pad, 256), 256, 0, c->stream>>>(c->master, c->grad, c->m, c->v, c->nparam_pad,
                                                                (float)lr, (float)b1, (float)b2, 1e-8f, c1, c2);
    C_CUDA(cudaGetLastError());
    return refresh_all(c);
}

// logical (Cout x 9 x Cin + Cout per layer) <-> padded layout
void logical_to_padded(const float* lg, std::vector<float>& pad, const long* poff) {
    long o = 0;
    for (int l = 0; l < kLayers; ++l) {
        for (int co = 0; co < kCout[l]; ++co)
            for (int t = 0; t < 9; ++t)
                for (int ci = 0; ci < kCin[l]; ++ci)
                    pad[poff[l] + ((long)co * 9 + t) * kCinP[l] + ci] = lg[o++];
        for (int co = 0; co < kCout[l]; ++co) pad[poff[l] + (long)kCoutP[l] * 9 * kCinP[l] + co] = lg[o++];
    }
}

void padded_to_logical(const std::vector<float>& pad, float* lg, const long* poff) {
    long o = 0;
    for (int l = 0; l < kLayers; ++l) {
        for (int co = 0; co < kCout[l]; ++co)
            for (int t = 0; t < 9; ++t)
                for (int ci = 0; ci < kCin[l]; ++ci)
                    lg[o++] = pad[poff[l] + ((long)co * 9 + t) * kCinP[l] + ci];
        for (int co = 0; co < kCout[l]; ++co) lg[o++] = pad[poff[l] + (long)kCoutP[l] * 9 * kCinP[l] + co];
    }
}

long logical_count() {
    long n = 0;
    for (int l = 0; l < kLayers; ++l) n += (long)kCout[l] * 9 * kCin[l] + kCout[l];
    return n;
}

uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}

int upload_host_batch(s2d_cnn* c, const float* x, const float* target, int B) {
    // host (omega, psi) pairs -> temporary dataset slots at the end of a
    // private staging area, then the packing kernel
    const long HW = (long)c->H * c->Wd;
    std::vector<float> s((size_t)B * HW * 3);
    for (long i = 0; i < (long)B * HW; ++i) {
        s[3 * i] = x[2 * i];
        s[3 * i + 1] = x[2 * i + 1];
        s[3 * i + 2] = target ? target[i] : 0.f;
    }
    float* tmp = nullptr;
    int* idx = nullptr;
    C_CUDA(cudaMalloc(&tmp, s.size() * sizeof(float)));
    C_CUDA(cudaMalloc(&idx, sizeof(int) * B));
    std::vector<int> id(B);
    for (int b = 0; b < B; ++b) id[b] = b;
    C_CUDA(cudaMemcpyAsync(tmp, s.data(), s.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    C_CUDA(cudaMemcpyAsync(idx, id.data(), sizeof(int) * B, cudaMemcpyHostToDevice, c->stream));
    k_pack<<<nblocks((long)B * HW, 256), 256, 0, c->stream>>>(tmp, nullptr, idx, B, HW, (float)(1.0 / c->scale[0]),
                                                              (float)(1.0 / c->scale[1]), (float)(1.0 / c->scale[2]),
                                                              c->X0, c->tgt);
    cudaError_t e = cudaGetLastError();
    cudaStreamSynchronize(c->stream);
    cudaFree(tmp);
    cudaFree(idx);
    if (e != cudaSuccess) return cerr(S2D_ERR_CUDA, cudaGetErrorString(e));
    return S2D_OK;
}

// Physical w (and psi) of a spectral field of the handle on its collocation grid.
template <typename T>
int state_to_phys(s2d_handle* h, const void* S, T* ow, T* op, bool with_psi) {
    using VT = typename Vec<T>::t;
    FieldSet fs{};
    fs.nf = with_psi ? 2 : 1;
    fs.op[0] = OP_W;
    fs.op[1] = OP_PSI;
    fs.out[0] = h->I[0];
    fs.out[1] = h->I[1];
    C_CUDA(Kern<T>::yinv(h->d, S, h->rk2, fs, h->tw, h->stream, h->L_yinv));
    const Launch& L = h->L_xrow;
    k_xinv_phys2<T><<<(h->d.M + L.G - 1) / L.G, L.threads, L.smem, h->stream>>>(
        h->d, (const VT*)h->I[0], with_psi ? (const VT*)h->I[1] : nullptr, (const VT*)h->tw, L.G, ow,
        with_psi ? op : nullptr);
    C_CUDA(cudaGetLastError());
    return S2D_OK;
}

int ensure_les_buffers(s2d_handle* h) {
    static std::atomic<bool> attr[64];  // per device, set once the attributes are (a second setter only repeats them)
    if (h->device >= 0 && h->device < 64 && !attr[h->device]) {
        C_CUDA(cudaFuncSetAttribute(k_xinv_phys2<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, h->max_smem));
        C_CUDA(cudaFuncSetAttribute(k_xinv_phys2<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, h->max_smem));
        const void* fns[] = {(const void*)k_cl_yinv<double>, (const void*)k_cl_yinv<float>,
                             (const void*)k_cl_xinv<double>, (const void*)k_cl_xinv<float>,
                             (const void*)k_cl_xfwd<double>, (const void*)k_cl_xfwd<float>,
                             (const void*)k_cl_ystore<double>, (const void*)k_cl_ystore<float>};
        for (const void* f : fns)
            C_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, h->max_smem));
        attr[h->device] = true;
    }
    const size_t cs = (size_t)h->d.KX * h->d.ldS * sizeof(double2);
    if (!h->pi) C_CUDA(cudaMalloc(&h->pi, cs));
    if (!h->Sdw) C_CUDA(cudaMalloc(&h->Sdw, cs));
    if (!h->phys) C_CUDA(cudaMalloc(&h->phys, 3 * (size_t)h->d.M * h->d.M * sizeof(double)));
    return S2D_OK;
}

// LesRun table of n runs followed by M + 1 doubles per run: the partial
// sums of k_cl_yinv (one per column tile, at most M) and their total.
int closure_table_impl(s2d_handle* const* runs, int n, void** tab) {
    const s2d_handle* h0 = runs[0];
    const size_t pstride = (size_t)h0->d.M + 1;
    const size_t head = (size_t)n * sizeof(LesRun<double>);
    void* t = nullptr;
    C_CUDA(cudaMalloc(&t, head + (size_t)n * pstride * sizeof(double)));
    std::vector<LesRun<double>> rows(n);
    for (int i = 0; i < n; ++i) {
        s2d_handle* h = runs[i];
        LesRun<double>& R = rows[i];
        R.S0 = (const double2*)h->S0;
        // a handle stepped with its closure on a second stream has its own
        // transform buffers; the batch (one stream) uses the handles' I
        char* ib = (char*)h->cl_I;
        R.I0 = (double2*)(ib ? ib : h->I[0]);
        R.I1 = (double2*)(ib ? ib + h->Ibytes : h->I[1]);
        R.I2 = (double2*)(ib ? ib + 2 * h->Ibytes : h->I[2]);
        // phys holds M*M 8-byte elements per field; FP32 runs use the front half
        R.src = (double2*)h->src;
        R.part = (double*)((char*)t + head) + (size_t)i * pstride;
    }
    const cudaError_t e = cudaMemcpy(t, rows.data(), head, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(t);
        return cerr(S2D_ERR_CUDA, cudaGetErrorString(e));
    }
    *tab = t;
    return S2D_OK;
}

template <typename T>
int closure_terms_t(s2d_cnn* c, s2d_handle* const* runs, int n, const void* tab, cudaStream_t st) {
    using VT = typename Vec<T>::t;
    const s2d_handle* h0 = runs[0];
    const Dims& d = h0->d;
    const LesRun<T>* R = (const LesRun<T>*)tab;
    const Launch& Ly = h0->L_yinv;
    const Launch& Lx = h0->L_xrow;
    const Launch& Ls = h0->L_ystore;
    const int nparts = (d.KX + Ly.G - 1) / Ly.G;   // k_cl_yinv's column tiles of the w field
    const VT* tw = (const VT*)h0->tw;
    const bool pdl = Ly.pdl;
    C_CUDA(launch_k(k_cl_yinv<T>, dim3(2 * nparts, n), Ly.threads, Ly.smem, st, pdl, d, R, h0->rk2, tw, Ly.G));
    const bool fused = c->fused;
    C_CUDA(launch_k(k_cl_xinv<T>, dim3((d.M + Lx.G - 1) / Lx.G, n), Lx.threads, Lx.smem, st, pdl, d, R, tw, Lx.G,
                    nparts, (float)(1.0 / c->scale[0]), (float)(1.0 / c->scale[1]), fused ? c->X0f : c->X0,
                    (int)fused));
    // the network runs on the caller's stream: borrow it for the forward pass
    cudaStream_t saved = c->stream;
    c->stream = st;
    const int r = fused ? forward_fused(c, n, true) : forward(c, n, false, pdl);
    c->stream = saved;
    if (r != S2D_OK) return r;
    C_CUDA(launch_k(k_cl_xfwd<T>, dim3((d.M / 2 + Lx.G - 1) / Lx.G, n), Lx.threads, Lx.smem, st, pdl, d, R,
                    nparts, (const float*)c->Y, -c->scale[2], tw, Lx.G, (T)(0.5 / ((double)d.M * (double)d.M))));
    C_CUDA(launch_k(k_cl_ystore<T>, dim3((d.KX + Ls.G - 1) / Ls.G, n), Ls.threads, Ls.smem, st, pdl, d, R, tw,
                    Ls.G, c->k_min * c->k_min));
    return S2D_OK;
}

template <typename T>
int physical_pair_t(s2d_handle* h, const void* S, int opA, int opB, void* outA, void* outB) {
    using VT = typename Vec<T>::t;
    int r = ensure_les_buffers(h);
    if (r != S2D_OK) return r;
    FieldSet fs{};
    fs.nf = outB ? 2 : 1;
    fs.op[0] = opA;
    fs.op[1] = opB;
    fs.out[0] = h->I[0];
    fs.out[1] = h->I[1];
    C_CUDA(Kern<T>::yinv(h->d, S, h->rk2, fs, h->tw, h->stream, h->L_yinv));
    const Launch& L = h->L_xrow;
    k_xinv_phys2<T><<<(h->d.M + L.G - 1) / L.G, L.threads, L.smem, h->stream>>>(
        h->d, (const VT*)h->I[0], outB ? (const VT*)h->I[1] : nullptr, (const VT*)h->tw, L.G, (T*)outA, (T*)outB);
    C_CUDA(cudaGetLastError());
    return S2D_OK;
}

}  // namespace

int s2d::ensure_closure_buffers(s2d_handle* h) {
    int r = ensure_les_buffers(h);
    if (r != S2D_OK) return r;
    if (!h->src) C_CUDA(cudaMalloc(&h->src, (size_t)h->d.KX * h->d.ldS * h->vsz));
    return S2D_OK;
}

int s2d::closure_table(s2d_handle* const* runs, int n, void** tab) { return closure_table_impl(runs, n, tab); }

int s2d::closure_terms(s2d_cnn* c, s2d_handle* const* runs, int n, const void* tab, cudaStream_t st) {
    if (!c || !runs || n <= 0 || !tab) return cerr(S2D_ERR_INVALID, "bad closure arguments");
    if (n > c->maxB) return cerr(S2D_ERR_INVALID, "more runs than the network's batch capacity");
    return runs[0]->prec == S2D_FP64 ? closure_terms_t<double>(c, runs, n, tab, st)
                                     : closure_terms_t<float>(c, runs, n, tab, st);
}

int s2d::cnn_grid(const s2d_cnn* c) { return c->H; }
int s2d::cnn_max_batch(const s2d_cnn* c) { return c->maxB; }

int s2d::physical_pair(s2d_handle* h, const void* S, int opA, int opB, void* outA, void* outB) {
    return h->prec == S2D_FP64 ? physical_pair_t<double>(h, S, opA, opB, outA, outB)
                               : physical_pair_t<float>(h, S, opA, opB, outA, outB);
}

// One LES step as an executable CUDA graph: the closure term of the state at
// the start of the step on clstream, concurrently with the first stage's
// inverse y-pass and x-pass on the handle's stream; the first stage's
// epilogue (the first reader of src) waits for it.  Rebuilt by every caller,
// so that it picks up new network scales and dt.
static int les_step_graph(s2d_handle* les, double dt, cudaGraphExec_t* out) {
    if (!std::isfinite(dt)) return cerr(S2D_ERR_INVALID, "dt must be finite");
    if (!les->src || !les->les_tab || !les->clstream) return cerr(S2D_ERR_INVALID, "no closure set");
    C_CUDA(cudaSetDevice(les->device));
    C_CUDA(cudaStreamBeginCapture(les->stream, cudaStreamCaptureModeThreadLocal));
    int r = S2D_OK;
    cudaError_t ec = cudaEventRecord(les->ev_fork, les->stream);
    if (ec == cudaSuccess) ec = cudaStreamWaitEvent(les->clstream, les->ev_fork, 0);
    if (ec == cudaSuccess) {
        r = s2d::closure_terms(les->cnn, &les, 1, les->les_tab, les->clstream);
        // the join is recorded even after a failure, so that the capture can end
        ec = cudaEventRecord(les->ev_join, les->clstream);
    }
    if (ec != cudaSuccess && r == S2D_OK) r = cerr(S2D_ERR_CUDA, cudaGetErrorString(ec));
    if (r == S2D_OK) r = s2d::launch_step_sourced(les, dt, les->ev_join);
    else cudaStreamWaitEvent(les->stream, les->ev_join, 0);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(les->stream, &g);
    if (r != S2D_OK || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return r != S2D_OK ? r : cerr(S2D_ERR_CUDA, cudaGetErrorString(e));
    }
    const cudaError_t e2 = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e2 != cudaSuccess) return cerr(S2D_ERR_CUDA, cudaGetErrorString(e2));
    return S2D_OK;
}

extern "C" {

S2D_API int s2d_cnn_create(int32_t grid, int32_t max_batch, uint64_t seed, int32_t device, s2d_cnn** out) {
    if (!out || grid < 8 || max_batch < 1) return cerr(S2D_ERR_INVALID, "bad network arguments");
    // activations are indexed with 32-bit offsets (32 channels per pixel)
    if ((long long)max_batch * grid * grid * 32 >= (1LL << 31))
        return cerr(S2D_ERR_INVALID, "max_batch * grid^2 * 32 must stay below 2^31");
    *out = nullptr;
    s2d_cnn* c = new (std::nothrow) s2d_cnn();
    if (!c) return cerr(S2D_ERR_NOMEM, "host allocation failed");
    c->device = device;
    c->H = c->Wd = grid;
    c->maxB = max_batch;
    // S2D_CNN_LAYERWISE=1: gradient-free forward passes one launch per layer
    // (for comparisons; s2d_cnn_set_fused switches it per network)
    if (const char* e = std::getenv("S2D_CNN_LAYERWISE")) c->fused = e[0] == '\0' || e[0] == '0';
    auto bail = [&](int code) {
        s2d_cnn_destroy(c);
        return code;
    };
    if (cudaSetDevice(device) != cudaSuccess) return bail(cerr(S2D_ERR_CUDA, "cudaSetDevice failed"));
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(cerr(S2D_ERR_CUDA, "stream creation failed"));
    {
        static std::atomic<bool> attr[64];  // per device, set once the attributes are (a second setter only repeats them)
        if (device >= 0 && device < 64 && !attr[device]) {
            const cudaFuncAttribute A = cudaFuncAttributeMaxDynamicSharedMemorySize;
            const bool set =
                cudaFuncSetAttribute(k_conv_tc<16, 32, 1, 0>, A, (int)ConvTile<16, 32>::SMEM) == cudaSuccess &&
                cudaFuncSetAttribute(k_conv_tc<32, 32, 1, 0>, A, (int)ConvTile<32, 32>::SMEM) == cudaSuccess &&
                cudaFuncSetAttribute(k_conv_tc<32, 16, 1, 1>, A, (int)ConvTile<32, 16>::SMEM) == cudaSuccess &&
                cudaFuncSetAttribute(k_conv_tc<16, 32, -1, 2>, A, (int)ConvTile<16, 32>::SMEM) == cudaSuccess &&
                cudaFuncSetAttribute(k_conv_tc<32, 32, -1, 2>, A, (int)ConvTile<32, 32>::SMEM) == cudaSuccess;
            if (!set) return bail(cerr(S2D_ERR_CUDA, "cudaFuncSetAttribute failed"));
            attr[device] = true;
        }
    }
    long off = 0;
    for (int l = 0; l < kLayers; ++l) {
        c->poff[l] = off;
        off += (long)kCoutP[l] * 9 * kCinP[l] + kCoutP[l];
    }
    c->poff[kLayers] = off;
    c->nparam_pad = off;
    const long P = (long)max_batch * grid * grid;
    int dev_sms = 152;
    cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, device);
    c->sms = dev_sms;
    c->wg_blocks = std::max(1, std::min(2 * dev_sms, max_batch * grid));
    c->part_n = (long)c->wg_blocks * (32 * 9 * 32 + 32);
    bool ok = cudaMalloc(&c->master, off * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&c->grad, off * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&c->m, off * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&c->v, off * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&c->X0, P * 16 * sizeof(__nv_bfloat16)) == cudaSuccess &&
              cudaMemset(c->X0, 0, P * 16 * sizeof(__nv_bfloat16)) == cudaSuccess &&
              cudaMalloc(&c->dZ6, P * 16 * sizeof(__nv_bfloat16)) == cudaSuccess &&
              cudaMalloc(&c->dZa, P * 32 * sizeof(__nv_bfloat16)) == cudaSuccess &&
              cudaMalloc(&c->dZb, P * 32 * sizeof(__nv_bfloat16)) == cudaSuccess &&
              cudaMalloc(&c->Y, P * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&c->tgt, P * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&c->part, c->part_n * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&c->lpart, 256 * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&c->idx, max_batch * sizeof(int)) == cudaSuccess &&
              cudaMalloc(&c->sumsq, 64) == cudaSuccess && cudaMalloc(&c->cflags, 64) == cudaSuccess &&
              cudaMemset(c->cflags, 0, 64) == cudaSuccess;
    for (int l = 0; l < kLayers && ok; ++l) {
        const size_t n = (size_t)kCoutP[l] * 9 * kCinP[l] * sizeof(__nv_bfloat16);
        ok = cudaMalloc(&c->Wb[l], n) == cudaSuccess && cudaMalloc(&c->WTb[l], n) == cudaSuccess;
    }
    for (int l = 0; l < kLayers - 1 && ok; ++l)
        ok = cudaMalloc(&c->Z[l], P * 32 * sizeof(__nv_bfloat16)) == cudaSuccess &&
             cudaMalloc(&c->A[l], P * 32 * sizeof(__nv_bfloat16)) == cudaSuccess;
    if (!ok) return bail(cerr(S2D_ERR_NOMEM, "cudaMalloc failed"));
    // allocated here, not at first use: the first use may be inside a graph capture
    if (ensure_net_buffers(c) != S2D_OK) return bail(S2D_ERR_NOMEM);
    {
        const int smax = 3 * grid * 32 * 2 + grid * 32 * 2;
        cudaFuncSetAttribute(k_conv_wgrad<16, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
        cudaFuncSetAttribute(k_conv_wgrad<32, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
        cudaFuncSetAttribute(k_conv_wgrad<32, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
        cudaFuncSetAttribute(k_wgrad_tc<16, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)WgTile<16, 32>::SMEM);
        cudaFuncSetAttribute(k_wgrad_tc<32, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)WgTile<32, 16>::SMEM);
        cudaFuncSetAttribute(k_wgrad_tc<32, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)WgTile<32, 32>::SMEM);
    }
    // He-uniform initialisation from a seeded counter-based generator
    std::vector<float> pad(off, 0.f);
    uint64_t ctr = 0;
    for (int l = 0; l < kLayers; ++l) {
        const double bound = std::sqrt(6.0 / (9.0 * kCin[l])) * (l == kLayers - 1 ? 0.5 : 1.0);
        for (int co = 0; co < kCout[l]; ++co)
            for (int t = 0; t < 9; ++t)
                for (int ci = 0; ci < kCin[l]; ++ci) {
                    const double u = (double)(mix64(seed * 0x100000001B3ULL + (ctr++)) >> 11) * (1.0 / 9007199254740992.0);
                    pad[c->poff[l] + ((long)co * 9 + t) * kCinP[l] + ci] = (float)((2.0 * u - 1.0) * bound);
                }
    }
    if (cudaMemcpy(c->master, pad.data(), off * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(cerr(S2D_ERR_CUDA, "parameter upload failed"));
    cudaMemset(c->m, 0, off * sizeof(float));
    cudaMemset(c->v, 0, off * sizeof(float));
    cudaMemset(c->grad, 0, off * sizeof(float));
    if (refresh_all(c) != S2D_OK) return bail(S2D_ERR_CUDA);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return bail(cerr(S2D_ERR_CUDA, "setup failed"));
    *out = c;
    return S2D_OK;
}

S2D_API void s2d_cnn_destroy(s2d_cnn* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    void* ptrs[] = {c->master, c->grad, c->m, c->v, c->X0, c->dZ6, c->dZa, c->dZb, c->Y, c->tgt, c->part,
                    c->lpart, c->idx, c->data, c->amp, c->sumsq, c->cflags, c->X0f, c->F[0], c->F[1], c->netbar};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (int l = 0; l < kLayers; ++l) {
        if (c->Wb[l]) cudaFree(c->Wb[l]);
        if (c->WTb[l]) cudaFree(c->WTb[l]);
    }
    for (int l = 0; l < kLayers - 1; ++l) {
        if (c->Z[l]) cudaFree(c->Z[l]);
        if (c->A[l]) cudaFree(c->A[l]);
        if (c->dZk[l]) cudaFree(c->dZk[l]);
    }
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

S2D_API int s2d_cnn_num_params(const s2d_cnn* c) {
    if (!c) return cerr(S2D_ERR_INVALID, "null network");
    return (int)logical_count();
}

S2D_API int s2d_cnn_get_params(s2d_cnn* c, float* p) {
    if (!c || !p) return cerr(S2D_ERR_INVALID, "null argument");
    C_CUDA(cudaSetDevice(c->device));
    std::vector<float> pad(c->nparam_pad);
    C_CUDA(cudaMemcpy(pad.data(), c->master, pad.size() * sizeof(float), cudaMemcpyDeviceToHost));
    padded_to_logical(pad, p, c->poff);
    return S2D_OK;
}

S2D_API int s2d_cnn_set_params(s2d_cnn* c, const float* p) {
    if (!c || !p) return cerr(S2D_ERR_INVALID, "null argument");
    C_CUDA(cudaSetDevice(c->device));
    std::vector<float> pad(c->nparam_pad, 0.f);
    logical_to_padded(p, pad, c->poff);
    C_CUDA(cudaMemcpy(c->master, pad.data(), pad.size() * sizeof(float), cudaMemcpyHostToDevice));
    C_CUDA(cudaMemset(c->m, 0, pad.size() * sizeof(float)));
    C_CUDA(cudaMemset(c->v, 0, pad.size() * sizeof(float)));
    c->step = 0;
    const int r = refresh_all(c);
    C_CUDA(cudaStreamSynchronize(c->stream));
    return r;
}

S2D_API int s2d_cnn_set_scales(s2d_cnn* c, const double* s) {
    if (!c || !s || !(s[0] > 0) || !(s[1] > 0) || !(s[2] > 0)) return cerr(S2D_ERR_INVALID, "scales must be > 0");
    for (int i = 0; i < 3; ++i) c->scale[i] = s[i];
    return S2D_OK;
}

S2D_API int s2d_cnn_get_scales(const s2d_cnn* c, double* s) {
    if (!c || !s) return cerr(S2D_ERR_INVALID, "null argument");
    for (int i = 0; i < 3; ++i) s[i] = c->scale[i];
    return S2D_OK;
}

S2D_API int s2d_cnn_set_band(s2d_cnn* c, double k_min) {
    if (!c || !(k_min >= 0.0) || !std::isfinite(k_min)) return cerr(S2D_ERR_INVALID, "k_min must be >= 0");
    c->k_min = k_min;
    return S2D_OK;
}

S2D_API int s2d_cnn_get_band(const s2d_cnn* c, double* k_min) {
    if (!c || !k_min) return cerr(S2D_ERR_INVALID, "null argument");
    *k_min = c->k_min;
    return S2D_OK;
}

S2D_API int s2d_cnn_forward_host(s2d_cnn* c, const float* x, int32_t B, float* y) {
    if (!c || !x || !y || B < 1 || B > c->maxB) return cerr(S2D_ERR_INVALID, "bad batch");
    C_CUDA(cudaSetDevice(c->device));
    int r = upload_host_batch(c, x, nullptr, B);
    if (r != S2D_OK) return r;
    r = forward(c, B, false);
    if (r != S2D_OK) return r;
    const long P = (long)B * c->H * c->Wd;
    std::vector<float> out(P);
    C_CUDA(cudaMemcpyAsync(out.data(), c->Y, P * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    C_CUDA(cudaStreamSynchronize(c->stream));
    for (long i = 0; i < P; ++i) y[i] = (float)(out[i] * c->scale[2]);
    return s2d_cnn_status(c);
}

S2D_API int s2d_cnn_grad_host(s2d_cnn* c, const float* x, const float* target, int32_t B, float* grads,
                              double* loss) {
    if (!c || !x || !target || B < 1 || B > c->maxB) return cerr(S2D_ERR_INVALID, "bad batch");
    C_CUDA(cudaSetDevice(c->device));
    int r = upload_host_batch(c, x, target, B);
    if (r != S2D_OK) return r;
    if ((r = forward(c, B, true)) != S2D_OK) return r;
    if ((r = loss_backward(c, B, true, loss)) != S2D_OK) return r;
    if (grads) {
        std::vector<float> pad(c->nparam_pad);
        C_CUDA(cudaMemcpy(pad.data(), c->grad, pad.size() * sizeof(float), cudaMemcpyDeviceToHost));
        padded_to_logical(pad, grads, c->poff);
    }
    return s2d_cnn_status(c);
}

S2D_API int s2d_cnn_keep_layer_grads(s2d_cnn* c, int32_t keep) {
    if (!c) return cerr(S2D_ERR_INVALID, "null network");
    C_CUDA(cudaSetDevice(c->device));
    C_CUDA(cudaStreamSynchronize(c->stream));
    const size_t n = (size_t)c->maxB * c->H * c->Wd * 32 * sizeof(__nv_bfloat16);
    for (int l = 0; l < kLayers - 1; ++l) {
        if (keep && !c->dZk[l] && cudaMalloc(&c->dZk[l], n) != cudaSuccess) {
            for (int j = 0; j < kLayers - 1; ++j) {
                cudaFree(c->dZk[j]);
                c->dZk[j] = nullptr;
            }
            c->keep = false;
            return cerr(S2D_ERR_NOMEM, "cudaMalloc of the layer-gradient buffers failed");
        }
        if (!keep && c->dZk[l]) {
            cudaFree(c->dZk[l]);
            c->dZk[l] = nullptr;
        }
    }
    c->keep = keep != 0;
    return S2D_OK;
}

S2D_API int s2d_cnn_get_tensor(s2d_cnn* c, int32_t kind, int32_t layer, int32_t batch, float* out) {
    if (!c || !out || layer < 0 || layer >= kLayers || batch < 1 || batch > c->maxB)
        return cerr(S2D_ERR_INVALID, "bad tensor request");
    const __nv_bfloat16* src = nullptr;
    int ch = 32;
    if (kind == 0) {                 // the layer's input activations
        src = layer == 0 ? c->X0 : c->A[layer - 1];
        ch = kCinP[layer];
    } else if (kind == 1) {          // its pre-activation z (hidden layers)
        if (layer == kLayers - 1) return cerr(S2D_ERR_INVALID, "the output layer keeps no pre-activation");
        src = c->Z[layer];
    } else if (kind == 2) {          // dL/dz of its output
        if (layer == kLayers - 1) {
            src = c->dZ6;
            ch = kCoutP[layer];
        } else {
            if (!c->keep) return cerr(S2D_ERR_INVALID, "layer gradients are kept only after s2d_cnn_keep_layer_grads");
            src = c->dZk[layer];
        }
    } else {
        return cerr(S2D_ERR_INVALID, "kind must be 0, 1 or 2");
    }
    C_CUDA(cudaSetDevice(c->device));
    const size_t n = (size_t)batch * c->H * c->Wd * ch;
    std::vector<__nv_bfloat16> h(n);
    C_CUDA(cudaMemcpyAsync(h.data(), src, n * sizeof(__nv_bfloat16), cudaMemcpyDeviceToHost, c->stream));
    C_CUDA(cudaStreamSynchronize(c->stream));
    for (size_t i = 0; i < n; ++i) out[i] = __bfloat162float(h[i]);
    return S2D_OK;
}

S2D_API int s2d_cnn_dataset_reserve(s2d_cnn* c, int32_t capacity) {
    if (!c || capacity < 1) return cerr(S2D_ERR_INVALID, "bad capacity");
    C_CUDA(cudaSetDevice(c->device));
    if (c->data) cudaFree(c->data);
    c->data = nullptr;
    C_CUDA(cudaMalloc(&c->data, (size_t)capacity * c->H * c->Wd * 3 * sizeof(float)));
    if (c->amp) cudaFree(c->amp);
    c->amp = nullptr;
    C_CUDA(cudaMalloc(&c->amp, (size_t)capacity * sizeof(float)));
    c->data_cap = capacity;
    c->data_n = 0;
    return S2D_OK;
}

S2D_API int s2d_cnn_dataset_size(const s2d_cnn* c) {
    if (!c) return cerr(S2D_ERR_INVALID, "null network");
    return c->data_n;
}

S2D_API int s2d_cnn_dataset_stats(s2d_cnn* c, double* rms) {
    if (!c || !rms || c->data_n < 1) return cerr(S2D_ERR_INVALID, "empty dataset");
    C_CUDA(cudaSetDevice(c->device));
    const long n = (long)c->data_n * c->H * c->Wd;
    double* part = nullptr;
    C_CUDA(cudaMalloc(&part, 3 * 256 * sizeof(double)));
    k_moments<<<256, 256, 0, c->stream>>>(c->data, c->amp, (long)c->H * c->Wd, n, part);
    std::vector<double> h(3 * 256);
    cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    cudaFree(part);
    if (e != cudaSuccess) return cerr(S2D_ERR_CUDA, cudaGetErrorString(e));
    for (int k = 0; k < 3; ++k) {
        double s = 0.0;
        for (int b = 0; b < 256; ++b) s += h[3 * b + k];
        rms[k] = std::sqrt(s / (double)n);
    }
    return S2D_OK;
}

S2D_API int s2d_cnn_train_epoch(s2d_cnn* c, int32_t first, int32_t count, int32_t batch, double lr, uint64_t seed,
                                double* mean_loss) {
    if (!c || batch < 1 || batch > c->maxB || first < 0 || count < batch || first + count > c->data_n)
        return cerr(S2D_ERR_INVALID, "bad training range");
    C_CUDA(cudaSetDevice(c->device));
    std::vector<int> order(count);
    for (int i = 0; i < count; ++i) order[i] = first + i;
    for (int i = count - 1; i > 0; --i) {   // Fisher-Yates with a seeded generator
        const int j = (int)(mix64(seed * 1315423911ULL + (uint64_t)i) % (uint64_t)(i + 1));
        std::swap(order[i], order[j]);
    }
    const long HW = (long)c->H * c->Wd;
    double tot = 0.0;
    int nb = 0;
    for (int s = 0; s + batch <= count; s += batch) {
        C_CUDA(cudaMemcpyAsync(c->idx, order.data() + s, sizeof(int) * batch, cudaMemcpyHostToDevice, c->stream));
        k_pack<<<nblocks((long)batch * HW, 256), 256, 0, c->stream>>>(
            c->data, c->amp, c->idx, batch, HW, (float)(1.0 / c->scale[0]), (float)(1.0 / c->scale[1]),
            (float)(1.0 / c->scale[2]), c->X0, c->tgt);
        C_CUDA(cudaGetLastError());
        int r = forward(c, batch, true);
        double l = 0.0;
        if (r == S2D_OK) r = loss_backward(c, batch, true, &l);
        if (r == S2D_OK) r = adam_step(c, lr);
        if (r != S2D_OK) return r;
        tot += l;
        ++nb;
    }
    C_CUDA(cudaStreamSynchronize(c->stream));
    if (mean_loss) *mean_loss = nb ? tot / nb : 0.0;
    return s2d_cnn_status(c);
}

S2D_API int s2d_cnn_eval(s2d_cnn* c, int32_t first, int32_t count, double* mean_loss) {
    if (!c || first < 0 || count < 1 || first + count > c->data_n) return cerr(S2D_ERR_INVALID, "bad range");
    C_CUDA(cudaSetDevice(c->device));
    const long HW = (long)c->H * c->Wd;
    double tot = 0.0;
    int nb = 0;
    for (int s = 0; s < count; s += c->maxB) {
        const int B = std::min(c->maxB, count - s);
        std::vector<int> id(B);
        for (int b = 0; b < B; ++b) id[b] = first + s + b;
        C_CUDA(cudaMemcpyAsync(c->idx, id.data(), sizeof(int) * B, cudaMemcpyHostToDevice, c->stream));
        k_pack<<<nblocks((long)B * HW, 256), 256, 0, c->stream>>>(c->data, c->amp, c->idx, B, HW,
                                                                  (float)(1.0 / c->scale[0]),
                                                                  (float)(1.0 / c->scale[1]),
                                                                  (float)(1.0 / c->scale[2]), c->X0, c->tgt);
        int r = forward(c, B, false);
        double l = 0.0;
        if (r == S2D_OK) r = loss_backward(c, B, false, &l);
        if (r != S2D_OK) return r;
        tot += l * B;
        nb += B;
    }
    if (mean_loss) *mean_loss = tot / nb;
    return s2d_cnn_status(c);
}

S2D_API int s2d_cnn_set_fused(s2d_cnn* c, int32_t on) {
    if (!c) return cerr(S2D_ERR_INVALID, "null network");
    c->fused = on != 0;
    return S2D_OK;
}

S2D_API int s2d_cnn_inject_stall(s2d_cnn* c, int32_t on) {
    if (!c) return cerr(S2D_ERR_INVALID, "null network");
    c->net_stall = on != 0;
    return S2D_OK;
}

S2D_API int s2d_cnn_status(s2d_cnn* c) {
    if (!c) return cerr(S2D_ERR_INVALID, "null network");
    C_CUDA(cudaSetDevice(c->device));
    unsigned int f = 0;
    C_CUDA(cudaMemcpyAsync(&f, c->cflags, sizeof(f), cudaMemcpyDeviceToHost, c->stream));
    C_CUDA(cudaMemsetAsync(c->cflags, 0, sizeof(f), c->stream));
    C_CUDA(cudaStreamSynchronize(c->stream));
    if (f & 4u) return cerr(S2D_ERR_TIMEOUT, "a tensor-core completion wait of the network gave up");
    return S2D_OK;
}

S2D_API int s2d_filter_state(s2d_handle* dns, s2d_handle* les) {
    if (!dns || !les) return cerr(S2D_ERR_INVALID, "null handle");
    if (dns->prec != S2D_FP64) return cerr(S2D_ERR_UNSUPPORTED, "filtering needs an FP64 DNS handle");
    if (les->d.K > dns->d.K) return cerr(S2D_ERR_INVALID, "the LES grid must be coarser than the DNS grid");
    C_CUDA(cudaSetDevice(dns->device));
    C_CUDA(cudaStreamSynchronize(les->stream));
    const int total = les->d.KX * les->d.KY;
    if (les->prec == S2D_FP64)
        k_filter_gather<double2><<<nblocks(total, 256), 256, 0, dns->stream>>>(
            dns->d, les->d, (const double2*)dns->S0, nullptr, 0.0, (double2*)les->S0, nullptr);
    else
        k_filter_gather<float2><<<nblocks(total, 256), 256, 0, dns->stream>>>(
            dns->d, les->d, (const double2*)dns->S0, nullptr, 0.0, (float2*)les->S0, nullptr);
    C_CUDA(cudaGetLastError());
    C_CUDA(cudaStreamSynchronize(dns->stream));
    return S2D_OK;
}

S2D_API int s2d_subgrid_flux(s2d_handle* dns, s2d_handle* les, double* pi_host) {
    if (!dns || !les) return cerr(S2D_ERR_INVALID, "null handle");
    if (dns->prec != S2D_FP64 || les->prec != S2D_FP64) return cerr(S2D_ERR_UNSUPPORTED, "needs FP64 handles");
    if (les->d.K > dns->d.K) return cerr(S2D_ERR_INVALID, "the LES grid must be coarser than the DNS grid");
    C_CUDA(cudaSetDevice(dns->device));
    int r = ensure_les_buffers(les);
    if (r != S2D_OK) return r;
    // N_dns: the DNS right-hand side of its current state
    const size_t cs = (size_t)dns->d.KX * dns->d.ldS * dns->vsz;
    if (!dns->Sdw) C_CUDA(cudaMalloc(&dns->Sdw, cs));
    {
        FieldSet fs{};
        fs.nf = 2;
        fs.op[0] = OP_U;
        fs.op[1] = OP_V;
        fs.out[0] = dns->I[0];
        fs.out[1] = dns->I[1];
        if (dns->ph.form != S2D_NL_BASDEVANT) return cerr(S2D_ERR_UNSUPPORTED, "DNS must use the Basdevant form");
        C_CUDA(Kern<double>::yinv(dns->d, dns->S0, dns->rk2, fs, dns->tw, dns->stream, dns->L_yinv));
        C_CUDA(Kern<double>::xpass_bas(dns->d, dns->I[0], dns->I[1], dns->tw, dns->stream, dns->L_xrow));
        C_CUDA(Kern<double>::yfwd_rk3(dns->d, dns->I[0], dns->I[1], dns->S0, dns->S1, dns->Sdw, nullptr, 0, 0.0,
                                      dns->ph, dns->tw, dns->flags, dns->stream, dns->L_yfwd));
    }
    C_CUDA(cudaStreamSynchronize(les->stream));
    const int total = les->d.KX * les->d.KY;
    k_filter_gather<double2><<<nblocks(total, 256), 256, 0, dns->stream>>>(dns->d, les->d, (const double2*)dns->S0,
                                                                   (const double2*)dns->Sdw, dns->ph.nu,
                                                                   (double2*)les->S0, (double2*)les->pi);
    C_CUDA(cudaGetLastError());
    C_CUDA(cudaStreamSynchronize(dns->stream));
    // N_les of the filtered state
    {
        FieldSet fs{};
        fs.nf = 2;
        fs.op[0] = OP_U;
        fs.op[1] = OP_V;
        fs.out[0] = les->I[0];
        fs.out[1] = les->I[1];
        C_CUDA(Kern<double>::yinv(les->d, les->S0, les->rk2, fs, les->tw, les->stream, les->L_yinv));
        C_CUDA(Kern<double>::xpass_bas(les->d, les->I[0], les->I[1], les->tw, les->stream, les->L_xrow));
        Phys ph = les->ph;
        ph.alpha = 0.0;
        ph.fk = 0;
        C_CUDA(Kern<double>::yfwd_rk3(les->d, les->I[0], les->I[1], les->S0, les->S1, les->Sdw, nullptr, 0, 0.0, ph,
                                      les->tw, les->flags, les->stream, les->L_yfwd));
        k_pi_finish<<<nblocks(total, 256), 256, 0, les->stream>>>(les->d, (const double2*)les->S0,
                                                                   (const double2*)les->Sdw, ph.nu, (double2*)les->pi);
        C_CUDA(cudaGetLastError());
    }
    if (pi_host) {
        double* d = nullptr;
        const size_t rb = (size_t)les->grid.cISize * les->grid.nyG * 2 * sizeof(double);
        C_CUDA(cudaMalloc(&d, rb));
        C_CUDA(Kern<double>::compact_to_ref(les->d, les->pi, les->grid.cISize, d, nullptr, les->stream));
        C_CUDA(cudaMemcpyAsync(pi_host, d, rb, cudaMemcpyDeviceToHost, les->stream));
        cudaStreamSynchronize(les->stream);
        cudaFree(d);
    }
    C_CUDA(cudaStreamSynchronize(les->stream));
    return S2D_OK;
}

S2D_API int s2d_cnn_dataset_add(s2d_cnn* c, s2d_handle* les) {
    if (!c || !les || !les->pi) return cerr(S2D_ERR_INVALID, "no subgrid flux computed for this LES handle");
    if (les->d.M != c->H) return cerr(S2D_ERR_INVALID, "network grid differs from the LES collocation grid");
    if (c->data_n >= c->data_cap) return cerr(S2D_ERR_INVALID, "dataset full");
    C_CUDA(cudaSetDevice(c->device));
    const long HW = (long)les->d.M * les->d.M;
    if (les->prec != S2D_FP64) return cerr(S2D_ERR_UNSUPPORTED, "training data needs an FP64 LES handle");
    double* pw = (double*)les->phys;
    double* pp = pw + HW;
    double* ppi = pw + 2 * HW;
    int r = state_to_phys<double>(les, les->S0, pw, pp, true);
    if (r == S2D_OK) r = state_to_phys<double>(les, les->pi, ppi, (double*)nullptr, false);
    if (r != S2D_OK) return r;
    k_to_sample<<<nblocks(HW, 256), 256, 0, les->stream>>>(pw, pp, ppi, HW, c->data + (size_t)c->data_n * HW * 3);
    C_CUDA(cudaGetLastError());
    C_CUDA(cudaMemsetAsync(c->sumsq, 0, sizeof(double), les->stream));
    k_sumsq<double><<<1, 256, 0, les->stream>>>(pw, HW, c->sumsq);   // one block: deterministic
    k_store_rms<<<1, 1, 0, les->stream>>>(c->sumsq, HW, c->amp + c->data_n);
    C_CUDA(cudaGetLastError());
    C_CUDA(cudaStreamSynchronize(les->stream));
    c->data_n += 1;
    return S2D_OK;
}

S2D_API int s2d_les_set_closure(s2d_handle* les, s2d_cnn* c) {
    if (!les) return cerr(S2D_ERR_INVALID, "null handle");
    if (c && les->d.M != c->H) return cerr(S2D_ERR_INVALID, "network grid differs from the LES collocation grid");
    C_CUDA(cudaSetDevice(les->device));
    if (c) {
        int r = s2d::ensure_closure_buffers(les);
        if (r != S2D_OK) return r;
        if (!les->cl_I) C_CUDA(cudaMalloc(&les->cl_I, 3 * les->Ibytes));
        if (!les->clstream) C_CUDA(cudaStreamCreateWithFlags(&les->clstream, cudaStreamNonBlocking));
        if (!les->ev_fork) C_CUDA(cudaEventCreateWithFlags(&les->ev_fork, cudaEventDisableTiming));
        if (!les->ev_join) C_CUDA(cudaEventCreateWithFlags(&les->ev_join, cudaEventDisableTiming));
        if (!les->les_tab) {
            r = closure_table_impl(&les, 1, &les->les_tab);
            if (r != S2D_OK) return r;
        }
    } else if (les->src) {
        C_CUDA(cudaStreamSynchronize(les->stream));
        cudaFree(les->src);
        les->src = nullptr;
        cudaFree(les->les_tab);
        les->les_tab = nullptr;
        cudaFree(les->cl_I);
        les->cl_I = nullptr;
    }
    les->cnn = c;
    return S2D_OK;
}

S2D_API int s2d_les_closure_term(s2d_handle* les) {
    if (!les || !les->cnn || !les->src || !les->les_tab) return cerr(S2D_ERR_INVALID, "no closure set");
    C_CUDA(cudaSetDevice(les->device));
    return s2d::closure_terms(les->cnn, &les, 1, les->les_tab, les->stream);
}

S2D_API int s2d_les_integrate_steps(s2d_handle* les, int32_t n, double dt) {
    if (!les || n < 0) return cerr(S2D_ERR_INVALID, "bad argument");
    if (!les->cnn) return s2d_integrate_steps(les, n, dt);
    if (n == 0) return S2D_OK;
    cudaGraphExec_t x = nullptr;
    const int r = les_step_graph(les, dt, &x);
    if (r != S2D_OK) return r;
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < n && e == cudaSuccess; ++i) e = cudaGraphLaunch(x, les->stream);
    cudaGraphExecDestroy(x);
    if (e != cudaSuccess) return cerr(S2D_ERR_CUDA, cudaGetErrorString(e));
    return S2D_OK;
}

S2D_API int s2d_les_time_steps(s2d_handle* les, int32_t n, double dt, double* ms) {
    if (!les || n <= 0 || !ms) return cerr(S2D_ERR_INVALID, "bad argument");
    if (!les->cnn) return cerr(S2D_ERR_INVALID, "no closure set");
    cudaGraphExec_t x = nullptr;
    int r = les_step_graph(les, dt, &x);
    if (r != S2D_OK) return r;
    cudaEvent_t a = nullptr, b = nullptr;
    cudaError_t e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    if (e == cudaSuccess) e = cudaStreamSynchronize(les->stream);
    if (e == cudaSuccess) e = cudaEventRecord(a, les->stream);
    for (int i = 0; i < n && e == cudaSuccess; ++i) e = cudaGraphLaunch(x, les->stream);
    if (e == cudaSuccess) e = cudaEventRecord(b, les->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    float f = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&f, a, b);
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    cudaGraphExecDestroy(x);
    if (e != cudaSuccess) return cerr(S2D_ERR_CUDA, cudaGetErrorString(e));
    *ms = f;
    return S2D_OK;
}

}  // extern "C"
