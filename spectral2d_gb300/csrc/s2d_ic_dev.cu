// s2d_ic_dev.cu -- the reproducible turbulent initial condition on the device.
//
// SetTurbulentVelocity / FourierVelocity (src/SetIC.F90:125-151, :175-364)
// with the same three stated changes as the host generator
// s2d_turbulent_ic_host (s2d_ic.cpp): a counter-based phase per (seed, kx,
// ky), a Hermitian kx = 0 column, and omega scaled so that ComputeSpectrum's
// TKE equals the requested value.  Four kernels on the handle's stream:
//
//   1. k_ic_shell_count: the shell mode counts of :295-354, a histogram over
//      every mode of the reference's (cISize, nyG) array with Hermitian
//      weights 1 (kx = 0 or kxMG) or 2 (:316-323); per-CTA counts in shared
//      memory, then integer atomics (exact, so order-independent);
//   2. k_ic_modes: per retained mode of the compact layout, the amplitude
//      sqrt(E(|k|)), the phase, u = -a ky/|k|, v = a kx/|k| (:252-261), the
//      shell normalisation (:351-352) and omega = i kx v - i ky u
//      (src/Spectral.F90:624-647), in FP64 with every operation rounded on
//      its own (no contraction), in the host generator's order; plus each
//      CTA's partial TKE sum (src/Analysis.F90:370-448: |u|^2 + |v|^2 =
//      k^2 |psi|^2 per mode, half weight on kx = 0);
//   3. k_ic_total: the partial sums added in a fixed order, the scale
//      sqrt(tke / TKE);
//   4. k_ic_store: the scaled omega into the state in the handle's
//      precision.
//
// The shell of a mode is round(|k|) (the bin edges 0, 0.5, 1.5, ...,
// kIntMax + 0.1 of BinarySearch, src/Analysis.F90:475-513, are never hit by
// an integer |k|^2), found in integers: r = floor(sqrt(k2)), shell r + 1 if
// k2 >= r^2 + r + 1, capped at the last bin.
#include "s2d.h"
#include "s2d_fft.cuh"
#include "s2d_internal.h"

#include <cuda_runtime.h>

#include <cmath>

namespace {

using namespace s2d;

constexpr int kThreads = 256;

__device__ __forceinline__ unsigned long long splitmix64_d(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ULL;
    unsigned long long z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// phase in [0, 2 pi): the top 53 bits of splitmix64(splitmix64(key)),
// key = seed<<42 ^ kx<<21 ^ (ky mod 2^21) (the host generator's hash)
__device__ __forceinline__ double mode_phase_d(unsigned long long seed, long long kx, long long ky) {
    const unsigned long long key = (seed << 42) ^ ((unsigned long long)kx << 21) ^ ((unsigned long long)ky & 0x1FFFFFULL);
    const unsigned long long h = splitmix64_d(splitmix64_d(key));
    const double u = __dmul_rn((double)(h >> 11), 1.0 / 9007199254740992.0);
    return __dmul_rn(2.0 * M_PI, u);
}

// 0-based bin of BinarySearch (1-based result minus one, capped at numBin-1)
__device__ __forceinline__ int shell_of(long long k2, int numBin) {
    long long r = (long long)sqrt((double)k2);
    while (r * r > k2) --r;
    while ((r + 1) * (r + 1) <= k2) ++r;
    const long long b = (k2 >= r * r + r + 1) ? r + 1 : r;   // round(|k|)
    return (int)(b < numBin - 1 ? b : numBin - 1);
}

__global__ void __launch_bounds__(kThreads) k_ic_shell_count(int C, int NY, int kxMG, int numBin,
                                                             unsigned long long* cnt) {
    extern __shared__ unsigned int hist[];
    for (int b = threadIdx.x; b < numBin; b += blockDim.x) hist[b] = 0u;
    __syncthreads();
    const long long n = (long long)C * NY;
    for (long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x; o < n; o += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(o / C);
        const int i = (int)(o - (long long)j * C);
        const long long ky = j > NY / 2 ? j - NY : j;
        const long long k2 = (long long)i * i + ky * ky;
        atomicAdd(&hist[shell_of(k2, numBin)], (i == 0 || i == kxMG) ? 1u : 2u);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < numBin; b += blockDim.x)
        if (hist[b]) atomicAdd(&cnt[b], (unsigned long long)hist[b]);
}

__device__ __forceinline__ double spectrum_shape_d(int kind, double k, double k0, double urms) {
    if (kind == S2D_SPECTRUM_SCHUMANN)   // 1.5 urms^2 (k/k0) exp(-k/k0), src/SetIC.F90:374-381
        return __dmul_rn(__ddiv_rn(__dmul_rn(__dmul_rn(__dmul_rn(1.5, urms), urms), k), k0), exp(-__ddiv_rn(k, k0)));
    const double kk = __dmul_rn(k, k);
    const double q = __ddiv_rn(k, k0);
    return __dmul_rn(__dmul_rn(kk, kk), exp(__dmul_rn(-2.0, __dmul_rn(q, q))));
}

// omega of retained mode (kx, ky), ky may be negative; kx = 0, ky < 0 is
// the conjugate of (0, -ky) (the Hermitian column)
__device__ __forceinline__ double2 ic_mode(int kx, int ky, unsigned long long seed, int kind, double k0, double urms,
                                           const unsigned long long* __restrict__ cnt, int numBin) {
    bool conj = false;
    if (kx == 0 && ky < 0) {
        ky = -ky;
        conj = true;
    }
    const double fkx = (double)kx, fky = (double)ky;
    const long long k2 = (long long)kx * kx + (long long)ky * ky;
    const double kmag = __dsqrt_rn(__dadd_rn(__dmul_rn(fkx, fkx), __dmul_rn(fky, fky)));
    const double E = spectrum_shape_d(kind, kmag, k0, urms);
    const double th = mode_phase_d(seed, kx, ky);
    const double amp = __dsqrt_rn(E);
    double s, c;
    sincos(th, &s, &c);
    const double ar = __dmul_rn(amp, c), ai = __dmul_rn(amp, s);
    const double nrm = __dsqrt_rn((double)cnt[shell_of(k2, numBin)]);
    const double ur = __ddiv_rn(__ddiv_rn(__dmul_rn(-ar, fky), kmag), nrm);
    const double ui = __ddiv_rn(__ddiv_rn(__dmul_rn(-ai, fky), kmag), nrm);
    const double vr = __ddiv_rn(__ddiv_rn(__dmul_rn(ar, fkx), kmag), nrm);
    const double vi = __ddiv_rn(__ddiv_rn(__dmul_rn(ai, fkx), kmag), nrm);
    double2 w;   // i kx v - i ky u
    w.x = __dsub_rn(__dmul_rn(-fkx, vi), __dmul_rn(-fky, ui));
    w.y = __dsub_rn(__dmul_rn(fkx, vr), __dmul_rn(fky, ur));
    if (conj) w.y = -w.y;
    return w;
}

// grid (ceil(KY / kThreads), KX): mode (kx = blockIdx.y, jc); W: FP64
// compact omega; part[blockIdx.y * gridDim.x + blockIdx.x]: the CTA's TKE sum
__global__ void __launch_bounds__(kThreads) k_ic_modes(Dims d, unsigned long long seed, int kind, double k0,
                                                       double urms, const unsigned long long* __restrict__ cnt,
                                                       int numBin, double2* W, double* part) {
    __shared__ double red[kThreads / 32];
    const int kx = blockIdx.y;
    const int jc = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0;
    if (jc < d.KY) {
        const int ky = jc <= d.K ? jc : jc - d.KY;
        const long long k2 = (long long)kx * kx + (long long)ky * ky;
        double2 w = make_double2(0.0, 0.0);
        if (k2 != 0 && k2 <= (long long)d.K * d.K) {
            w = ic_mode(kx, ky, seed, kind, k0, urms, cnt, numBin);
            // |u|^2 + |v|^2 = k^2 |psi|^2, psi = w / k^2; half weight on kx = 0
            const double fk2 = (double)k2;
            const double pr = __ddiv_rn(w.x, fk2), pi = __ddiv_rn(w.y, fk2);
            e = __dmul_rn(fk2, __dadd_rn(__dmul_rn(pr, pr), __dmul_rn(pi, pi)));
            if (kx == 0) e = __dmul_rn(0.5, e);
        }
        W[(size_t)kx * d.ldS + jc] = w;
    }
    // fixed-order CTA sum: warp butterflies, then the warps in order
    for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xFFFFFFFFu, e, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = e;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < kThreads / 32; ++i) t += red[i];
        part[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = t;
    }
}

// one CTA: the partial sums in order, then scale = sqrt(tke / TKE) (1 when
// tke <= 0 or TKE = 0) in scale[0]
__global__ void __launch_bounds__(kThreads) k_ic_total(const double* __restrict__ part, int n, double tke,
                                                       double* scale) {
    __shared__ double red[kThreads];
    double t = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) t += part[i];
    red[threadIdx.x] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < kThreads; ++i) s += red[i];
        scale[0] = (tke > 0.0 && s > 0.0) ? sqrt(tke / s) : 1.0;
    }
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_ic_store(Dims d, const double2* __restrict__ W,
                                                       const double* __restrict__ scale,
                                                       typename Vec<T>::t* S) {
    const int kx = blockIdx.y;
    const int jc = blockIdx.x * blockDim.x + threadIdx.x;
    if (jc >= d.KY) return;
    const size_t off = (size_t)kx * d.ldS + jc;
    const double s = scale[0];
    const double2 w = W[off];
    typename Vec<T>::t o;
    o.x = (T)__dmul_rn(w.x, s);
    o.y = (T)__dmul_rn(w.y, s);
    S[off] = o;
}

size_t up256(size_t x) { return (x + 255) / 256 * 256; }

}  // namespace

namespace s2d {

// The turbulent initial condition into h->S0, computed on the device (see
// the file comment); the handle's intermediate buffers are its scratch.
int set_turbulent_device(s2d_handle* h, uint64_t seed, int spectrum, double k0, double urms, double tke) {
    const Dims& d = h->d;
    const int C = h->grid.cISize, NY = h->grid.nyG, kxMG = h->grid.kxMG, kyMG = h->grid.kyMG;
    const double kMaxG = std::sqrt((double)kxMG * kxMG + (double)kyMG * kyMG);
    const int numBin = (int)(kMaxG + 1.0) + 1;   // src/SetIC.F90:269-292
    const dim3 grid((d.KY + kThreads - 1) / kThreads, d.KX);
    const int nparts = (int)(grid.x * grid.y);
    const size_t wbytes = up256((size_t)d.KX * d.ldS * sizeof(double2));
    const size_t pbytes = up256((size_t)nparts * sizeof(double));
    const size_t cbytes = up256((size_t)numBin * sizeof(unsigned long long)) + 256;
    if (wbytes + pbytes + cbytes > 3 * h->Ibytes) return set_error(S2D_ERR_UNSUPPORTED, "IC scratch too small");
    if ((size_t)numBin * sizeof(unsigned int) > 48 * 1024)
        return set_error(S2D_ERR_UNSUPPORTED, "too many spectrum bins for the shell-count kernel");
    char* base = (char*)h->Ibase;
    double2* W = (double2*)base;
    double* part = (double*)(base + wbytes);
    unsigned long long* cnt = (unsigned long long*)(base + wbytes + pbytes);
    double* scale = (double*)(base + wbytes + pbytes + up256((size_t)numBin * sizeof(unsigned long long)));
    cudaStream_t st = h->stream;
    if (cudaMemsetAsync(cnt, 0, (size_t)numBin * sizeof(unsigned long long), st) != cudaSuccess)
        return set_error(S2D_ERR_CUDA, "IC: memset failed");
    k_ic_shell_count<<<2 * h->sms, kThreads, (size_t)numBin * sizeof(unsigned int), st>>>(C, NY, kxMG, numBin, cnt);
    k_ic_modes<<<grid, kThreads, 0, st>>>(d, (unsigned long long)seed, spectrum, k0, urms, cnt, numBin, W, part);
    k_ic_total<<<1, kThreads, 0, st>>>(part, nparts, tke, scale);
    if (h->prec == S2D_FP64) k_ic_store<double><<<grid, kThreads, 0, st>>>(d, W, scale, (double2*)h->S0);
    else k_ic_store<float><<<grid, kThreads, 0, st>>>(d, W, scale, (float2*)h->S0);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(S2D_ERR_CUDA, cudaGetErrorString(e));
    if (cudaStreamSynchronize(st) != cudaSuccess) return set_error(S2D_ERR_CUDA, "IC: stream synchronisation failed");
    return S2D_OK;
}

}  // namespace s2d

extern "C" {

S2D_API int s2d_set_turbulent(s2d_handle* h, uint64_t seed, int32_t spectrum, double k0, double urms, double tke) {
    if (!h) return s2d::set_error(S2D_ERR_INVALID, "null handle");
    if (spectrum != S2D_SPECTRUM_SCHUMANN && spectrum != S2D_SPECTRUM_K4_GAUSS)
        return s2d::set_error(S2D_ERR_INVALID, "unknown spectrum");
    if (!(k0 > 0.0) || !std::isfinite(k0) || !std::isfinite(urms) || !std::isfinite(tke))
        return s2d::set_error(S2D_ERR_INVALID, "k0 must be > 0; urms and tke finite");
    if (cudaSetDevice(h->device) != cudaSuccess) return s2d::set_error(S2D_ERR_CUDA, "cudaSetDevice failed");
    return s2d::set_turbulent_device(h, seed, spectrum, k0, urms, tke);
}

}  // extern "C"
