// s2d_capi.cu -- C-ABI of the Spectral2D GB300 library (see include/s2d.h).
//
// Host logic: grid setup (GetGridSize, src/Spectral.F90:117-219), FFT plans
// and twiddle tables, device buffers, launch shapes, the RK3 step
// (IntegrateOneStep, src/TimeIntegration.F90:130-210) as 9 kernel launches
// (3 stages x {inverse y-pass, x-pass, forward y-pass + stage update}; 12
// when the forward y-pass and the stage update are split), its CUDA graph,
// host I/O in the reference layout (the truncated part of an output array is
// written on a second stream while the step runs), diagnostics and initial
// conditions.  No framework types cross this boundary.
#include "s2d.h"
#include "s2d_internal.h"
#include "s2d_plan.h"

#include <cuda_runtime.h>
#include <sys/mman.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace s2d;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define S2D_CUDA(call)                                                                          \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return fail(S2D_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),   \
                        __FILE__, __LINE__);                                                    \
    } while (0)

#define S2D_TRY(call)                   \
    do {                                \
        int r_ = (call);                \
        if (r_ != S2D_OK) return r_;    \
    } while (0)

// FMA-form twiddle blocks of a plan (s2d_plan.h) in a vector.
template <typename T>
std::vector<TwEnt<T>> fma_tables(Dims* d) {
    std::vector<TwEnt<T>> tab((size_t)fma_table_entries(*d));
    fill_fma_tables<T>(d, tab.data(), (int)tab.size());
    return tab;
}

int kIntMaxBins(int kxMG, int kyMG) {
    const double kMax = std::sqrt((double)(kxMG * kxMG + kyMG * kyMG));
    const int kIntMax = (int)(kMax + 1.0);
    return kIntMax + 1;
}

}  // namespace


namespace {

// G transforms of threads_per_group threads per CTA: at most target_threads
// per CTA, at least one warp, and no more transforms per CTA than spread the
// kernel's `items` transforms over two CTAs per SM (small grids would
// otherwise leave most SMs idle).
int pick_launch(const s2d_handle* h, int threads_per_group, size_t bytes_per_group, int target_threads, long items,
                Launch* L, const char* what) {
    const size_t cap_pair = (size_t)h->max_smem / 2;
    if (bytes_per_group > (size_t)h->max_smem)
        return fail(S2D_ERR_UNSUPPORTED, "%s: %zu bytes of shared memory per transform exceed %d", what,
                    bytes_per_group, h->max_smem);
    if (threads_per_group > 512)
        return fail(S2D_ERR_UNSUPPORTED, "%s: %d threads per transform exceed 512", what, threads_per_group);
    const int gmax = std::max(1, target_threads / threads_per_group);
    const int gmin = std::max(1, (32 + threads_per_group - 1) / threads_per_group);
    const long gfill = (items + 2L * h->sms - 1) / (2L * h->sms);
    int G = (int)std::max<long>(gmin, std::min<long>(gmax, gfill));
    while (G > 1 && (G * threads_per_group > 512 || G * bytes_per_group > cap_pair)) --G;
    L->G = G;
    L->threads = G * threads_per_group;
    L->smem = G * bytes_per_group;
    L->blocks = 0;
    return S2D_OK;
}

__global__ void k_round_f32(const double* __restrict__ in, float* out, long n) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}
cudaError_t round_to_f32(const double* in, float* out, long n, cudaStream_t st) {
    k_round_f32<<<(int)std::min<long>((n + 255) / 256, 152L * 8), 256, 0, st>>>(in, out, n);
    return cudaGetLastError();
}

// join: an event on another stream that the epilogue (the first kernel that
// reads h->src) waits for; the kernels before it run concurrently with that
// stream's work
template <typename T>
int launch_rhs_stage(s2d_handle* h, int stage, double dt, cudaEvent_t* ev, cudaEvent_t join = nullptr) {
    const Dims& d = h->d;
    const bool bas = h->ph.form == S2D_NL_BASDEVANT;
    FieldSet fs{};
    fs.nf = bas ? 2 : 3;
    // Basdevant: the scaled factors of u and v from their tables
    fs.op[0] = bas ? OP_TU : OP_U;
    fs.op[1] = bas ? OP_TV : OP_V;
    fs.op[2] = OP_W;
    fs.tab[0] = h->fu;
    fs.tab[1] = h->fv;
    fs.tabf[0] = h->fu32;
    fs.tabf[1] = h->fv32;
    fs.out[0] = h->I[0];
    fs.out[1] = h->I[1];
    fs.out[2] = h->I[2];
    const void* win = (stage <= 1) ? h->S0 : h->S1;
    if (ev) S2D_CUDA(cudaEventRecord(ev[0], h->stream));
    S2D_CUDA(Kern<T>::yinv(d, win, bas ? h->rk2s : h->rk2, fs, h->tw, h->stream, h->L_yinv));
    if (ev) S2D_CUDA(cudaEventRecord(ev[1], h->stream));
    if (bas) S2D_CUDA(Kern<T>::xpass_bas(d, h->I[0], h->I[1], h->tw, h->stream, h->L_xrow, true));
    else S2D_CUDA(Kern<T>::xpass_rhs(d, h->I[0], h->I[1], h->I[2], h->tw, h->stream, h->L_xpass));
    if (ev) S2D_CUDA(cudaEventRecord(ev[2], h->stream));
    if (h->Fv) {
        // K3 in two launches (FP64, Basdevant): the column FFTs take three
        // CTAs per SM; the products' spectra go through I[2] (free in this
        // form) and Fv in the compact layout
        S2D_CUDA(Kern<T>::yfwd_col(d, h->I[0], h->I[1], h->I[2], h->Fv, h->tw, h->stream, h->L_ycol));
        // the epilogue after a cross-stream join is an ordinary launch
        if (join) S2D_CUDA(cudaStreamWaitEvent(h->stream, join, 0));
        S2D_CUDA(Kern<T>::stage(d, h->I[2], h->Fv, h->S0, h->S1, h->Sdw, h->src, stage, dt, h->ph, h->flags,
                                h->stream, h->L_ycol.pdl && !join, h->cc, h->vk));
    } else {
        Launch L = h->L_yfwd;
        if (join) {
            S2D_CUDA(cudaStreamWaitEvent(h->stream, join, 0));
            L.pdl = false;
        }
        S2D_CUDA(Kern<T>::yfwd_rk3(d, h->I[0], h->I[1], h->S0, h->S1, h->Sdw, h->src, stage, dt, h->ph, h->tw,
                                   h->flags, h->stream, L));
    }
    if (ev) S2D_CUDA(cudaEventRecord(ev[3], h->stream));
    return S2D_OK;
}

int launch_rhs_stage_any(s2d_handle* h, int stage, double dt, cudaEvent_t* ev, cudaEvent_t join = nullptr) {
    return h->prec == S2D_FP64 ? launch_rhs_stage<double>(h, stage, dt, ev, join)
                               : launch_rhs_stage<float>(h, stage, dt, ev, join);
}

int launch_step(s2d_handle* h, double dt) {
    for (int s = 1; s <= 3; ++s) S2D_TRY(launch_rhs_stage_any(h, s, dt, nullptr));
    return S2D_OK;
}

int check_ref_dims(const s2d_handle* h, int cISize, int nyG) {
    if (cISize != h->grid.cISize || nyG != h->grid.nyG)
        return fail(S2D_ERR_INVALID, "array shape (%d,%d) does not match (cISize,nyG)=(%d,%d)", cISize, nyG,
                    h->grid.cISize, h->grid.nyG);
    return S2D_OK;
}

int ensure_ref_stage(s2d_handle* h) {
    if (h->ref_stage) return S2D_OK;
    S2D_CUDA(cudaMalloc(&h->ref_stage, 2 * h->ref_bytes));
    return S2D_OK;
}

// A host array of a host-array call, as the kernels reach it: in place
// through a device-usable address (page-locked memory; pageable memory where
// the device reads the host page tables, as on Grace; device memory), or,
// with dev null, through the staging arrays and copies.
struct HostArray {
    double* host = nullptr;
    double* dev = nullptr;
    bool pageable = false;   // in place through the host page tables
};

// Whether 16 pages spread over [p, p + n) are resident.  The device writes
// pageable memory in place only where its pages exist already: a page the
// GPU touches first is faulted in by the host (45 ms for the 84 MB of fresh
// np.zeros pages of a 2048^2 output pair on GB300, against 0.4 ms resident),
// while a staging copy lets the CPU populate them.
bool pages_resident(const void* p, size_t n) {
    const long ps = sysconf(_SC_PAGESIZE);
    if (ps <= 0 || n == 0) return false;
    const uintptr_t mask = ~(uintptr_t)(ps - 1);
    const uintptr_t first = (uintptr_t)p & mask, last = ((uintptr_t)p + n - 1) & mask;
    constexpr int kSamples = 16;
    for (int i = 0; i < kSamples; ++i) {
        const uintptr_t q = (first + (last - first) / (kSamples - 1) * (uintptr_t)i) & mask;
        unsigned char v = 0;
        if (mincore((void*)q, (size_t)ps, &v) != 0 || !(v & 1)) return false;
    }
    return true;
}

HostArray host_array(const s2d_handle* h, const double* p) {
    HostArray a;
    a.host = const_cast<double*>(p);
    if (!p || h->io_copy_only) return a;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return a;
    }
    if (at.type == cudaMemoryTypeHost) {
        a.dev = (double*)at.devicePointer;
    } else if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) {
        if (at.device == h->device) a.dev = a.host;
    } else if (h->pageable_direct && pages_resident(p, h->ref_bytes)) {
        a.dev = a.host;
        a.pageable = true;
    }
    return a;
}

// Only the retained rectangle of the reference array is read (kx <= K in rows
// ky = 0..K and ky = -K..-1, i.e. rows 0..K and M-K..M-1): the rest is
// truncated away, so it is neither read nor copied.
int upload_ref(s2d_handle* h, const HostArray& w) {
    const double* src = w.dev;
    if (!src) {
        S2D_TRY(ensure_ref_stage(h));
        const size_t pitch = (size_t)h->grid.cISize * 2 * sizeof(double);
        const size_t width = (size_t)h->d.KX * 2 * sizeof(double);
        const size_t lo = (size_t)(h->d.M - h->d.K) * pitch;
        const int K = h->d.K;
        S2D_CUDA(cudaMemcpy2DAsync(h->ref_stage, pitch, w.host, pitch, width, K + 1, cudaMemcpyDefault,
                                   h->stream));
        S2D_CUDA(cudaMemcpy2DAsync((char*)h->ref_stage + lo, pitch, (const char*)w.host + lo, pitch, width, K,
                                   cudaMemcpyDefault, h->stream));
        src = h->ref_stage;
    }
    if (h->prec == S2D_FP64)
        S2D_CUDA(Kern<double>::rect_to_compact(h->d, src, h->grid.cISize, h->S0, h->stream));
    else
        S2D_CUDA(Kern<float>::rect_to_compact(h->d, src, h->grid.cISize, h->S0, h->stream));
    return S2D_OK;
}

// Outputs in the reference layout are zero outside the retained rectangle
// (Truncate, src/Spectral.F90:788-802): columns kx > K of rows 0..K and
// M-K..M-1, and the whole rows K+1..M-K-1.  That part does not depend on the
// state, so it is written on the handle's second stream, which a host-array
// step issues before the step and so overlaps with it: by a small kernel for
// pageable arrays reached in place (a copy into pageable memory may hold the
// host until it ends), else by copies from a device buffer of zeros.
int send_zeros(s2d_handle* h, const HostArray& a, const HostArray& b) {
    if (!a.host && !b.host) return S2D_OK;
    const int K = h->d.K, M = h->d.M, C = h->grid.cISize;
    if (!h->xstream) S2D_CUDA(cudaStreamCreateWithFlags(&h->xstream, cudaStreamNonBlocking));
    if (a.pageable || b.pageable)
        S2D_CUDA(launch_zero_truncated(h->d, C, a.pageable ? a.dev : nullptr, b.pageable ? b.dev : nullptr, 48,
                                       h->xstream));
    const size_t pitch = (size_t)C * 2 * sizeof(double);
    const size_t kx_off = (size_t)h->d.KX * 2 * sizeof(double);
    const size_t tail = pitch - kx_off;                       // columns K+1..C-1 of one row
    const size_t mid = (size_t)(M - 2 * K - 1) * pitch;       // rows K+1..M-K-1
    for (const HostArray* x : {&a, &b}) {
        if (!x->host || x->pageable) continue;
        if (!h->zeros) {
            h->zeros_bytes = std::max(mid, tail);
            S2D_CUDA(cudaMalloc(&h->zeros, h->zeros_bytes));
            S2D_CUDA(cudaMemsetAsync(h->zeros, 0, h->zeros_bytes, h->xstream));
        }
        char* c = (char*)x->host;
        S2D_CUDA(cudaMemcpy2DAsync(c + kx_off, pitch, h->zeros, tail, tail, K + 1, cudaMemcpyDefault,
                                   h->xstream));
        S2D_CUDA(cudaMemcpy2DAsync(c + (size_t)(M - K) * pitch + kx_off, pitch, h->zeros, tail, tail, K,
                                   cudaMemcpyDefault, h->xstream));
        if (mid) S2D_CUDA(cudaMemcpyAsync(c + (size_t)(K + 1) * pitch, h->zeros, mid, cudaMemcpyDefault,
                                          h->xstream));
    }
    return S2D_OK;
}

// Waits for the second stream on every exit of a host-array call, so that
// no write into the caller's arrays is left in flight when it returns.
struct CopyStreamJoin {
    s2d_handle* h;
    ~CopyStreamJoin() {
        if (h->xstream) cudaStreamSynchronize(h->xstream);
    }
};

// Reference-layout outputs: the retained rectangle written in place by the
// conversion kernel, or into the staging arrays and copied; the rest by
// send_zeros, which the caller issues first.
int download_ref(s2d_handle* h, const void* S, const HostArray& w, const HostArray& p) {
    if (!w.host && !p.host) return S2D_OK;
    if ((w.host && !w.dev) || (p.host && !p.dev)) S2D_TRY(ensure_ref_stage(h));
    double* dW = w.dev ? w.dev : (w.host ? h->ref_stage : nullptr);
    double* dP = p.dev ? p.dev : (p.host ? (double*)((char*)h->ref_stage + h->ref_bytes) : nullptr);
    if (h->prec == S2D_FP64)
        S2D_CUDA(Kern<double>::compact_to_rect(h->d, S, h->grid.cISize, dW, dP, h->stream));
    else
        S2D_CUDA(Kern<float>::compact_to_rect(h->d, S, h->grid.cISize, dW, dP, h->stream));
    const size_t pitch = (size_t)h->grid.cISize * 2 * sizeof(double);
    const size_t width = (size_t)h->d.KX * 2 * sizeof(double);
    const size_t lo = (size_t)(h->d.M - h->d.K) * pitch;
    const int K = h->d.K;
    for (int f = 0; f < 2; ++f) {
        const HostArray& x = f == 0 ? w : p;
        if (!x.host || x.dev) continue;
        char* dst = (char*)x.host;
        const char* src = (const char*)(f == 0 ? dW : dP);
        S2D_CUDA(cudaMemcpy2DAsync(dst, pitch, src, pitch, width, K + 1, cudaMemcpyDefault, h->stream));
        S2D_CUDA(cudaMemcpy2DAsync(dst + lo, pitch, src + lo, pitch, width, K, cudaMemcpyDefault, h->stream));
    }
    S2D_CUDA(cudaStreamSynchronize(h->stream));
    if (h->xstream) S2D_CUDA(cudaStreamSynchronize(h->xstream));
    return S2D_OK;
}

void drop_graph(s2d_handle* h) {
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    if (h->graph) cudaGraphDestroy(h->graph);
    h->gexec = nullptr;
    h->graph = nullptr;
}

int build_graph(s2d_handle* h, double dt) {
    drop_graph(h);
    S2D_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int r = launch_step(h, dt);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (r != S2D_OK) {
        if (g) cudaGraphDestroy(g);
        return r;
    }
    if (e != cudaSuccess) return fail(S2D_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    h->graph = g;
    S2D_CUDA(cudaGraphInstantiate(&h->gexec, g, 0));
    h->graph_dt = dt;
    return S2D_OK;
}

// Spectrum -> (Ek, tke, eps, enstDiss) as ComputeSpectrum (src/Analysis.F90:414-448).
int spectrum_impl(s2d_handle* h, std::vector<double>& Ek) {
    const int nb = kIntMaxBins(h->grid.kxMG, h->grid.kyMG);
    Ek.assign(nb, 0.0);
    const int nk = h->d.K + 1;
    if (h->prec == S2D_FP64) S2D_CUDA(Kern<double>::spectrum(h->d, h->S0, h->dscratch, h->stream));
    else S2D_CUDA(Kern<float>::spectrum(h->d, h->S0, h->dscratch, h->stream));
    S2D_CUDA(cudaMemcpyAsync(Ek.data(), h->dscratch, sizeof(double) * std::min(nk, nb), cudaMemcpyDeviceToHost,
                             h->stream));
    S2D_CUDA(cudaStreamSynchronize(h->stream));
    return S2D_OK;
}

}  // namespace

int s2d::handle_nx(const s2d_handle* h) { return h->cfg.nx; }

int s2d::set_error(int code, const char* msg) { return fail(code, "%s", msg); }

// ============================================================================
// C-ABI
// ============================================================================

extern "C" {

S2D_API int s2d_version(void) { return 100; }

S2D_API const char* s2d_last_error(void) { return g_err.c_str(); }

S2D_API int s2d_get_grid_size(int32_t nx, int32_t ny, int32_t dealias, s2d_grid* o) {
    if (!o) return fail(S2D_ERR_INVALID, "null output");
    if (nx <= 0 || ny <= 0) return fail(S2D_ERR_INVALID, "nx, ny must be positive");
    std::memset(o, 0, sizeof(*o));
    o->nx = nx;
    o->ny = ny;
    o->dealias = dealias;
    if (dealias == S2D_NO_DEALIASING) {
        o->nxG = nx;
        o->nyG = ny;
    } else if (dealias == S2D_DEALIAS_3_2_RULE) {
        o->nxG = 3 * nx / 2;
        o->nyG = 3 * ny / 2;
    } else {
        return fail(S2D_ERR_UNSUPPORTED, "dealias=%d is an empty case in the reference", dealias);
    }
    o->kxLG = 0;
    o->kyLG = -o->nyG / 2 + 1;
    o->kxMG = o->nxG / 2;
    o->kyMG = o->nyG / 2;
    o->kxLU = 0;
    o->kyLU = -ny / 2 + 1;
    o->kxMU = nx / 2;
    o->kyMU = ny / 2;
    o->kMax = (double)o->kxMU;
    o->rISize = 2 * (o->nxG / 2 + 1);
    o->cISize = o->nxG / 2 + 1;
    return S2D_OK;
}

S2D_API int s2d_create(const s2d_config* cfg, s2d_handle** out) { return s2d::create_handle(cfg, nullptr, out); }

}  // extern "C"

int s2d::create_handle(const s2d_config* cfg, cudaStream_t ext_stream, s2d_handle** out) {
    if (!cfg || !out) return fail(S2D_ERR_INVALID, "null argument");
    *out = nullptr;
    if (cfg->dealias != S2D_DEALIAS_3_2_RULE)
        return fail(S2D_ERR_UNSUPPORTED,
                    "only the 3/2 rule is supported (without dealiasing the reference truncation is "
                    "undefined on the ky=0 row)");
    if (cfg->nx != cfg->ny) return fail(S2D_ERR_UNSUPPORTED, "nx must equal ny");
    if (cfg->nx < 8 || cfg->nx % 8 != 0) return fail(S2D_ERR_INVALID, "nx must be a positive multiple of 8");
    if (cfg->precision != S2D_FP64 && cfg->precision != S2D_FP32)
        return fail(S2D_ERR_INVALID, "precision must be S2D_FP64 or S2D_FP32");
    if (!(cfg->nu >= 0.0) || !std::isfinite(cfg->nu)) return fail(S2D_ERR_INVALID, "nu must be finite, >= 0");

    s2d_handle* h = new (std::nothrow) s2d_handle();
    if (!h) return fail(S2D_ERR_NOMEM, "host allocation failed");
    h->cfg = *cfg;
    h->prec = cfg->precision;
    h->vsz = h->prec == S2D_FP64 ? sizeof(double2) : sizeof(float2);
    h->device = cfg->device;
    int r = s2d_get_grid_size(cfg->nx, cfg->ny, cfg->dealias, &h->grid);
    if (r != S2D_OK) {
        delete h;
        return r;
    }
    Dims& d = h->d;
    d.K = cfg->nx / 2;
    d.KX = d.K + 1;
    d.KY = 2 * d.K + 1;
    d.M = h->grid.nxG;
    d.ldS = d.KY + 1;                  // even pitch: 16-byte aligned FP32 columns
    d.ldI = (d.KX + 3) / 4 * 4;
    if (!factor_plan(d.M, &d)) {
        const int M = d.M;
        delete h;
        return fail(S2D_ERR_UNSUPPORTED, "padded grid %d is not 2^a 3^b with 12 | M", M);
    }
    d.Tg = d.M / kElemsPerThread;
    d.rows = d.M;
    d.kx0 = 0;
    {
        const char* xg = std::getenv("S2D_XPASS_GENERIC");
        d.xgen = (xg && xg[0] == '1') ? 1 : 0;
    }
    h->ph.nu = cfg->nu;
    h->ph.alpha = cfg->alpha;
    h->ph.form = cfg->nonlinear_form;
    if (h->ph.form != S2D_NL_BASDEVANT && h->ph.form != S2D_NL_CONSERVATIVE) {
        delete h;
        return fail(S2D_ERR_INVALID, "nonlinear_form must be S2D_NL_BASDEVANT or S2D_NL_CONSERVATIVE");
    }
    h->ph.fk = cfg->forcing_amp != 0.0 ? cfg->forcing_k : 0;
    if (h->ph.fk < 0 || h->ph.fk > d.K) {
        const int K = d.K;
        delete h;
        return fail(S2D_ERR_INVALID, "forcing wavenumber %d outside [0, %d]", cfg->forcing_k, K);
    }
    {
        // amp cos(kf y) on the 1-based grid y_j = 2 pi j / nyG: coefficient
        // amp/2 exp(i kf dy) at ky = +kf (and the conjugate at -kf).
        const double dy = 2.0 * M_PI / (double)d.M;
        h->ph.f_re = 0.5 * cfg->forcing_amp * std::cos(h->ph.fk * dy);
        h->ph.f_im = 0.5 * cfg->forcing_amp * std::sin(h->ph.fk * dy);
    }

    auto bail = [&](int code) {
        s2d_destroy(h);
        return code;
    };
    if (cudaSetDevice(h->device) != cudaSuccess) return bail(fail(S2D_ERR_CUDA, "cudaSetDevice(%d) failed", h->device));
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, h->device) != cudaSuccess)
        return bail(fail(S2D_ERR_CUDA, "cudaGetDeviceProperties failed"));
    h->max_smem = (int)prop.sharedMemPerBlockOptin - 1024;
    h->sms = prop.multiProcessorCount;
    {
        const char* io = std::getenv("S2D_HOST_IO");
        h->io_copy_only = io && std::strcmp(io, "copy") == 0;
        int pageable = 0;
        if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, h->device) != cudaSuccess)
            pageable = 0;
        h->pageable_direct = pageable == 1 && !h->io_copy_only;
    }
    {
        static std::atomic<bool> configured[64];  // per device, set once the attributes are (a second setter only repeats them)
        if (h->device >= 0 && h->device < 64 && !configured[h->device]) {
            if (configure_kernels(h->max_smem) != cudaSuccess)
                return bail(fail(S2D_ERR_CUDA, "cudaFuncSetAttribute failed"));
            configured[h->device] = true;
        }
    }
    if (ext_stream) {
        h->stream = ext_stream;
        h->own_stream = false;
    } else if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        return bail(fail(S2D_ERR_CUDA, "stream creation failed"));
    }

    const size_t state_bytes = (size_t)d.KX * d.ldS * h->vsz;
    h->Ibytes = (size_t)d.M * d.ldI * h->vsz;
#define S2D_ALLOC(p, n)                                                                                   \
    do {                                                                                                  \
        if (cudaMalloc((void**)&(p), (n)) != cudaSuccess)                                                \
            return bail(fail(S2D_ERR_NOMEM, "cudaMalloc of %zu bytes failed", (size_t)(n)));             \
        cudaMemsetAsync((p), 0, (n), h->stream);                                                          \
    } while (0)
    S2D_ALLOC(h->S0, state_bytes);
    S2D_ALLOC(h->S1, state_bytes);
    if (h->prec == S2D_FP64 && h->ph.form == S2D_NL_BASDEVANT) {
        S2D_ALLOC(h->Fv, state_bytes);
        S2D_ALLOC(h->cc, (size_t)d.KX * d.ldS * 2 * sizeof(double));
        S2D_ALLOC(h->vk, (size_t)d.KX * d.ldS * sizeof(double));
    }
    S2D_ALLOC(h->Ibase, 3 * h->Ibytes);
    h->I[0] = h->Ibase;
    h->I[1] = (char*)h->Ibase + h->Ibytes;
    h->I[2] = (char*)h->Ibase + 2 * h->Ibytes;
    S2D_ALLOC(h->rk2, (size_t)d.KX * d.ldS * sizeof(double));
    if (h->ph.form == S2D_NL_BASDEVANT) {
        S2D_ALLOC(h->rk2s, (size_t)d.KX * d.ldS * sizeof(double));
        S2D_ALLOC(h->fu, (size_t)d.KX * d.ldS * sizeof(double));
        S2D_ALLOC(h->fv, (size_t)d.KX * d.ldS * sizeof(double));
        if (h->prec == S2D_FP32) {
            S2D_ALLOC(h->fu32, (size_t)d.KX * d.ldS * sizeof(float));
            S2D_ALLOC(h->fv32, (size_t)d.KX * d.ldS * sizeof(float));
        }
    }
    // complex twiddles (M entries) followed by the FMA-form blocks
    std::vector<TwEnt<double>> tabd;
    std::vector<TwEnt<float>> tabf;
    if (h->prec == S2D_FP64) tabd = fma_tables<double>(&d);
    else tabf = fma_tables<float>(&d);
    d.tab_bytes = (long long)(((size_t)d.M * h->vsz + 63) / 64 * 64);
    const size_t tab_size = h->prec == S2D_FP64 ? tabd.size() * sizeof(TwEnt<double>)
                                                : tabf.size() * sizeof(TwEnt<float>);
    {
        // room for the FMA-form blocks of every radix plan (s2d_set_fft_plan)
        size_t cap = tab_size;
        for (int p = 0; p < kNumPlans; ++p) {
            Dims dp = d;
            if (factor_plan(d.M, &dp, p))
                cap = std::max(cap, (size_t)fma_table_entries(dp) *
                                        (h->prec == S2D_FP64 ? sizeof(TwEnt<double>) : sizeof(TwEnt<float>)));
        }
        h->tab_cap = cap;
    }
    S2D_ALLOC(h->tw, (size_t)d.tab_bytes + h->tab_cap + 64);
    S2D_ALLOC(h->flags, 64);
    S2D_ALLOC(h->red64, 8 * sizeof(unsigned long long));
    h->dscratch_n = std::max<size_t>(d.K + 1, 4096);
    S2D_ALLOC(h->dscratch, h->dscratch_n * sizeof(double));
#undef S2D_ALLOC
    h->ref_bytes = (size_t)h->grid.cISize * h->grid.nyG * 2 * sizeof(double);

    // twiddles exp(-2 pi i t / M)
    {
        std::vector<double> twd(2 * (size_t)d.M);
        fill_twiddles(d.M, twd.data());
        if (h->prec == S2D_FP64) {
            if (cudaMemcpy(h->tw, twd.data(), twd.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
                return bail(fail(S2D_ERR_CUDA, "twiddle upload failed"));
        } else {
            std::vector<float> twf(twd.begin(), twd.end());
            if (cudaMemcpy(h->tw, twf.data(), twf.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
                return bail(fail(S2D_ERR_CUDA, "twiddle upload failed"));
        }
        const void* src = h->prec == S2D_FP64 ? (const void*)tabd.data() : (const void*)tabf.data();
        if (tab_size && cudaMemcpy((char*)h->tw + d.tab_bytes, src, tab_size, cudaMemcpyHostToDevice) != cudaSuccess)
            return bail(fail(S2D_ERR_CUDA, "twiddle table upload failed"));
    }
    if (Kern<double>::init_rk2(d, h->rk2, h->stream) != cudaSuccess ||
        (h->rk2s && Kern<double>::init_rk2(d, h->rk2s, h->stream, std::sqrt(0.5) / (double)d.M) != cudaSuccess) ||
        (h->fu && Kern<double>::init_uv_factors(d, h->rk2s, h->fu, h->fv, h->stream) != cudaSuccess) ||
        (h->fu32 && (round_to_f32(h->fu, h->fu32, (long)d.KX * d.ldS, h->stream) != cudaSuccess ||
                     round_to_f32(h->fv, h->fv32, (long)d.KX * d.ldS, h->stream) != cudaSuccess)) ||
        (h->cc && Kern<double>::init_stage_factors(d, h->ph.nu, h->cc, h->vk, h->stream) != cudaSuccess))
        return bail(fail(S2D_ERR_CUDA, "rk2 init failed"));

    // launch shapes: about 256 threads per CTA so that at least two CTAs
    // share an SM and one CTA's barrier phases overlap the other's FP64 work
    const size_t tb = (size_t)d.M * h->vsz;
    const int tgt = 256;
    int rr;
    const int nf = h->ph.form == S2D_NL_BASDEVANT ? 2 : 3;
    if ((rr = pick_launch(h, d.Tg, tb, tgt, (long)nf * d.KX, &h->L_yinv, "inverse y-pass")) != S2D_OK)
        return bail(rr);
    if ((rr = pick_launch(h, d.Tg, 2 * tb, tgt, d.M / 2, &h->L_xpass, "x-pass")) != S2D_OK) return bail(rr);
    {
        // forward y-pass: G columns x 2 fields, run in rounds of c transforms
        Launch L{};
        if ((rr = pick_launch(h, d.Tg, 2 * tb, tgt, d.KX, &L, "forward y-pass")) != S2D_OK) return bail(rr);
        int c = std::max(1, std::min(2 * L.G, tgt / d.Tg));
        while ((2 * L.G) % c) --c;
        L.threads = c * d.Tg;
        h->L_yfwd = L;
    }
    if ((rr = pick_launch(h, d.Tg, tb, tgt, d.M, &h->L_xrow, "row transform")) != S2D_OK) return bail(rr);
    if ((rr = pick_launch(h, d.Tg, tb, tgt, d.KX, &h->L_ystore, "column transform")) != S2D_OK) return bail(rr);
    if ((rr = pick_launch(h, d.Tg, tb, tgt, 2L * d.KX, &h->L_ycol, "forward y-pass (split)")) != S2D_OK)
        return bail(rr);
    // every kernel of a step is launched as a programmatic dependent of the
    // one before it (S2D_PDL=0: plain stream order)
    {
        const char* e = std::getenv("S2D_PDL");
        const bool pdl = !(e && e[0] == '0');
        for (Launch* L : {&h->L_yinv, &h->L_xpass, &h->L_yfwd, &h->L_xrow, &h->L_ystore, &h->L_ycol}) L->pdl = pdl;
    }

    if (cudaStreamSynchronize(h->stream) != cudaSuccess) return bail(fail(S2D_ERR_CUDA, "setup failed"));
    *out = h;
    return S2D_OK;
}

// One RK3 step whose source term h->src is produced on another stream: the
// first stage's inverse y-pass and x-pass run concurrently with that work,
// its epilogue waits for src_ready.
int s2d::launch_step_sourced(s2d_handle* h, double dt, cudaEvent_t src_ready) {
    S2D_TRY(launch_rhs_stage_any(h, 1, dt, nullptr, src_ready));
    for (int s = 2; s <= 3; ++s) S2D_TRY(launch_rhs_stage_any(h, s, dt, nullptr));
    return S2D_OK;
}

extern "C" {

S2D_API void s2d_destroy(s2d_handle* h) {
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    drop_graph(h);
    void* ptrs[] = {h->S0,    h->S1,        h->Sdw,   h->Ibase, h->rk2,      h->rk2s, h->fu, h->fv, h->fu32, h->fv32, h->cc, h->vk, h->tw,  h->ref_stage,
                    h->flags, h->red64,     h->dscratch, h->src, h->pi, h->phys, h->les_tab, h->Fv,
                    h->zeros, h->cl_I};
    if (h->xstream) cudaStreamSynchronize(h->xstream);
    if (h->clstream) cudaStreamSynchronize(h->clstream);
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (h->xstream) cudaStreamDestroy(h->xstream);
    if (h->clstream) cudaStreamDestroy(h->clstream);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    if (h->stream && h->own_stream) cudaStreamDestroy(h->stream);
    delete h;
}

static_assert(kNumPlans == S2D_FFT_PLANS, "plan count of the header");

S2D_API int s2d_set_fft_plan(s2d_handle* h, int32_t plan) {
    if (!h) return fail(S2D_ERR_INVALID, "null handle");
    if (plan < 0 || plan >= kNumPlans) return fail(S2D_ERR_INVALID, "plan %d outside [0, %d)", plan, kNumPlans);
    if (plan == h->plan) return S2D_OK;
    if (h->cnn) return fail(S2D_ERR_INVALID, "detach the closure before changing the radix plan");
    S2D_CUDA(cudaSetDevice(h->device));
    Dims d = h->d;
    if (!factor_plan(d.M, &d, plan)) return fail(S2D_ERR_UNSUPPORTED, "radix plan %d does not apply", plan);
    S2D_CUDA(cudaStreamSynchronize(h->stream));
    if (h->prec == S2D_FP64) {
        const std::vector<TwEnt<double>> t = fma_tables<double>(&d);
        if (t.size() * sizeof(TwEnt<double>) > h->tab_cap) return fail(S2D_ERR_UNSUPPORTED, "twiddle table too big");
        if (!t.empty())
            S2D_CUDA(cudaMemcpy((char*)h->tw + d.tab_bytes, t.data(), t.size() * sizeof(TwEnt<double>),
                                cudaMemcpyHostToDevice));
    } else {
        const std::vector<TwEnt<float>> t = fma_tables<float>(&d);
        if (t.size() * sizeof(TwEnt<float>) > h->tab_cap) return fail(S2D_ERR_UNSUPPORTED, "twiddle table too big");
        if (!t.empty())
            S2D_CUDA(cudaMemcpy((char*)h->tw + d.tab_bytes, t.data(), t.size() * sizeof(TwEnt<float>),
                                cudaMemcpyHostToDevice));
    }
    h->d = d;
    h->plan = plan;
    drop_graph(h);   // the step's graph holds the old plan's Dims
    return S2D_OK;
}

S2D_API int s2d_get_fft_plan(const s2d_handle* h, int32_t* plan) {
    if (!h || !plan) return fail(S2D_ERR_INVALID, "null argument");
    *plan = h->plan;
    return S2D_OK;
}

S2D_API int s2d_tune_fft_plan(s2d_handle* h, double dt, int32_t* plan, double* ms) {
    if (!h || !std::isfinite(dt)) return fail(S2D_ERR_INVALID, "null handle or bad dt");
    S2D_CUDA(cudaSetDevice(h->device));
    const size_t bytes = (size_t)h->d.KX * h->d.ldS * h->vsz;
    void* save = nullptr;
    S2D_CUDA(cudaMalloc(&save, bytes));
    S2D_CUDA(cudaMemcpyAsync(save, h->S0, bytes, cudaMemcpyDeviceToDevice, h->stream));
    const int start = h->plan;
    double best = 1e300;
    int bp = start;
    int r = S2D_OK;
    // about 0.1 s of steps per candidate, at least 3
    const int n = std::max(3, std::min(200, (int)(4.0e8 / ((double)h->d.M * h->d.M + 1.0))));
    for (int p = 0; p < kNumPlans && r == S2D_OK; ++p) {
        if (s2d_set_fft_plan(h, p) != S2D_OK) continue;
        double t = 0.0;
        r = s2d_integrate_steps(h, 1, dt);   // warm-up (graph build)
        if (r == S2D_OK) r = s2d_time_steps(h, n, dt, &t, nullptr);
        if (r != S2D_OK) break;
        if (ms) ms[p] = t / n;
        if (t < best) {
            best = t;
            bp = p;
        }
    }
    cudaMemcpyAsync(h->S0, save, bytes, cudaMemcpyDeviceToDevice, h->stream);
    cudaStreamSynchronize(h->stream);
    cudaFree(save);
    if (r != S2D_OK) {
        s2d_set_fft_plan(h, start);
        return r;
    }
    S2D_TRY(s2d_set_fft_plan(h, bp));
    if (plan) *plan = bp;
    return S2D_OK;
}

S2D_API int s2d_set_state(s2d_handle* h, const double* wC, int32_t cISize, int32_t nyG) {
    if (!h || !wC) return fail(S2D_ERR_INVALID, "null argument");
    S2D_TRY(check_ref_dims(h, cISize, nyG));
    S2D_CUDA(cudaSetDevice(h->device));
    S2D_TRY(upload_ref(h, host_array(h, wC)));
    S2D_CUDA(cudaStreamSynchronize(h->stream));
    return S2D_OK;
}

S2D_API int s2d_get_state(s2d_handle* h, double* wC, double* psiC, int32_t cISize, int32_t nyG) {
    if (!h) return fail(S2D_ERR_INVALID, "null handle");
    S2D_TRY(check_ref_dims(h, cISize, nyG));
    S2D_CUDA(cudaSetDevice(h->device));
    CopyStreamJoin join{h};
    const HostArray w = host_array(h, wC), p = host_array(h, psiC);
    S2D_TRY(send_zeros(h, w, p));
    return download_ref(h, h->S0, w, p);
}

S2D_API int s2d_integrate_one_step(s2d_handle* h, double dt) {
    if (!h) return fail(S2D_ERR_INVALID, "null handle");
    if (!std::isfinite(dt)) return fail(S2D_ERR_INVALID, "dt must be finite");
    S2D_CUDA(cudaSetDevice(h->device));
    return launch_step(h, dt);
}

S2D_API int s2d_integrate_steps(s2d_handle* h, int32_t n, double dt) {
    if (!h) return fail(S2D_ERR_INVALID, "null handle");
    if (n < 0 || !std::isfinite(dt)) return fail(S2D_ERR_INVALID, "bad step count or dt");
    S2D_CUDA(cudaSetDevice(h->device));
    if (n == 0) return S2D_OK;
    if (!h->gexec || h->graph_dt != dt) S2D_TRY(build_graph(h, dt));
    for (int i = 0; i < n; ++i) S2D_CUDA(cudaGraphLaunch(h->gexec, h->stream));
    return S2D_OK;
}

S2D_API int s2d_integrate_one_step_host(s2d_handle* h, double* wC, double* psiC, int32_t cISize, int32_t nyG,
                                        double dt) {
    if (!h || !wC) return fail(S2D_ERR_INVALID, "null argument");
    S2D_TRY(check_ref_dims(h, cISize, nyG));
    S2D_CUDA(cudaSetDevice(h->device));
    CopyStreamJoin join{h};
    const HostArray w = host_array(h, wC), p = host_array(h, psiC);
    S2D_TRY(send_zeros(h, w, p));  // only the truncated part: disjoint from the rectangle read in
    S2D_TRY(upload_ref(h, w));
    S2D_TRY(launch_step(h, dt));
    return download_ref(h, h->S0, w, p);
}

S2D_API int s2d_compute_rhs(s2d_handle* h, double* dW, int32_t cISize, int32_t nyG) {
    if (!h || !dW) return fail(S2D_ERR_INVALID, "null argument");
    S2D_TRY(check_ref_dims(h, cISize, nyG));
    S2D_CUDA(cudaSetDevice(h->device));
    if (!h->Sdw) S2D_CUDA(cudaMalloc(&h->Sdw, (size_t)h->d.KX * h->d.ldS * h->vsz));
    CopyStreamJoin join{h};
    const HostArray x = host_array(h, dW);
    S2D_TRY(send_zeros(h, x, HostArray{}));
    S2D_TRY(launch_rhs_stage_any(h, 0, 0.0, nullptr));
    return download_ref(h, h->Sdw, x, HostArray{});
}

S2D_API int s2d_spectrum_bins(const s2d_handle* h) {
    if (!h) return fail(S2D_ERR_INVALID, "null handle");
    return kIntMaxBins(h->grid.kxMG, h->grid.kyMG);
}

S2D_API int s2d_spectrum(s2d_handle* h, double* Ek, int32_t nbins, double* tke, double* eps, double* enstDiss) {
    if (!h) return fail(S2D_ERR_INVALID, "null handle");
    const int nb = kIntMaxBins(h->grid.kxMG, h->grid.kyMG);
    if (Ek && nbins != nb) return fail(S2D_ERR_INVALID, "nbins=%d, expected %d", nbins, nb);
    S2D_CUDA(cudaSetDevice(h->device));
    std::vector<double> E;
    S2D_TRY(spectrum_impl(h, E));
    // src/Analysis.F90:414-448 (dk = 1): sums over bins in order
    double t = 0.0, e = 0.0, z = 0.0;
    for (int i = 0; i < nb; ++i) {
        const double k = (double)i;
        t = t + E[i] * 1.0;
        e = e + k * k * E[i] * 1.0;
        z = z + (k * k) * (k * k) * E[i] * 1.0;
    }
    if (Ek) std::memcpy(Ek, E.data(), sizeof(double) * nb);
    if (tke) *tke = t;
    if (eps) *eps = 2.0 * h->cfg.nu * e;
    if (enstDiss) *enstDiss = 2.0 * h->cfg.nu * z;
    return S2D_OK;
}

S2D_API int s2d_enstrophy(s2d_handle* h, double* out) {
    if (!h || !out) return fail(S2D_ERR_INVALID, "null argument");
    S2D_CUDA(cudaSetDevice(h->device));
    const int nblk = 304;
    if (h->prec == S2D_FP64) S2D_CUDA(Kern<double>::enstrophy_partial(h->d, h->S0, h->dscratch, nblk, h->stream));
    else S2D_CUDA(Kern<float>::enstrophy_partial(h->d, h->S0, h->dscratch, nblk, h->stream));
    std::vector<double> part(nblk);
    S2D_CUDA(cudaMemcpyAsync(part.data(), h->dscratch, sizeof(double) * nblk, cudaMemcpyDeviceToHost, h->stream));
    S2D_CUDA(cudaStreamSynchronize(h->stream));
    double s = 0.0;
    for (double p : part) s += p;
    *out = 0.5 * s;
    return S2D_OK;
}

S2D_API int s2d_minmax_abs(s2d_handle* h, double out[4]) {
    if (!h || !out) return fail(S2D_ERR_INVALID, "null argument");
    S2D_CUDA(cudaSetDevice(h->device));
    unsigned long long init[4];
    const double big = 1.0e308;
    init[0] = 0ULL;
    std::memcpy(&init[1], &big, 8);
    init[2] = 0ULL;
    std::memcpy(&init[3], &big, 8);
    S2D_CUDA(cudaMemcpyAsync(h->red64, init, sizeof(init), cudaMemcpyHostToDevice, h->stream));
    if (h->prec == S2D_FP64) S2D_CUDA(Kern<double>::minmax(h->d, h->S0, h->red64, h->stream));
    else S2D_CUDA(Kern<float>::minmax(h->d, h->S0, h->red64, h->stream));
    unsigned long long res[4];
    S2D_CUDA(cudaMemcpyAsync(res, h->red64, sizeof(res), cudaMemcpyDeviceToHost, h->stream));
    S2D_CUDA(cudaStreamSynchronize(h->stream));
    for (int i = 0; i < 4; ++i) std::memcpy(&out[i], &res[i], 8);
    // the reference array also stores the zero-padded modes beyond the
    // retained rectangle, so its minimum magnitude is zero
    out[1] = 0.0;
    out[3] = 0.0;
    return S2D_OK;
}

S2D_API int s2d_set_taylor_green(s2d_handle* h) {
    if (!h) return fail(S2D_ERR_INVALID, "null handle");
    S2D_CUDA(cudaSetDevice(h->device));
    const int M = h->d.M;
    // SIN(2 PI i / nxG) for 1-based i (src/SetIC.F90:91-94), FP64 libm
    std::vector<double> s(M);
    for (int i = 0; i < M; ++i) s[i] = std::sin(2.0 * M_PI * (double)(i + 1) / (double)M);
    double* ds = nullptr;
    S2D_CUDA(cudaMalloc(&ds, sizeof(double) * M));
    cudaError_t e = cudaMemcpyAsync(ds, s.data(), sizeof(double) * M, cudaMemcpyHostToDevice, h->stream);
    // physical omega in I[0..1] (M*M reals fit in 2 intermediates), its
    // x-spectrum in I[2], then the y-transform into S0
    if (e == cudaSuccess) {
        if (h->prec == S2D_FP64) {
            e = Kern<double>::fill_tg(h->d, ds, ds, h->I[0], h->stream);
            if (e == cudaSuccess) e = Kern<double>::xfwd_phys(h->d, h->I[0], h->I[2], h->tw, h->stream, h->L_xrow);
            if (e == cudaSuccess) e = Kern<double>::yfwd_store(h->d, h->I[2], h->S0, h->tw, h->stream, h->L_ystore);
        } else {
            e = Kern<float>::fill_tg(h->d, ds, ds, h->I[0], h->stream);
            if (e == cudaSuccess) e = Kern<float>::xfwd_phys(h->d, h->I[0], h->I[2], h->tw, h->stream, h->L_xrow);
            if (e == cudaSuccess) e = Kern<float>::yfwd_store(h->d, h->I[2], h->S0, h->tw, h->stream, h->L_ystore);
        }
    }
    cudaError_t e2 = cudaStreamSynchronize(h->stream);
    cudaFree(ds);
    if (e != cudaSuccess) return fail(S2D_ERR_CUDA, "Taylor-Green setup failed: %s", cudaGetErrorString(e));
    if (e2 != cudaSuccess) return fail(S2D_ERR_CUDA, "Taylor-Green setup failed: %s", cudaGetErrorString(e2));
    return S2D_OK;
}

S2D_API int s2d_cfl_dt(s2d_handle* h, double cfl, double* dt) {
    if (!h || !dt) return fail(S2D_ERR_INVALID, "null argument");
    if (!(cfl > 0.0)) return fail(S2D_ERR_INVALID, "cfl must be positive");
    S2D_CUDA(cudaSetDevice(h->device));
    FieldSet fs{};
    fs.nf = 2;
    fs.op[0] = OP_U;
    fs.op[1] = OP_V;
    fs.out[0] = h->I[0];
    fs.out[1] = h->I[1];
    S2D_CUDA(cudaMemsetAsync(h->red64, 0, sizeof(unsigned long long), h->stream));
    if (h->prec == S2D_FP64) {
        S2D_CUDA(Kern<double>::yinv(h->d, h->S0, h->rk2, fs, h->tw, h->stream, h->L_yinv));
        S2D_CUDA(Kern<double>::xinv_cfl(h->d, h->I[0], h->I[1], h->tw, h->red64, h->stream, h->L_xrow));
    } else {
        S2D_CUDA(Kern<float>::yinv(h->d, h->S0, h->rk2, fs, h->tw, h->stream, h->L_yinv));
        S2D_CUDA(Kern<float>::xinv_cfl(h->d, h->I[0], h->I[1], h->tw, h->red64, h->stream, h->L_xrow));
    }
    unsigned long long bits = 0;
    S2D_CUDA(cudaMemcpyAsync(&bits, h->red64, 8, cudaMemcpyDeviceToHost, h->stream));
    S2D_CUDA(cudaStreamSynchronize(h->stream));
    double m;
    std::memcpy(&m, &bits, 8);
    if (!(m > 0.0) || !std::isfinite(m)) return fail(S2D_ERR_NONFINITE, "max(|u|/dx+|v|/dy) = %g", m);
    *dt = cfl / m;
    return S2D_OK;
}

S2D_API int s2d_skewness(s2d_handle* h, double* xskew, double* yskew) {
    if (!h) return fail(S2D_ERR_INVALID, "null handle");
    S2D_CUDA(cudaSetDevice(h->device));
    const Dims& d = h->d;
    std::vector<double> rows(3 * (size_t)d.M);
    double sk[2];
    double* dev = nullptr;
    S2D_CUDA(cudaMalloc(&dev, rows.size() * sizeof(double)));
    // x: a = du/dx = i kx u, b = dw/dx (src/Analysis.F90:142-179);
    // y: a = dv/dy = i ky v, b = dw/dy (src/Analysis.F90:188-225)
    const int ops[2][2] = {{OP_UX, OP_WX}, {OP_VY, OP_WY}};
    int r = S2D_OK;
    for (int pass = 0; pass < 2 && r == S2D_OK; ++pass) {
        FieldSet fs{};
        fs.nf = 2;
        fs.op[0] = ops[pass][0];
        fs.op[1] = ops[pass][1];
        fs.out[0] = h->I[0];
        fs.out[1] = h->I[1];
        cudaError_t e;
        if (h->prec == S2D_FP64) {
            e = Kern<double>::yinv(d, h->S0, h->rk2, fs, h->tw, h->stream, h->L_yinv);
            if (e == cudaSuccess) e = Kern<double>::xinv_moments(d, h->I[0], h->I[1], h->tw, dev, h->stream, h->L_xrow);
        } else {
            e = Kern<float>::yinv(d, h->S0, h->rk2, fs, h->tw, h->stream, h->L_yinv);
            if (e == cudaSuccess) e = Kern<float>::xinv_moments(d, h->I[0], h->I[1], h->tw, dev, h->stream, h->L_xrow);
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(rows.data(), dev, rows.size() * sizeof(double),
                                                  cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) {
            r = fail(S2D_ERR_CUDA, "skewness: %s", cudaGetErrorString(e));
            break;
        }
        double s1 = 0.0, s2 = 0.0, s3 = 0.0;
        for (int y = 0; y < d.M; ++y) {
            s1 += rows[3 * y];
            s2 += rows[3 * y + 1];
            s3 += rows[3 * y + 2];
        }
        const double fact = (double)d.M * (double)d.M;
        s1 /= fact;
        s2 /= fact;
        s3 /= fact;
        sk[pass] = -2.0 * s1 / (std::sqrt(s2) * s3);
    }
    cudaFree(dev);
    if (r != S2D_OK) return r;
    if (xskew) *xskew = sk[0];
    if (yskew) *yskew = sk[1];
    return S2D_OK;
}

S2D_API int s2d_check_finite(s2d_handle* h) {
    if (!h) return fail(S2D_ERR_INVALID, "null handle");
    S2D_CUDA(cudaSetDevice(h->device));
    unsigned int f = 0;
    S2D_CUDA(cudaMemcpyAsync(&f, h->flags, sizeof(f), cudaMemcpyDeviceToHost, h->stream));
    S2D_CUDA(cudaMemsetAsync(h->flags, 0, sizeof(f), h->stream));
    S2D_CUDA(cudaStreamSynchronize(h->stream));
    if (f & 1u) return fail(S2D_ERR_NONFINITE, "non-finite vorticity written by a stage update");
    return S2D_OK;
}

S2D_API int s2d_synchronize(s2d_handle* h) {
    if (!h) return fail(S2D_ERR_INVALID, "null handle");
    S2D_CUDA(cudaSetDevice(h->device));
    S2D_CUDA(cudaStreamSynchronize(h->stream));
    return S2D_OK;
}

S2D_API int s2d_time_steps(s2d_handle* h, int32_t n, double dt, double* ms, double* kernel_ms) {
    if (!h || !ms || n <= 0) return fail(S2D_ERR_INVALID, "bad argument");
    S2D_CUDA(cudaSetDevice(h->device));
    cudaEvent_t e0, e1;
    S2D_CUDA(cudaEventCreate(&e0));
    S2D_CUDA(cudaEventCreate(&e1));
    int r = S2D_OK;
    if (!kernel_ms) {
        if (!h->gexec || h->graph_dt != dt) r = build_graph(h, dt);
        if (r == S2D_OK) {
            S2D_CUDA(cudaStreamSynchronize(h->stream));
            S2D_CUDA(cudaEventRecord(e0, h->stream));
            for (int i = 0; i < n && r == S2D_OK; ++i)
                if (cudaGraphLaunch(h->gexec, h->stream) != cudaSuccess) r = fail(S2D_ERR_CUDA, "graph launch failed");
            S2D_CUDA(cudaEventRecord(e1, h->stream));
        }
    } else {
        const int nev = 3 * 4 * n;
        std::vector<cudaEvent_t> ev(nev);
        for (auto& e : ev) S2D_CUDA(cudaEventCreate(&e));
        S2D_CUDA(cudaStreamSynchronize(h->stream));
        S2D_CUDA(cudaEventRecord(e0, h->stream));
        for (int i = 0; i < n && r == S2D_OK; ++i)
            for (int s = 1; s <= 3 && r == S2D_OK; ++s) r = launch_rhs_stage_any(h, s, dt, &ev[(i * 3 + s - 1) * 4]);
        S2D_CUDA(cudaEventRecord(e1, h->stream));
        S2D_CUDA(cudaEventSynchronize(e1));
        kernel_ms[0] = kernel_ms[1] = kernel_ms[2] = 0.0;
        if (r == S2D_OK)
            for (int q = 0; q < 3 * n; ++q)
                for (int k = 0; k < 3; ++k) {
                    float t = 0.f;
                    cudaEventElapsedTime(&t, ev[q * 4 + k], ev[q * 4 + k + 1]);
                    kernel_ms[k] += t;
                }
        for (auto& e : ev) cudaEventDestroy(e);
    }
    S2D_CUDA(cudaEventSynchronize(e1));
    float t = 0.f;
    S2D_CUDA(cudaEventElapsedTime(&t, e0, e1));
    *ms = t;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return r;
}

S2D_API int s2d_kernels_per_step(const s2d_handle* h) {
    if (!h) return fail(S2D_ERR_INVALID, "null handle");
    return h->Fv ? 12 : 9;
}

S2D_API int s2d_host_alloc(size_t bytes, void** ptr) {
    if (!ptr) return fail(S2D_ERR_INVALID, "null argument");
    S2D_CUDA(cudaMallocHost(ptr, bytes));
    return S2D_OK;
}

S2D_API int s2d_host_free(void* ptr) {
    if (ptr) S2D_CUDA(cudaFreeHost(ptr));
    return S2D_OK;
}

S2D_API int s2d_probe_fp64_peak(int32_t device, double* tflops) {
    if (!tflops) return fail(S2D_ERR_INVALID, "null argument");
    S2D_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop{};
    S2D_CUDA(cudaGetDeviceProperties(&prop, device));
    double* sink = nullptr;
    S2D_CUDA(cudaMalloc(&sink, 1024 * sizeof(double)));
    cudaStream_t st;
    S2D_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    const int threads = 256, blocks = prop.multiProcessorCount * 8, iters = 4096;
    cudaEvent_t e0, e1;
    S2D_CUDA(cudaEventCreate(&e0));
    S2D_CUDA(cudaEventCreate(&e1));
    S2D_CUDA(launch_fp64_probe(sink, blocks, threads, iters, st));  // warm-up
    S2D_CUDA(cudaEventRecord(e0, st));
    const int reps = 5;
    for (int i = 0; i < reps; ++i) S2D_CUDA(launch_fp64_probe(sink, blocks, threads, iters, st));
    S2D_CUDA(cudaEventRecord(e1, st));
    S2D_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    S2D_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    const double flops = 2.0 * 8.0 * iters * (double)threads * blocks * reps;
    *tflops = flops / (ms * 1e-3) / 1e12;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    cudaFree(sink);
    return S2D_OK;
}

}  // extern "C"
