// s2d_slab.cu -- one rank's slab of a run decomposed over several ranks.
//
// The reference splits one run over MPI ranks in slabs and lets FFTW-MPI do
// an all-to-all transpose inside every 2-D transform (src/Alloc.F90:90-100,
// src/Spectral.F90:340-349, :760, :780).  Here the decomposition follows the
// two-pass structure of the right-hand side instead:
//
//   phase 0  K1, the inverse y-pass, on the rank's kx columns
//            [kx0, kx0 + nkx) of the spectral state (all M physical rows of
//            u and v), then the first send buffer is packed;
//   (caller) all-to-all: segment s of the send buffer goes to rank s;
//   phase 1  the received blocks are unpacked, K2 (inverse x-FFT, products,
//            forward x-FFT) runs on the rank's physical rows [y0, y0 + ny)
//            (all kx columns), then the second send buffer is packed;
//   (caller) all-to-all;
//   phase 2  unpacked, then K3 (forward y-pass and the RK3 stage update of
//            src/TimeIntegration.F90:156-209 with Truncate) on the rank's kx
//            columns.
//
// Two transposes per right-hand side, six per RK3 step.  The kernels are the
// single-run kernels, handed a column view of the arrays (Dims::KX = nkx,
// Dims::kx0 = kx0, pointers moved to column kx0) or a row range (Dims::rows),
// so every column and row is computed by the same code in the same order as
// in a single run: a decomposed run equals the single run bit for bit.  The
// library moves no data between ranks: the caller's all-to-all does (MPI,
// NCCL, or plain copies when the ranks share a process), as FFTW-MPI's
// caller provides the communicator.
//
// Pack layout.  Exchange 0 (after K1): send segment s holds, for field f in
// (u, v), rows [y0_s, y0_s + ny_s) x this rank's columns, row-major
// ([f][row][col]); receive segment s holds this rank's rows x rank s's
// columns.  Exchange 1 (after K2): send segment s holds this rank's rows x
// rank s's columns; receive segment s holds rank s's rows x this rank's
// columns.  Segments follow one another in rank order.
#include "s2d.h"
#include "s2d_fft.cuh"
#include "s2d_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <new>

namespace s2d {
namespace {

constexpr int kMaxRanks = S2D_SLAB_MAX_RANKS;

struct Segs {
    int r0[kMaxRanks], c0[kMaxRanks], nr[kMaxRanks], nc[kMaxRanks];
    long long off[kMaxRanks];   // element offset of the segment in the buffer
};

// blockIdx.y = segment, blockIdx.z = field: the block rows x cols of field f
// of the half-spectral arrays to (PACK) or from the packed buffer
template <typename VT, bool PACK>
__global__ void __launch_bounds__(256) k_slab_copy(VT* I0, VT* I1, int ldI, Segs sg, VT* buf) {
    const int seg = blockIdx.y, f = blockIdx.z;
    VT* I = f ? I1 : I0;
    const int nr = sg.nr[seg], nc = sg.nc[seg], r0 = sg.r0[seg], c0 = sg.c0[seg];
    const long long base = sg.off[seg] + (long long)f * nr * nc;
    for (int i = blockIdx.x; i < nr; i += gridDim.x) {
        VT* row = I + (size_t)(r0 + i) * ldI + c0;
        VT* b = buf + base + (long long)i * nc;
        for (int j = threadIdx.x; j < nc; j += blockDim.x) {
            if (PACK) b[j] = row[j];
            else row[j] = b[j];
        }
    }
}

}  // namespace
}  // namespace s2d

using namespace s2d;

struct s2d_slab {
    s2d_handle* h = nullptr;
    int rank = 0, nranks = 1;
    int kx0[kMaxRanks] = {}, nkx[kMaxRanks] = {}, y0[kMaxRanks] = {}, ny[kMaxRanks] = {};
    void* send = nullptr;
    void* recv = nullptr;
    size_t buf_elems = 0;
    double* stage_ref = nullptr;   // reference-layout staging of get_columns
};

namespace {

void partition(int KX, int M, int P, int* kx0, int* nkx, int* y0, int* ny) {
    for (int r = 0; r < P; ++r) {
        kx0[r] = (int)((long long)r * KX / P);
        nkx[r] = (int)((long long)(r + 1) * KX / P) - kx0[r];
        y0[r] = (int)((long long)r * M / P);
        ny[r] = (int)((long long)(r + 1) * M / P) - y0[r];
    }
}

// segment tables of exchange e: the send side (pack) and the receive side (unpack)
void segments(const s2d_slab* s, int e, Segs* snd, Segs* rcv) {
    const int r = s->rank;
    long long os = 0, orv = 0;
    for (int q = 0; q < s->nranks; ++q) {
        if (e == 0) {   // after K1: rows of q x my columns out; my rows x columns of q in
            snd->r0[q] = s->y0[q]; snd->nr[q] = s->ny[q]; snd->c0[q] = s->kx0[r]; snd->nc[q] = s->nkx[r];
            rcv->r0[q] = s->y0[r]; rcv->nr[q] = s->ny[r]; rcv->c0[q] = s->kx0[q]; rcv->nc[q] = s->nkx[q];
        } else {        // after K2: my rows x columns of q out; rows of q x my columns in
            snd->r0[q] = s->y0[r]; snd->nr[q] = s->ny[r]; snd->c0[q] = s->kx0[q]; snd->nc[q] = s->nkx[q];
            rcv->r0[q] = s->y0[q]; rcv->nr[q] = s->ny[q]; rcv->c0[q] = s->kx0[r]; rcv->nc[q] = s->nkx[r];
        }
        snd->off[q] = os;
        rcv->off[q] = orv;
        os += 2LL * snd->nr[q] * snd->nc[q];
        orv += 2LL * rcv->nr[q] * rcv->nc[q];
    }
}

template <typename T>
cudaError_t slab_copy(s2d_slab* s, const Segs& sg, bool pack, void* buf) {
    using VT = typename Vec<T>::t;
    s2d_handle* h = s->h;
    const dim3 grid(std::max(1, std::min(1024, h->d.M / s->nranks)), s->nranks, 2);
    if (pack)
        k_slab_copy<VT, true><<<grid, 256, 0, h->stream>>>((VT*)h->I[0], (VT*)h->I[1], h->d.ldI, sg, (VT*)buf);
    else
        k_slab_copy<VT, false><<<grid, 256, 0, h->stream>>>((VT*)h->I[0], (VT*)h->I[1], h->d.ldI, sg, (VT*)buf);
    return cudaGetLastError();
}

template <typename T>
int slab_phase(s2d_slab* s, int stage, int phase, double dt) {
    using VT = typename Vec<T>::t;
    s2d_handle* h = s->h;
    const int r = s->rank;
    const int c0 = s->kx0[r];
    Dims dv = h->d;   // column view: columns [c0, c0 + nkx) as columns 0..nkx-1
    dv.KX = s->nkx[r];
    dv.kx0 = c0;
    const size_t cs = (size_t)c0 * h->d.ldS;   // column offset in the compact arrays
    Segs snd{}, rcv{};
    auto launch = [](Launch L) { L.pdl = false; return L; };
    cudaError_t e = cudaSuccess;
    if (phase == 0) {
        FieldSet fs{};
        fs.nf = 2;
        fs.op[0] = OP_TU;
        fs.op[1] = OP_TV;
        fs.tab[0] = h->fu + cs;
        fs.tab[1] = h->fv + cs;
        fs.tabf[0] = h->fu32 ? h->fu32 + cs : nullptr;
        fs.tabf[1] = h->fv32 ? h->fv32 + cs : nullptr;
        fs.out[0] = (VT*)h->I[0] + c0;
        fs.out[1] = (VT*)h->I[1] + c0;
        const VT* win = (const VT*)((stage <= 1) ? h->S0 : h->S1) + cs;
        e = Kern<T>::yinv(dv, win, h->rk2s + cs, fs, h->tw, h->stream, launch(h->L_yinv));
        if (e == cudaSuccess) {
            segments(s, 0, &snd, &rcv);
            e = slab_copy<T>(s, snd, true, s->send);
        }
    } else if (phase == 1) {
        segments(s, 0, &snd, &rcv);
        e = slab_copy<T>(s, rcv, false, s->recv);
        if (e == cudaSuccess) {
            Dims dr = h->d;   // row range [y0, y0 + ny)
            dr.rows = s->ny[r];
            const size_t ro = (size_t)s->y0[r] * h->d.ldI;
            e = Kern<T>::xpass_bas(dr, (VT*)h->I[0] + ro, (VT*)h->I[1] + ro, h->tw, h->stream, launch(h->L_xrow),
                                   true);
        }
        if (e == cudaSuccess) {
            segments(s, 1, &snd, &rcv);
            e = slab_copy<T>(s, snd, true, s->send);
        }
    } else {
        segments(s, 1, &snd, &rcv);
        e = slab_copy<T>(s, rcv, false, s->recv);
        VT* S0 = (VT*)h->S0 + cs;
        VT* S1 = (VT*)h->S1 + cs;
        if (e == cudaSuccess && h->Fv) {   // the single run's split K3 (FP64)
            VT* Fu = (VT*)h->I[2] + cs;
            VT* Fv = (VT*)h->Fv + cs;
            e = Kern<T>::yfwd_col(dv, (VT*)h->I[0] + c0, (VT*)h->I[1] + c0, Fu, Fv, h->tw, h->stream,
                                  launch(h->L_ycol));
            if (e == cudaSuccess)
                e = Kern<T>::stage(dv, Fu, Fv, S0, S1, nullptr, nullptr, stage, dt, h->ph, h->flags, h->stream,
                                   false, h->cc + 2 * cs, h->vk + cs);
        } else if (e == cudaSuccess) {     // the fused K3 (FP32)
            e = Kern<T>::yfwd_rk3(dv, (VT*)h->I[0] + c0, (VT*)h->I[1] + c0, S0, S1, nullptr, nullptr, stage, dt,
                                  h->ph, h->tw, h->flags, h->stream, launch(h->L_yfwd));
        }
    }
    if (e != cudaSuccess) return set_error(S2D_ERR_CUDA, cudaGetErrorString(e));
    return S2D_OK;
}

}  // namespace

extern "C" {

S2D_API int s2d_slab_partition(int32_t nx, int32_t nranks, int32_t rank, int32_t part[4]) {
    if (!part || nx < 8 || nx % 8 || nranks < 1 || nranks > kMaxRanks || rank < 0 || rank >= nranks)
        return set_error(S2D_ERR_INVALID, "bad nx, nranks or rank");
    const int K = nx / 2, KX = K + 1, M = 3 * nx / 2;
    if (nranks > KX) return set_error(S2D_ERR_INVALID, "more ranks than kx columns");
    int a[kMaxRanks], b[kMaxRanks], c[kMaxRanks], d[kMaxRanks];
    partition(KX, M, nranks, a, b, c, d);
    part[0] = a[rank];
    part[1] = b[rank];
    part[2] = c[rank];
    part[3] = d[rank];
    return S2D_OK;
}

S2D_API int s2d_slab_create(const s2d_config* cfg, int32_t rank, int32_t nranks, s2d_slab** out) {
    if (!cfg || !out) return set_error(S2D_ERR_INVALID, "null argument");
    *out = nullptr;
    if (nranks < 1 || nranks > kMaxRanks || rank < 0 || rank >= nranks)
        return set_error(S2D_ERR_INVALID, "rank or nranks out of range");
    if (cfg->nonlinear_form != S2D_NL_BASDEVANT)
        return set_error(S2D_ERR_UNSUPPORTED, "a slab runs the Basdevant form of the nonlinear term");
    s2d_slab* s = new (std::nothrow) s2d_slab();
    if (!s) return set_error(S2D_ERR_NOMEM, "host allocation failed");
    int r = create_handle(cfg, nullptr, &s->h);
    if (r != S2D_OK) {
        delete s;
        return r;
    }
    s2d_handle* h = s->h;
    if (nranks > h->d.KX) {
        s2d_slab_destroy(s);
        return set_error(S2D_ERR_INVALID, "more ranks than kx columns");
    }
    s->rank = rank;
    s->nranks = nranks;
    partition(h->d.KX, h->d.M, nranks, s->kx0, s->nkx, s->y0, s->ny);
    // largest side of either exchange: 2 M nkx (exchange 0 out, 1 in) or 2 ny KX
    s->buf_elems = std::max((size_t)2 * h->d.M * s->nkx[rank], (size_t)2 * s->ny[rank] * h->d.KX);
    const size_t bytes = s->buf_elems * h->vsz;
    if (cudaMalloc(&s->send, bytes) != cudaSuccess || cudaMalloc(&s->recv, bytes) != cudaSuccess ||
        cudaMalloc((void**)&s->stage_ref, 2 * h->ref_bytes) != cudaSuccess) {
        s2d_slab_destroy(s);
        return set_error(S2D_ERR_NOMEM, "cudaMalloc of the exchange buffers failed");
    }
    *out = s;
    return S2D_OK;
}

S2D_API void s2d_slab_destroy(s2d_slab* s) {
    if (!s) return;
    if (s->h) cudaSetDevice(s->h->device);
    cudaFree(s->send);
    cudaFree(s->recv);
    cudaFree(s->stage_ref);
    s2d_destroy(s->h);
    delete s;
}

S2D_API int s2d_slab_handle(s2d_slab* s, s2d_handle** h) {
    if (!s || !h) return set_error(S2D_ERR_INVALID, "null argument");
    *h = s->h;
    return S2D_OK;
}

S2D_API int s2d_slab_exchange(s2d_slab* s, int32_t exchange, void** send, void** recv, int64_t* send_bytes,
                              int64_t* recv_bytes) {
    if (!s || (exchange != 0 && exchange != 1)) return set_error(S2D_ERR_INVALID, "bad slab or exchange");
    Segs snd{}, rcv{};
    segments(s, exchange, &snd, &rcv);
    if (send) *send = s->send;
    if (recv) *recv = s->recv;
    for (int q = 0; q < s->nranks; ++q) {
        if (send_bytes) send_bytes[q] = 2LL * snd.nr[q] * snd.nc[q] * (int64_t)s->h->vsz;
        if (recv_bytes) recv_bytes[q] = 2LL * rcv.nr[q] * rcv.nc[q] * (int64_t)s->h->vsz;
    }
    return S2D_OK;
}

S2D_API int s2d_slab_phase(s2d_slab* s, int32_t stage, int32_t phase, double dt) {
    if (!s || stage < 1 || stage > 3 || phase < 0 || phase > 2 || !std::isfinite(dt))
        return set_error(S2D_ERR_INVALID, "bad slab, stage, phase or dt");
    if (cudaSetDevice(s->h->device) != cudaSuccess) return set_error(S2D_ERR_CUDA, "cudaSetDevice failed");
    return s->h->prec == S2D_FP64 ? slab_phase<double>(s, stage, phase, dt) : slab_phase<float>(s, stage, phase, dt);
}

S2D_API int s2d_slab_get_columns(s2d_slab* s, double* wC, double* psiC, int32_t cISize, int32_t nyG) {
    if (!s || (!wC && !psiC)) return set_error(S2D_ERR_INVALID, "null argument");
    s2d_handle* h = s->h;
    if (cISize != h->grid.cISize || nyG != h->grid.nyG) return set_error(S2D_ERR_INVALID, "array shape mismatch");
    if (cudaSetDevice(h->device) != cudaSuccess) return set_error(S2D_ERR_CUDA, "cudaSetDevice failed");
    const int r = s->rank, c0 = s->kx0[r], K = h->d.K, M = h->d.M, C = cISize;
    Dims dv = h->d;
    dv.KX = s->nkx[r];
    dv.kx0 = c0;
    const size_t cs = (size_t)c0 * h->d.ldS;
    double* sw = s->stage_ref;
    double* sp = (double*)((char*)s->stage_ref + h->ref_bytes);
    cudaError_t e = h->prec == S2D_FP64
                        ? Kern<double>::compact_to_rect(dv, (const double2*)h->S0 + cs, C, sw + 2 * c0, sp + 2 * c0,
                                                        h->stream)
                        : Kern<float>::compact_to_rect(dv, (const float2*)h->S0 + cs, C, sw + 2 * c0, sp + 2 * c0,
                                                       h->stream);
    const size_t pitch = (size_t)C * 2 * sizeof(double), width = (size_t)s->nkx[r] * 2 * sizeof(double);
    const size_t lo = (size_t)(M - K) * pitch, col = (size_t)c0 * 2 * sizeof(double);
    for (int a = 0; a < 2 && e == cudaSuccess; ++a) {
        double* dst = a == 0 ? wC : psiC;
        const char* src = (const char*)(a == 0 ? sw : sp);
        if (!dst) continue;
        e = cudaMemcpy2DAsync((char*)dst + col, pitch, src + col, pitch, width, K + 1, cudaMemcpyDefault, h->stream);
        if (e == cudaSuccess)
            e = cudaMemcpy2DAsync((char*)dst + lo + col, pitch, src + lo + col, pitch, width, K, cudaMemcpyDefault,
                                  h->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return set_error(S2D_ERR_CUDA, cudaGetErrorString(e));
    return S2D_OK;
}

}  // extern "C"
