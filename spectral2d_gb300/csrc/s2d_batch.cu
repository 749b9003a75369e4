// s2d_batch.cu -- ensembles of independent runs of uneven sizes, advanced by
// one persistent launch per RK3 stage (three per step), replayed from a CUDA
// graph.
//
// Work of one stage = for every run: K1 tiles (inverse y-pass), K2 tiles
// (x-pass), K3 tiles (forward y-pass + stage update).  Tasks (run, phase,
// tile) sit in one table ordered phase-major; CTAs of the persistent grid take
// them in order from an atomic counter.  A K2 tile of run r needs every K1
// tile of r, a K3 tile every K2 tile of r: the CTA waits (bounded spin) on
// r's per-phase completion counter.  Every task it waits for was taken
// earlier by a CTA that is already running and itself only waits for earlier
// tasks, so the queue cannot deadlock even when not all CTAs are resident.
// A wait that exceeds the iteration limit sets S2D_ERR_TIMEOUT's flag and
// skips the task instead of hanging.  The last CTA to leave resets the
// counters, so the next replay starts clean.
//
// Every task uses the whole CTA: K1/K2 tiles hold G = threads/Tg transforms,
// K3 tiles threads/(2 Tg) columns x 2 fields, so one task is 12*threads
// complex elements of shared memory whatever the run's size (Tg = M/12 must
// divide the CTA size: nx a power of two from 16 to 2048).
//
// The tuner (s2d_batch_tune) times candidate tile schedules -- threads per
// CTA (and so transforms per tile) and CTAs per SM -- on the actual ensemble
// and keeps the fastest; the state is restored afterwards.
#include "s2d.h"
#include "s2d_internal.h"
#include "s2d_step.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <vector>

namespace s2d {

template <typename T>
struct RunDev {
    Dims d;
    Phys ph;
    typename Vec<T>::t* S0;
    typename Vec<T>::t* S1;
    typename Vec<T>::t* I0;
    typename Vec<T>::t* I1;
    const typename Vec<T>::t* src;   // closure term added to dW, or null
    const double* rk2;
    const typename Vec<T>::t* tw;
    double dt;
    int G12;        // transforms per K1 / K2 tile
    int G3;         // columns per K3 tile
    int ntask[3];   // tiles per phase
    int pad;
};

constexpr int kSpinLimit = 1 << 22;   // ~1 s of 200 ns sleeps

__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// X32: the batch holds an FP32 run of M = 3072, whose x-pass tiles take the
// register radix-12/16 body of the single run (k_xpass32).  That body needs
// 128 registers in this kernel, the rest 64, so only such batches get the
// variant that contains it (at 64 registers a 256^2 FP32 stage took 1.11
// instead of 1.62 ms).
template <typename T, bool X32>
__global__ void __launch_bounds__(512) k_batch_stage(const RunDev<T>* __restrict__ runs, int nruns,
                                                     const int4* __restrict__ tasks, int ntasks, int stage,
                                                     int* ctrl, int* done, unsigned int* flags) {
    using VT = typename Vec<T>::t;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    VT* bufs = reinterpret_cast<VT*>(smem_raw);
    __shared__ RunDev<T> R;
    __shared__ int s_task, s_ok, s_last;
    bool bad = false;
    for (;;) {
        if (threadIdx.x == 0) s_task = atomicAdd(&ctrl[0], 1);
        __syncthreads();
        const int t = s_task;
        if (t >= ntasks) break;
        const int4 tk = tasks[t];
        const int r = tk.x, ph = tk.y, blk = tk.z;
        {
            const int* src = reinterpret_cast<const int*>(&runs[r]);
            int* dst = reinterpret_cast<int*>(&R);
            for (int i = threadIdx.x; i < (int)(sizeof(RunDev<T>) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
        }
        if (threadIdx.x == 0) {
            int ok = 1;
            if (ph > 0) {
                const int need = runs[r].ntask[ph - 1];
                int it = 0;
                while (ld_acquire(&done[r * 3 + ph - 1]) < need) {
                    if (++it > kSpinLimit) {
                        ok = 0;
                        atomicOr(flags, 2u);
                        break;
                    }
                    __nanosleep(200);
                }
            }
            s_ok = ok;
        }
        __syncthreads();
        if (s_ok) {
            if (ph == 0) {
                FieldSet fs{};
                fs.nf = 2;
                fs.op[0] = OP_U;
                fs.op[1] = OP_V;
                fs.out[0] = R.I0;
                fs.out[1] = R.I1;
                yinv_body<T>(R.d, stage <= 1 ? R.S0 : R.S1, R.rk2, fs, R.tw, R.G12, blk, bufs);
            } else if (ph == 1) {
                bool done32 = false;
                if constexpr (sizeof(T) == 4 && X32) {
                    // FP32 rows of M = 3072: the register radix-12/16 x-pass of
                    // the single run (k_xpass32), one row per 256 threads
                    if (R.d.M == kX32M && !R.d.xgen) {
                        const int g = threadIdx.x / 256, y = blk * R.G12 + g;
                        xpass32_m3072_row(R.d, R.I0, R.I1, R.tw, y, y < R.d.rows && g < R.G12,
                                          threadIdx.x - g * 256, bufs + (size_t)g * kX32Buf);
                        done32 = true;
                    }
                }
                if (!done32) xpass_bas_body<T>(R.d, R.I0, R.I1, R.tw, R.G12, (T)1, blk, bufs);
            } else {
                bad |= yfwd_body<T>(R.d, R.I0, R.I1, R.S0, R.S1, nullptr, R.src, stage, R.dt, R.ph, R.tw, R.G3,
                                    blk, bufs);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(&done[r * 3 + ph], 1);
        }
    }
    if (bad) atomicOr(flags, 1u);
    // the last CTA to leave resets the queue and the counters
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = (atomicAdd(&ctrl[1], 1) == (int)gridDim.x - 1);
    }
    __syncthreads();
    if (s_last) {
        for (int i = threadIdx.x; i < 3 * nruns; i += blockDim.x) done[i] = 0;
        if (threadIdx.x == 0) {
            ctrl[0] = 0;
            ctrl[1] = 0;
        }
        __threadfence();
    }
}

}  // namespace s2d

using namespace s2d;

struct s2d_batch {
    int n = 0;
    int prec = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<s2d_handle*> runs;
    std::vector<double> dt;
    void* d_runs = nullptr;
    int4* d_tasks = nullptr;
    int ntasks = 0;
    int* d_ctrl = nullptr;
    int* d_done = nullptr;
    unsigned int* d_flags = nullptr;
    int threads = 256;
    int ctas_per_sm = 0;
    int grid = 0;
    size_t smem = 0;
    int sms = 0;
    int max_smem = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    s2d_cnn* cnn = nullptr;   // closure network of every run (LES batches)
    void* cl_tab = nullptr;   // its device table (closure_table)
    int stall_run = -1;       // s2d_batch_inject_stall
    bool x32 = false;         // an FP32 run of M = 3072: the k_batch_stage variant with k_xpass32's body
};

namespace {

int berr(int code, const char* m) { return set_error(code, m); }

#define B_CUDA(call)                                                        \
    do {                                                                    \
        cudaError_t e_ = (call);                                            \
        if (e_ != cudaSuccess) return berr(S2D_ERR_CUDA, cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
cudaError_t launch_stage(s2d_batch* b, int stage) {
    if (b->x32)
        k_batch_stage<T, true><<<b->grid, b->threads, b->smem, b->stream>>>(
            (const RunDev<T>*)b->d_runs, b->n, b->d_tasks, b->ntasks, stage, b->d_ctrl, b->d_done, b->d_flags);
    else
        k_batch_stage<T, false><<<b->grid, b->threads, b->smem, b->stream>>>(
            (const RunDev<T>*)b->d_runs, b->n, b->d_tasks, b->ntasks, stage, b->d_ctrl, b->d_done, b->d_flags);
    return cudaGetLastError();
}

cudaError_t launch_step(s2d_batch* b) {
    if (b->cnn && closure_terms(b->cnn, b->runs.data(), b->n, b->cl_tab, b->stream) != S2D_OK)
        return cudaErrorUnknown;
    for (int s = 1; s <= 3; ++s) {
        cudaError_t e = b->prec == S2D_FP64 ? launch_stage<double>(b, s) : launch_stage<float>(b, s);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

void drop_graph(s2d_batch* b) {
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->gexec = nullptr;
    b->graph = nullptr;
}

// Tile shapes for a CTA of `threads`, the task table and the run table.
template <typename T>
int configure(s2d_batch* b, int threads, int ctas_per_sm) {
    using VT = typename Vec<T>::t;
    std::vector<RunDev<T>> rd(b->n);
    size_t smem = 0;
    std::vector<int4> tasks[3];
    for (int i = 0; i < b->n; ++i) {
        const s2d_handle* h = b->runs[i];
        RunDev<T>& R = rd[i];
        std::memset(&R, 0, sizeof(R));
        R.d = h->d;
        R.ph = h->ph;
        R.S0 = (VT*)h->S0;
        R.S1 = (VT*)h->S1;
        R.I0 = (VT*)h->I[0];
        R.I1 = (VT*)h->I[1];
        R.src = b->cnn ? (const VT*)h->src : nullptr;
        R.rk2 = h->rk2s;   // Basdevant runs: u, v prescaled (no scale in the x-pass)
        R.tw = (const VT*)h->tw;
        R.dt = b->dt[i];
        const int Tg = h->d.Tg;
        if (Tg > threads || threads % Tg) return berr(S2D_ERR_UNSUPPORTED, "tile shape does not fit a run");
        R.G12 = threads / Tg;
        R.G3 = std::max(1, threads / (2 * Tg));
        R.ntask[0] = 2 * ((h->d.KX + R.G12 - 1) / R.G12);
        R.ntask[1] = (h->d.M + R.G12 - 1) / R.G12;
        R.ntask[2] = (h->d.KX + R.G3 - 1) / R.G3;
        smem = std::max(smem, (size_t)R.G12 * h->d.M * sizeof(VT));
        if (sizeof(T) == 4 && h->d.M == kX32M)   // the register radix-12/16 x-pass (s2d_xpass32.cuh)
            smem = std::max(smem, (size_t)R.G12 * kX32Buf * sizeof(VT));
        smem = std::max(smem, (size_t)2 * R.G3 * h->d.M * sizeof(VT));
        for (int p = 0; p < 3; ++p)
            for (int k = 0; k < R.ntask[p]; ++k) tasks[p].push_back(make_int4(i, p, k, 0));
        // injected stall: the x-pass tiles of this run wait for one more
        // inverse y-pass tile than the table holds, so their bounded waits
        // run out (S2D_ERR_TIMEOUT) -- a host-made fault for tests
        if (i == b->stall_run) R.ntask[0] += 1;
    }
    if (smem > (size_t)b->max_smem) return berr(S2D_ERR_UNSUPPORTED, "tile needs too much shared memory");
    std::vector<int4> all;
    for (int p = 0; p < 3; ++p) all.insert(all.end(), tasks[p].begin(), tasks[p].end());
    int occ = 0;
    if (b->x32)
        B_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batch_stage<T, true>, threads, smem));
    else
        B_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batch_stage<T, false>, threads, smem));
    if (occ < 1) return berr(S2D_ERR_UNSUPPORTED, "persistent kernel does not fit an SM");
    const int cps = ctas_per_sm > 0 ? std::min(ctas_per_sm, occ) : occ;
    B_CUDA(cudaStreamSynchronize(b->stream));
    if (b->d_tasks) cudaFree(b->d_tasks);
    b->d_tasks = nullptr;
    B_CUDA(cudaMalloc(&b->d_tasks, all.size() * sizeof(int4)));
    B_CUDA(cudaMemcpy(b->d_tasks, all.data(), all.size() * sizeof(int4), cudaMemcpyHostToDevice));
    B_CUDA(cudaMemcpy(b->d_runs, rd.data(), rd.size() * sizeof(RunDev<T>), cudaMemcpyHostToDevice));
    b->ntasks = (int)all.size();
    b->threads = threads;
    b->ctas_per_sm = cps;
    b->grid = cps * b->sms;
    b->smem = smem;
    drop_graph(b);
    return S2D_OK;
}

int configure_any(s2d_batch* b, int threads, int cps) {
    return b->prec == S2D_FP64 ? configure<double>(b, threads, cps) : configure<float>(b, threads, cps);
}

int upload_dt(s2d_batch* b) {
    const size_t rsz = b->prec == S2D_FP64 ? sizeof(RunDev<double>) : sizeof(RunDev<float>);
    const size_t off = b->prec == S2D_FP64 ? offsetof(RunDev<double>, dt) : offsetof(RunDev<float>, dt);
    for (int i = 0; i < b->n; ++i)
        B_CUDA(cudaMemcpyAsync((char*)b->d_runs + i * rsz + off, &b->dt[i], sizeof(double), cudaMemcpyHostToDevice,
                               b->stream));
    B_CUDA(cudaStreamSynchronize(b->stream));
    return S2D_OK;
}

int build_graph(s2d_batch* b) {
    drop_graph(b);
    B_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = launch_step(b);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return berr(S2D_ERR_CUDA, "batch graph capture failed");
    }
    b->graph = g;
    B_CUDA(cudaGraphInstantiate(&b->gexec, g, 0));
    return S2D_OK;
}

}  // namespace

extern "C" {

S2D_API int s2d_batch_create(int32_t nruns, const s2d_config* cfgs, s2d_batch** out) {
    if (!cfgs || !out || nruns <= 0) return berr(S2D_ERR_INVALID, "bad batch arguments");
    *out = nullptr;
    for (int i = 0; i < nruns; ++i) {
        const int nx = cfgs[i].nx;
        if (nx < 16 || nx > 2048 || (nx & (nx - 1)))
            return berr(S2D_ERR_UNSUPPORTED, "batch runs need nx a power of two in [16, 2048]");
        if (cfgs[i].precision != cfgs[0].precision || cfgs[i].device != cfgs[0].device)
            return berr(S2D_ERR_INVALID, "batch runs must share precision and device");
        if (cfgs[i].nonlinear_form != S2D_NL_BASDEVANT)
            return berr(S2D_ERR_UNSUPPORTED, "batch runs use the Basdevant form");
    }
    s2d_batch* b = new (std::nothrow) s2d_batch();
    if (!b) return berr(S2D_ERR_NOMEM, "host allocation failed");
    b->n = nruns;
    b->prec = cfgs[0].precision;
    b->device = cfgs[0].device;
    b->dt.assign(nruns, 0.0);
    auto bail = [&](int code) {
        s2d_batch_destroy(b);
        return code;
    };
    if (cudaSetDevice(b->device) != cudaSuccess) return bail(berr(S2D_ERR_CUDA, "cudaSetDevice failed"));
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(berr(S2D_ERR_CUDA, "stream creation failed"));
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, b->device) != cudaSuccess) return bail(berr(S2D_ERR_CUDA, "device query"));
    b->sms = prop.multiProcessorCount;
    b->max_smem = (int)prop.sharedMemPerBlockOptin - 1024;
    for (int i = 0; i < nruns; ++i) {
        s2d_handle* h = nullptr;
        const int r = create_handle(&cfgs[i], b->stream, &h);
        if (r != S2D_OK) return bail(r);
        b->runs.push_back(h);
        if (h->prec == S2D_FP32 && h->d.M == kX32M && !h->d.xgen) b->x32 = true;
    }
    {
        static std::atomic<bool> attr[64];  // per device, set once the attributes are (a second setter only repeats them)
        if (b->device >= 0 && b->device < 64 && !attr[b->device]) {
            const int dyn = b->max_smem - (int)sizeof(RunDev<double>) - 64;
            if (cudaFuncSetAttribute(k_batch_stage<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_batch_stage<float, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_batch_stage<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) !=
                    cudaSuccess)
                return bail(berr(S2D_ERR_CUDA, "cudaFuncSetAttribute failed"));
            attr[b->device] = true;
        }
        b->max_smem = b->max_smem - (int)sizeof(RunDev<double>) - 64;
    }
    const size_t rsz = b->prec == S2D_FP64 ? sizeof(RunDev<double>) : sizeof(RunDev<float>);
    if (cudaMalloc(&b->d_runs, rsz * nruns) != cudaSuccess || cudaMalloc(&b->d_ctrl, 64) != cudaSuccess ||
        cudaMalloc(&b->d_done, sizeof(int) * 3 * nruns) != cudaSuccess || cudaMalloc(&b->d_flags, 64) != cudaSuccess)
        return bail(berr(S2D_ERR_NOMEM, "cudaMalloc failed"));
    cudaMemset(b->d_ctrl, 0, 64);
    cudaMemset(b->d_done, 0, sizeof(int) * 3 * nruns);
    cudaMemset(b->d_flags, 0, 64);
    int maxTg = 1;
    for (auto* h : b->runs) maxTg = std::max(maxTg, h->d.Tg);
    const int r = configure_any(b, std::max(256, maxTg), 0);
    if (r != S2D_OK) return bail(r);
    *out = b;
    return S2D_OK;
}

S2D_API void s2d_batch_destroy(s2d_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graph(b);
    for (auto* h : b->runs) s2d_destroy(h);
    void* ptrs[] = {b->d_runs, b->d_tasks, b->d_ctrl, b->d_done, b->d_flags, b->cl_tab};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

S2D_API int s2d_batch_size(const s2d_batch* b) {
    if (!b) return berr(S2D_ERR_INVALID, "null batch");
    return b->n;
}

S2D_API int s2d_batch_run(s2d_batch* b, int32_t i, s2d_handle** h) {
    if (!b || !h || i < 0 || i >= b->n) return berr(S2D_ERR_INVALID, "bad run index");
    *h = b->runs[i];
    return S2D_OK;
}

S2D_API int s2d_batch_set_dt(s2d_batch* b, const double* dt) {
    if (!b || !dt) return berr(S2D_ERR_INVALID, "null argument");
    for (int i = 0; i < b->n; ++i) {
        if (!std::isfinite(dt[i])) return berr(S2D_ERR_INVALID, "dt must be finite");
        b->dt[i] = dt[i];
    }
    B_CUDA(cudaSetDevice(b->device));
    return upload_dt(b);
}

S2D_API int s2d_batch_inject_stall(s2d_batch* b, int32_t run) {
    if (!b || run < -1 || run >= b->n) return berr(S2D_ERR_INVALID, "bad run index");
    B_CUDA(cudaSetDevice(b->device));
    B_CUDA(cudaStreamSynchronize(b->stream));
    b->stall_run = run;
    return configure_any(b, b->threads, b->ctas_per_sm);
}

S2D_API int s2d_batch_set_closure(s2d_batch* b, s2d_cnn* c) {
    if (!b) return berr(S2D_ERR_INVALID, "null batch");
    B_CUDA(cudaSetDevice(b->device));
    B_CUDA(cudaStreamSynchronize(b->stream));
    if (c) {
        if (b->n > cnn_max_batch(c)) return berr(S2D_ERR_INVALID, "more runs than the network's batch capacity");
        for (auto* h : b->runs)
            if (h->d.K != b->runs[0]->d.K || h->d.M != cnn_grid(c))
                return berr(S2D_ERR_INVALID, "closure batches need every run on the network's grid");
        for (auto* h : b->runs) {
            const int r = ensure_closure_buffers(h);
            if (r != S2D_OK) return r;
        }
        if (!b->cl_tab) {
            const int r = closure_table(b->runs.data(), b->n, &b->cl_tab);
            if (r != S2D_OK) return r;
        }
    } else if (b->cl_tab) {
        cudaFree(b->cl_tab);
        b->cl_tab = nullptr;
    }
    b->cnn = c;
    return configure_any(b, b->threads, b->ctas_per_sm);
}

S2D_API int s2d_batch_integrate_steps(s2d_batch* b, int32_t n) {
    if (!b || n < 0) return berr(S2D_ERR_INVALID, "bad argument");
    B_CUDA(cudaSetDevice(b->device));
    if (n == 0) return S2D_OK;
    if (!b->gexec) {
        const int r = build_graph(b);
        if (r != S2D_OK) return r;
    }
    for (int i = 0; i < n; ++i) B_CUDA(cudaGraphLaunch(b->gexec, b->stream));
    return S2D_OK;
}

S2D_API int s2d_batch_time_steps(s2d_batch* b, int32_t n, double* ms) {
    if (!b || !ms || n <= 0) return berr(S2D_ERR_INVALID, "bad argument");
    B_CUDA(cudaSetDevice(b->device));
    if (!b->gexec) {
        const int r = build_graph(b);
        if (r != S2D_OK) return r;
    }
    cudaEvent_t e0, e1;
    B_CUDA(cudaEventCreate(&e0));
    B_CUDA(cudaEventCreate(&e1));
    B_CUDA(cudaStreamSynchronize(b->stream));
    B_CUDA(cudaEventRecord(e0, b->stream));
    for (int i = 0; i < n; ++i) B_CUDA(cudaGraphLaunch(b->gexec, b->stream));
    B_CUDA(cudaEventRecord(e1, b->stream));
    B_CUDA(cudaEventSynchronize(e1));
    float t = 0.f;
    B_CUDA(cudaEventElapsedTime(&t, e0, e1));
    *ms = t;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return S2D_OK;
}

S2D_API int s2d_batch_status(s2d_batch* b) {
    if (!b) return berr(S2D_ERR_INVALID, "null batch");
    B_CUDA(cudaSetDevice(b->device));
    unsigned int f = 0;
    B_CUDA(cudaMemcpyAsync(&f, b->d_flags, sizeof(f), cudaMemcpyDeviceToHost, b->stream));
    B_CUDA(cudaMemsetAsync(b->d_flags, 0, sizeof(f), b->stream));
    B_CUDA(cudaStreamSynchronize(b->stream));
    if (f & 2u) return berr(S2D_ERR_TIMEOUT, "a persistent-kernel dependency wait gave up");
    if (f & 1u) return berr(S2D_ERR_NONFINITE, "non-finite vorticity in a batch run");
    return S2D_OK;
}

S2D_API int s2d_batch_synchronize(s2d_batch* b) {
    if (!b) return berr(S2D_ERR_INVALID, "null batch");
    B_CUDA(cudaSetDevice(b->device));
    B_CUDA(cudaStreamSynchronize(b->stream));
    return S2D_OK;
}

S2D_API int s2d_batch_tune(s2d_batch* b, int32_t* threads_out, int32_t* ctas_per_sm_out, double* ms_out) {
    if (!b) return berr(S2D_ERR_INVALID, "null batch");
    B_CUDA(cudaSetDevice(b->device));
    // save every run's state (tuning advances it)
    std::vector<void*> save(b->n, nullptr);
    for (int i = 0; i < b->n; ++i) {
        s2d_handle* h = b->runs[i];
        const size_t bytes = (size_t)h->d.KX * h->d.ldS * h->vsz;
        B_CUDA(cudaMalloc(&save[i], bytes));
        B_CUDA(cudaMemcpyAsync(save[i], h->S0, bytes, cudaMemcpyDeviceToDevice, b->stream));
    }
    int maxTg = 1;
    for (auto* h : b->runs) maxTg = std::max(maxTg, h->d.Tg);
    // radix plan of each run size (not with a closure attached: its tables
    // hold the runs' plans): every plan of one size at a time, the others
    // fixed, on the current tile schedule
    if (!b->cnn) {
        std::vector<int> sizes;
        for (auto* h : b->runs)
            if (std::find(sizes.begin(), sizes.end(), h->d.M) == sizes.end()) sizes.push_back(h->d.M);
        for (int M : sizes) {
            double bms = 1e300;
            int bp = -1;
            for (int p = 0; p < S2D_FFT_PLANS; ++p) {
                bool ok = true;
                for (auto* h : b->runs)
                    if (h->d.M == M && s2d_set_fft_plan(h, p) != S2D_OK) ok = false;
                if (!ok || configure_any(b, b->threads, b->ctas_per_sm) != S2D_OK) continue;
                double ms = 0.0;
                if (s2d_batch_integrate_steps(b, 1) != S2D_OK) continue;
                if (s2d_batch_time_steps(b, 2, &ms) != S2D_OK) continue;
                if (ms < bms) {
                    bms = ms;
                    bp = p;
                }
            }
            if (bp < 0) bp = 0;
            for (auto* h : b->runs)
                if (h->d.M == M) s2d_set_fft_plan(h, bp);
        }
    }
    double best = 1e300;
    int bt = 0, bc = 0;
    for (int threads : {128, 256, 512}) {
        if (threads < maxTg) continue;
        for (int cps = 1; cps <= 4; ++cps) {
            if (configure_any(b, threads, cps) != S2D_OK) continue;
            if (b->ctas_per_sm != cps) continue;   // occupancy cap reached
            double ms = 0.0;
            if (s2d_batch_integrate_steps(b, 1) != S2D_OK) continue;   // warm-up
            if (s2d_batch_time_steps(b, 2, &ms) != S2D_OK) continue;
            if (ms < best) {
                best = ms;
                bt = threads;
                bc = cps;
            }
        }
    }
    for (int i = 0; i < b->n; ++i) {
        s2d_handle* h = b->runs[i];
        const size_t bytes = (size_t)h->d.KX * h->d.ldS * h->vsz;
        B_CUDA(cudaMemcpyAsync(h->S0, save[i], bytes, cudaMemcpyDeviceToDevice, b->stream));
    }
    B_CUDA(cudaStreamSynchronize(b->stream));
    for (void* p : save) cudaFree(p);
    if (!bt) return berr(S2D_ERR_UNSUPPORTED, "no tile schedule could be timed");
    const int r = configure_any(b, bt, bc);
    if (r != S2D_OK) return r;
    if (threads_out) *threads_out = bt;
    if (ctas_per_sm_out) *ctas_per_sm_out = bc;
    if (ms_out) *ms_out = best / 2.0;
    return s2d_batch_status(b);
}

}  // extern "C"
