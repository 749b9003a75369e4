// s2d_internal.h -- shared declarations of the Spectral2D GB300 library.
//
// Device data layout (one handle = one simulation, all buffers device-resident):
//
//   compact spectral state  S[kx][jc]   kx in [0,K], jc in [0,2K] with
//                                       ky = jc (jc <= K) or jc - (2K+1);
//                                       column pitch ldS; the retained
//                                       rectangle of the reference's
//                                       (cISize, nyG) array, K = nx/2.
//   half-spectral rows      I[y][kx]    y in [0,M) (physical, after the
//                                       y-transform), kx in [0,K]; row pitch ldI.
//
// M = 3*nx/2 is the padded collocation grid of the 3/2 rule.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "s2d.h"

namespace s2d {

constexpr int kMaxPasses = 16;
constexpr int kElemsPerThread = 12;   // FFT elements held per thread per pass
// the FP32 x-pass with register radix-12/16 passes (s2d_xpass32.cuh): row
// length and its padded shared-memory buffer (elements)
constexpr int kX32M = 3072;
constexpr int kX32Buf = kX32M + kX32M / 16;

// Twiddles of one butterfly of a radix-4 (or radix-2) pass in FMA form:
// w_r = i^q_r * c_r * (1 + i t_r) with |t_r| <= 1, so that x*w_r costs two
// FMAs on (x*i^q_r) and the scale c_r is folded into the butterfly's
// additions (t0 = a + c2*C, E = B + (c3/c1)*D, y = t + c1*E ...).
// q packs q_1 | q_2 << 2 | q_3 << 4.
template <typename T>
struct __align__(16) TwEnt {
    T t1, t2, t3;
    T c1, c2, r31;  // c_1, c_2, c_3 / c_1
    int q;
    int pad;
};

// Geometry and FFT plan shared by every kernel of one handle.
struct Dims {
    int K;      // nx/2: largest retained |kx|, |ky|
    int KX;     // K+1 retained kx columns
    int KY;     // 2K+1 retained ky rows
    int M;      // padded grid points per direction (3/2 rule)
    int ldS;    // compact column pitch (elements)
    int ldI;    // half-spectral row pitch (elements)
    int Tg;     // threads per transform = M / kElemsPerThread
    int npass;  // FFT passes
    int radix[kMaxPasses];
    // per pass: offset (entries) of its TwEnt block, -1 if the pass uses the
    // plain complex table (first pass, or a radix-3 pass after the first)
    int twoff[kMaxPasses];
    long long tab_bytes;  // byte offset of the TwEnt table after the complex table
    // per pass, with Ns the product of the earlier radices: ceil(2^32 / Ns)
    // (0 for Ns = 1), for j mod Ns by a multiply-high, and M / (Ns R)
    unsigned mg[kMaxPasses];
    int tstep[kMaxPasses];
    // slabs of a decomposed run (s2d_slab.cu); a whole run has rows = M and
    // kx0 = 0.  rows: physical rows the x-pass processes.  kx0: true kx of
    // column 0 of the arrays a kernel is handed (a slab's column view: KX
    // columns from kx0 on), used where the wavenumber enters the arithmetic
    // (truncation, 1/k^2, stage factors, forcing)
    int rows;
    int kx0;
    // 1: the FP32 x-pass of M = 3072 runs the generic engine instead of the
    // register radix-12/16 passes (s2d_xpass32.cuh); S2D_XPASS_GENERIC=1
    // (read by s2d_create) sets it, for comparisons
    int xgen;
};

// mg[] and tstep[] of a plan whose M, npass and radix[] are set.
inline void set_pass_constants(Dims* d) {
    int ns = 1;
    for (int p = 0; p < d->npass; ++p) {
        d->mg[p] = ns > 1 ? 0xFFFFFFFFu / (unsigned)ns + 1u : 0u;
        d->tstep[p] = d->M / (ns * d->radix[p]);
        ns *= d->radix[p];
    }
}

// Terms of dW beyond the reference's (drag and a Kolmogorov source).
struct Phys {
    double nu;
    double alpha;     // linear drag coefficient
    int fk;           // forcing wavenumber (0 = none)
    double f_re, f_im;  // coefficient at (kx=0, ky=+fk); conjugate at -fk
    int form;         // S2D_NL_BASDEVANT or S2D_NL_CONSERVATIVE
};

// Spectral operators applied when a column is read for the inverse y-pass.
enum FieldOp : int {
    OP_W = 0,    // omega
    OP_U = 1,    // u = i ky psi
    OP_V = 2,    // v = -i kx psi
    OP_PSI = 3,  // psi = omega / k^2
    OP_WX = 4,   // i kx omega
    OP_WY = 5,   // i ky omega
    OP_UX = 6,   // i kx u
    OP_VY = 7,   // i ky v
    OP_TU = 8,   // u with its factor ky/k^2 (scaled) read from the field's table
    OP_TV = 9,   // v with its factor -kx/k^2 (scaled) read from the field's table
};

// tab[f]: per-mode factor table of field f (compact layout) for OP_TU /
// OP_TV; the other operators read the 1/k^2 table the kernel is given.
struct FieldSet {
    int nf;
    int op[4];
    void* out[4];
    const double* tab[4];
    const float* tabf[4];   // FP32 runs: OP_TU / OP_TV factors already rounded (or null)
};

// Launch shape for one kernel: G groups of Tg threads, dynamic smem bytes.
// pdl: launched as a programmatic dependent of the previous kernel on the
// stream (see pdl_enter / launch_k below).
struct Launch {
    int G;
    int threads;
    size_t smem;
    int blocks;
    bool pdl = false;
};

#ifdef __CUDACC__
// Programmatic dependent launch.  A kernel launched with the programmatic
// stream-serialization attribute may be scheduled while the previous kernel
// on the stream still runs; every such kernel calls pdl_enter() first, in
// every thread: it waits until the previous grid has completed and its
// writes are visible (so the order of the whole chain stays transitive),
// then lets the next grid be scheduled behind this one.  Launched without
// the attribute both instructions return at once.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
#endif

// <<<grid, block, smem, st>>> with the programmatic stream-serialization
// attribute when pdl is set; the kernel must begin with pdl_enter().
template <typename... P, typename... A>
inline cudaError_t launch_k(void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, bool pdl,
                            A&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k, static_cast<A&&>(args)...);
}

// ---- kernel launchers (s2d_kernels.cu); T = float or double -------------
template <typename T>
struct Kern {
    static cudaError_t yinv(const Dims& d, const void* S, const double* rk2, const FieldSet& fs,
                            const void* tw, cudaStream_t st, const Launch& L);
    static cudaError_t xpass_rhs(const Dims& d, void* Iu, void* Iv, const void* Iw, const void* tw,
                                 cudaStream_t st, const Launch& L);
    // prescaled: u and v came from the rk2s table (scaled by sqrt(0.5)/M), so
    // their products carry the 1/(2 M^2) of the forward transform already
    static cudaError_t xpass_bas(const Dims& d, void* Iu, void* Iv, const void* tw, cudaStream_t st,
                                 const Launch& L, bool prescaled = false);
    static cudaError_t yfwd_rk3(const Dims& d, const void* Iu, const void* Iv, void* S0, void* S1,
                                void* Sdw, const void* src, int stage, double dt, const Phys& ph,
                                const void* tw, unsigned int* flags, cudaStream_t st, const Launch& L);
    // K3 in two launches: forward y-FFT of the columns of both products into
    // compact arrays Fu, Fv, then the epilogue (dW, stage update, Truncate)
    static cudaError_t yfwd_col(const Dims& d, const void* Iu, const void* Iv, void* Fu, void* Fv,
                                const void* tw, cudaStream_t st, const Launch& L);
    static cudaError_t stage(const Dims& d, const void* Fu, const void* Fv, void* S0, void* S1, void* Sdw,
                             const void* src, int stage, double dt, const Phys& ph, unsigned int* flags,
                             cudaStream_t st, bool pdl = false, const double* cc = nullptr,
                             const double* vk = nullptr);
    // cc (2 per mode) = (kx^2 - ky^2, kx ky), vk = nu k^2: the Basdevant stage
    // factors as tables (stage() computes them when given none)
    static cudaError_t init_stage_factors(const Dims& d, double nu, double* cc, double* vk, cudaStream_t st);
    static cudaError_t ref_to_compact(const Dims& d, const double* ref, int C, void* S,
                                      cudaStream_t st);
    static cudaError_t compact_to_ref(const Dims& d, const void* S, int C, double* refW,
                                      double* refPsi, cudaStream_t st);
    // the retained rectangle only, by 32 x 32 tiles (ref may be a host array
    // the device reaches directly)
    static cudaError_t rect_to_compact(const Dims& d, const double* ref, int C, void* S, cudaStream_t st);
    static cudaError_t compact_to_rect(const Dims& d, const void* S, int C, double* refW, double* refPsi,
                                       cudaStream_t st);
    static cudaError_t spectrum(const Dims& d, const void* S, double* Ek, cudaStream_t st);
    static cudaError_t enstrophy_partial(const Dims& d, const void* S, double* part, int nblocks,
                                         cudaStream_t st);
    static cudaError_t minmax(const Dims& d, const void* S, unsigned long long* out4,
                              cudaStream_t st);
    static cudaError_t xinv_cfl(const Dims& d, const void* Iu, const void* Iv, const void* tw,
                                unsigned long long* maxbits, cudaStream_t st, const Launch& L);
    static cudaError_t xinv_moments(const Dims& d, const void* Ia, const void* Ib, const void* tw,
                                    double* out, cudaStream_t st, const Launch& L);
    static cudaError_t fill_tg(const Dims& d, const double* sx, const double* sy, void* phys,
                               cudaStream_t st);
    static cudaError_t xfwd_phys(const Dims& d, const void* phys, void* Iout, const void* tw,
                                 cudaStream_t st, const Launch& L);
    static cudaError_t yfwd_store(const Dims& d, const void* I, void* S, const void* tw,
                                  cudaStream_t st, const Launch& L);
    // rk2[kx][jc] = factor / k^2 (0 at k = 0)
    static cudaError_t init_rk2(const Dims& d, double* rk2, cudaStream_t st, double factor = 1.0);
    // fu = ky * rk2, fv = -kx * rk2 per mode: the factors OP_U / OP_V form
    // in the kernel, as tables (the same products, so the same bits)
    static cudaError_t init_uv_factors(const Dims& d, const double* rk2, double* fu, double* fv, cudaStream_t st);
    static size_t smem_limit_yinv();
};

}  // namespace s2d

struct s2d_cnn;

// One simulation: configuration, plan, launch shapes and device buffers.
struct s2d_handle {
    s2d_config cfg;
    s2d_grid grid;
    s2d::Dims d;
    s2d::Phys ph;
    int prec;            // S2D_FP64 / S2D_FP32
    size_t vsz;          // bytes of one complex element of the state
    int device;
    cudaStream_t stream = nullptr;
    bool own_stream = true;
    void* S0 = nullptr;  // w^n
    void* S1 = nullptr;  // stage vorticity
    void* Sdw = nullptr; // dW for compute_rhs (lazily allocated)
    void* src = nullptr; // optional additive source of dW (compact layout), e.g. a closure term
    void* pi = nullptr;  // subgrid flux of the filtered DNS (compact layout, LES handles)
    void* phys = nullptr;          // 3 physical fields on the collocation grid (closure), 8 B/element
    struct s2d_cnn* cnn = nullptr; // closure network used by s2d_les_integrate_steps
    void* les_tab = nullptr;       // device table of closure_terms for this handle alone
    // s2d_les_integrate_steps: the closure term runs on clstream (forked at
    // ev_fork, joined at ev_join) with its own transform buffers cl_I (three
    // arrays of Ibytes), concurrently with the first stage's transforms
    void* cl_I = nullptr;
    cudaStream_t clstream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    void* Ibase = nullptr;
    void* I[3] = {nullptr, nullptr, nullptr};
    size_t Ibytes = 0;
    double* rk2 = nullptr;
    // Basdevant form: rk2 times sqrt(0.5)/M.  The step's inverse y-pass takes
    // u = i ky psi and v = -i kx psi through it, so that the products u v and
    // v^2 - u^2 carry the normalisation 1/(2 M^2) of the forward transform and
    // the x-pass does not multiply its 2 (K+1) outputs per row by it
    double* rk2s = nullptr;
    // ky * rk2s and -kx * rk2s per mode: the step's inverse y-pass reads the
    // factor of u and of v instead of forming it (a conversion and a multiply
    // on the FP64 pipe per mode saved)
    double* fu = nullptr;
    double* fv = nullptr;
    // FP32 handles: the same factors rounded to FP32 once (the rounding the
    // FP32 inverse y-pass applies per mode), read in half the bytes and with
    // no FP64 conversion
    float* fu32 = nullptr;
    float* fv32 = nullptr;
    void* tw = nullptr;
    double* ref_stage = nullptr;   // reference-layout staging (2 arrays)
    size_t ref_bytes = 0;          // bytes of one reference-layout array
    unsigned int* flags = nullptr;
    unsigned long long* red64 = nullptr;  // 8 reduction words
    double* dscratch = nullptr;           // spectrum / partial sums
    size_t dscratch_n = 0;
    void* Fv = nullptr;   // FP64 Basdevant: second compact array of the split K3 (the first is I[2])
    double* cc = nullptr;  // ... and its stage kernel's factors (kx^2 - ky^2, kx ky) per mode
    double* vk = nullptr;  // ... and nu k^2 per mode
    // host-array calls: the truncated part of an output array (outside the
    // retained rectangle) is copied from this buffer of zeros on xstream,
    // concurrently with the step on stream
    void* zeros = nullptr;
    size_t zeros_bytes = 0;
    cudaStream_t xstream = nullptr;
    // kernels may read and write pageable host arrays in place (the device
    // reads the host page tables); false also when S2D_HOST_IO=copy
    bool pageable_direct = false;
    bool io_copy_only = false;   // S2D_HOST_IO=copy: every host array through copies
    s2d::Launch L_yinv, L_xpass, L_yfwd, L_xrow, L_ystore, L_ycol;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    double graph_dt = 0.0;
    int plan = 0;          // radix order of the FFTs (s2d_plan.h, s2d_set_fft_plan)
    size_t tab_cap = 0;    // bytes reserved for the FMA-form twiddle blocks (the largest plan's)
    int max_smem = 0;
    int sms = 152;
};

namespace s2d {

// s2d_create with an optional external stream (not owned by the handle).
int create_handle(const s2d_config* cfg, cudaStream_t ext_stream, s2d_handle** out);

// Shared-memory attribute setup (called once per process and device).
cudaError_t configure_kernels(int max_smem_optin);

// Physical fields (operators opA, opB of the spectral field S, see FieldOp)
// on the M x M collocation grid, row-major, in the handle's precision; outB
// may be null.  Asynchronous on the handle's stream.
int physical_pair(s2d_handle* h, const void* S, int opA, int opB, void* outA, void* outB);

// Closure terms of n LES runs of one grid and precision (the network's grid):
// physical (w, psi) of every run, its rms vorticity, one network forward over
// all n runs, rescale, forward transform with truncation into each run's src.
// closure_table allocates the device table the kernels read (per-run
// pointers and partial sums; free with cudaFree); closure_terms enqueues the
// work on st.  Every run needs src and phys buffers (ensure_closure_buffers).
int ensure_closure_buffers(s2d_handle* h);
int closure_table(s2d_handle* const* runs, int n, void** tab);
int closure_terms(struct s2d_cnn* c, s2d_handle* const* runs, int n, const void* tab, cudaStream_t st);
// One RK3 step of h whose source h->src is written on another stream: the
// first stage's epilogue waits for src_ready (s2d_capi.cu).
int launch_step_sourced(s2d_handle* h, double dt, cudaEvent_t src_ready);
// the network's grid and batch capacity
int cnn_grid(const struct s2d_cnn* c);
int cnn_max_batch(const struct s2d_cnn* c);

// The turbulent initial condition (s2d_set_turbulent) computed on the
// device into h->S0; synchronises the handle's stream (s2d_ic_dev.cu).
int set_turbulent_device(s2d_handle* h, uint64_t seed, int spectrum, double k0, double urms, double tke);

// Record msg as this thread's last error (s2d_last_error) and return code.
int set_error(int code, const char* msg);

// nx of a handle (the IC generator works on host arrays of that grid).
int handle_nx(const s2d_handle* h);

cudaError_t launch_fp64_probe(double* sink, int blocks, int threads, int iters, cudaStream_t st);

// Zeros of the truncated part (outside the retained rectangle) of one or two
// reference-layout arrays a, b (either may be null), blocks x 2 CTAs.
cudaError_t launch_zero_truncated(const Dims& d, int C, double* a, double* b, int blocks, cudaStream_t st);

}  // namespace s2d
