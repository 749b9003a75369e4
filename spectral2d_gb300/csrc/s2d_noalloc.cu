// s2d_noalloc.cu -- ComputeRHS for callers that cannot allocate device memory.
//
// Some callers may not call cudaMalloc: a host code whose device memory is
// owned by another runtime or a fixed pool, code running where allocation is
// forbidden (an allocation would synchronise the device or is disallowed by
// the caller's memory policy), or a plug-in that may only work inside the
// buffers it is handed.  For them s2d_compute_rhs_noalloc evaluates the
// right-hand side of src/Spectral.F90:396-482 on caller-provided device arrays
// and keeps all of its own scratch (compact state, 1/k^2 table, twiddle
// tables, the two half-spectral intermediates and dW) in one file-scope
// __device__ array of S2D_NOALLOC_SCRATCH_BYTES.  Every GPU that loads the
// library holds that array until the process exits.
//
// Nothing here calls cudaMalloc, cudaFree, malloc/new or any allocating
// library routine: the plan and twiddle tables are built by the handle
// path's own builders (s2d_plan.h) into static host buffers and copied into
// the scratch array when nx changes on a device; calls with the nx whose
// tables are resident reuse the cached plan and upload nothing.
#include "s2d.h"
#include "s2d_internal.h"
#include "s2d_plan.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

using namespace s2d;

static __device__ __align__(256) unsigned char g_s2d_noalloc_scratch[S2D_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
constexpr int kMaxM = 3 * S2D_NOALLOC_MAX_NX / 2;

struct DevState {
    bool ready;              // symbol address resolved for this device
    unsigned char* base;     // device address of g_s2d_noalloc_scratch
    int tables_nx;           // nx whose twiddle and 1/k^2 tables are resident (0: none)
    int ntab;                // FMA-form twiddle entries of that plan
    Dims plan;               // that plan (radices, pass constants, table offsets)
    int max_smem;
};
DevState g_dev[kMaxDevices];

// static host staging for the twiddle tables (no heap)
double g_host_tw[2 * kMaxM];
TwEnt<double> g_host_tab[kMaxM];

// The status code is the only error report: writing a message would need
// the library's message buffer, whose update may allocate.
int err(int code, const char*) { return code; }

size_t up256(size_t x) { return (x + 255) / 256 * 256; }

// Geometry and radix plan of the handle path (s2d_plan.h), FP64.
bool plan_noalloc(int nx, Dims* d) {
    std::memset(d, 0, sizeof(*d));
    d->K = nx / 2;
    d->KX = d->K + 1;
    d->KY = 2 * d->K + 1;
    d->M = 3 * nx / 2;
    d->ldS = d->KY + 1;
    d->ldI = (d->KX + 3) / 4 * 4;
    if (!factor_plan(d->M, d)) return false;
    d->Tg = d->M / kElemsPerThread;
    d->rows = d->M;
    d->tab_bytes = (long long)up256((size_t)d->M * sizeof(double2));
    return true;
}

// Carve the scratch array: twiddles (+ FMA blocks) | rk2 | S | Sdw | I0 | I1.
struct Carve {
    size_t tw, rk2, S, Sdw, I0, I1, end;
};

Carve carve(const Dims& d, int ntab) {
    Carve c{};
    const size_t state = (size_t)d.KX * d.ldS * sizeof(double2);
    const size_t inter = (size_t)d.M * d.ldI * sizeof(double2);
    const size_t twb = up256((size_t)d.M * sizeof(double2)) + (size_t)ntab * sizeof(TwEnt<double>);
    c.tw = 0;
    c.rk2 = c.tw + up256(twb);
    c.S = c.rk2 + up256((size_t)d.KX * d.ldS * sizeof(double));
    c.Sdw = c.S + up256(state);
    c.I0 = c.Sdw + up256(state);
    c.I1 = c.I0 + up256(inter);
    c.end = c.I1 + up256(inter);
    return c;
}

Launch shape(int Tg, size_t bytes_per_group, int max_smem) {
    Launch L{};
    int G = (256 / Tg) > 1 ? 256 / Tg : 1;
    while (G > 1 && (G * Tg > 512 || G * bytes_per_group > (size_t)max_smem / 2)) --G;
    L.G = G;
    L.threads = G * Tg;
    L.smem = G * bytes_per_group;
    return L;
}

}  // namespace

extern "C" {

S2D_API int s2d_compute_rhs_noalloc(int32_t nx, double nu, const double* wC_dev, double* dW_dev, void* stream) {
    if (!wC_dev || !dW_dev) return err(S2D_ERR_INVALID, "null device array");
    if (nx < 8 || nx % 8 != 0)
        return err(S2D_ERR_INVALID, "nx must be a positive multiple of 8");
    if (nx > S2D_NOALLOC_MAX_NX)
        return err(S2D_ERR_INVALID, "nx exceeds S2D_NOALLOC_MAX_NX, the size the static scratch holds");
    if (!(nu >= 0.0) || !std::isfinite(nu)) return err(S2D_ERR_INVALID, "nu must be finite, >= 0");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return err(S2D_ERR_CUDA, "no current CUDA device");
    cudaStream_t st = (cudaStream_t)stream;
    DevState& ds = g_dev[dev];
    if (!ds.ready) {
        // once per device, with that device current: the host-side name of
        // the array is not a device address, so resolve it here
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_s2d_noalloc_scratch) != cudaSuccess || !p)
            return err(S2D_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed");
        int optin = 0;
        if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
            return err(S2D_ERR_CUDA, "cudaDeviceGetAttribute failed");
        ds.max_smem = optin - 1024;
        if (configure_kernels(ds.max_smem) != cudaSuccess) return err(S2D_ERR_CUDA, "cudaFuncSetAttribute failed");
        ds.base = (unsigned char*)p;
        ds.tables_nx = 0;
        ds.ready = true;
    }
    unsigned char* B = ds.base;
    Dims d;
    int ntab;
    if (ds.tables_nx == nx) {   // tables of this nx resident: the cached plan, no upload
        d = ds.plan;
        ntab = ds.ntab;
    } else {
        if (!plan_noalloc(nx, &d)) return err(S2D_ERR_UNSUPPORTED, "padded grid is not 2^a 3^b");
        ntab = fill_fma_tables<double>(&d, g_host_tab, kMaxM);
        if (ntab < 0) return err(S2D_ERR_INVALID, "twiddle table exceeds its static buffer");
        if (carve(d, ntab).end > S2D_NOALLOC_SCRATCH_BYTES)
            return err(S2D_ERR_INVALID, "grid does not fit the static scratch");
        fill_twiddles(d.M, g_host_tw);
        const Carve c0 = carve(d, ntab);
        ds.tables_nx = 0;   // until the new tables are queued
        // the copies are queued on st before any kernel of this call that reads them
        if (cudaMemcpyAsync(B + c0.tw, g_host_tw, (size_t)d.M * sizeof(double2), cudaMemcpyHostToDevice, st) !=
                cudaSuccess ||
            (ntab > 0 && cudaMemcpyAsync(B + c0.tw + d.tab_bytes, g_host_tab, (size_t)ntab * sizeof(TwEnt<double>),
                                         cudaMemcpyHostToDevice, st) != cudaSuccess))
            return err(S2D_ERR_CUDA, "twiddle upload failed");
        // pageable source buffers: the copies have read them when cudaMemcpyAsync returns
        if (Kern<double>::init_rk2(d, (double*)(B + c0.rk2), st) != cudaSuccess)
            return err(S2D_ERR_CUDA, "1/k^2 table kernel failed");
        ds.plan = d;
        ds.ntab = ntab;
        ds.tables_nx = nx;
    }
    const Carve c = carve(d, ntab);
    Phys ph{};
    ph.nu = nu;
    ph.form = S2D_NL_BASDEVANT;
    const size_t tb = (size_t)d.M * sizeof(double2);
    const Launch Ly = shape(d.Tg, tb, ds.max_smem);
    const Launch Lx = Ly;
    Launch Lf = shape(d.Tg, 2 * tb, ds.max_smem);
    {
        int cc = (256 / d.Tg) > 1 ? 256 / d.Tg : 1;
        if (cc > 2 * Lf.G) cc = 2 * Lf.G;
        while ((2 * Lf.G) % cc) --cc;
        Lf.threads = cc * d.Tg;
    }
    FieldSet fs{};
    fs.nf = 2;
    fs.op[0] = OP_U;
    fs.op[1] = OP_V;
    fs.out[0] = B + c.I0;
    fs.out[1] = B + c.I1;
    const int C = d.M / 2 + 1;
    // every region of the scratch is fully written before it is read; the
    // stage kernel gets no status word (a NaN/Inf in dW is not reported)
    if (Kern<double>::ref_to_compact(d, wC_dev, C, B + c.S, st) != cudaSuccess ||
        Kern<double>::yinv(d, B + c.S, (const double*)(B + c.rk2), fs, B + c.tw, st, Ly) != cudaSuccess ||
        Kern<double>::xpass_bas(d, B + c.I0, B + c.I1, B + c.tw, st, Lx) != cudaSuccess ||
        Kern<double>::yfwd_rk3(d, B + c.I0, B + c.I1, B + c.S, B + c.S, B + c.Sdw, nullptr, 0, 0.0, ph, B + c.tw,
                               nullptr, st, Lf) != cudaSuccess ||
        Kern<double>::compact_to_ref(d, B + c.Sdw, C, dW_dev, nullptr, st) != cudaSuccess)
        return err(S2D_ERR_CUDA, "kernel launch failed");
    return S2D_OK;
}

}  // extern "C"
