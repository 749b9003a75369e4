// s2d_io.cu -- checkpoints and restart files.
//
// Checkpoint: the handle's spectral state as raw bytes after a header with
// the run's parameters, so that a run resumed from it continues bit for bit.
// The reference writes restarts but has no reader, so it cannot resume
// (src/IO.F90:98-143).
//
// Restart: the physical fields Omega, Psi, u, v on the nxG x nyG collocation
// grid, as the reference's WriteRestart writes them to /FlowData/{Omega,Psi,
// u,v} with header attributes nx, ny, nadv, time, nu (src/IO.F90:306-424),
// here as one little-endian binary file (64-byte header, then the four
// arrays, x fastest) and an XDMF sidecar that points into it (the reference's
// sidecar is src/IO.F90:583-650; HDF5 itself is not available).  Point
// (i, j), 0-based, sits at x = 2 pi (i+1)/nxG, y = 2 pi (j+1)/nyG
// (src/SetIC.F90:91-94).  s2d_read_restart loads Omega back through the
// forward transform.
#include "s2d.h"
#include "s2d_internal.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace s2d;

namespace {

struct CkptHeader {
    char magic[8];          // "S2DCKPT1"
    int32_t nx, ny, precision, form;
    double nu, alpha, forcing_amp;
    int32_t forcing_k, ldS;
    int64_t nadv;
    double time;
    int64_t bytes;
};

struct RestHeader {
    char magic[8];          // "S2DREST1"
    int32_t nx, ny, nxG, nyG;
    int64_t nadv;
    double time, nu;
    char pad[16];
};
static_assert(sizeof(RestHeader) == 64, "restart header is 64 bytes");

int ioerr(int code, const std::string& m) { return set_error(code, m.c_str()); }

#define IO_CUDA(call)                                                                 \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess) return ioerr(S2D_ERR_CUDA, cudaGetErrorString(e_));    \
    } while (0)

// Physical fields (opA, opB) of the state as double arrays of nyG x nxG.
int fields_to_host(s2d_handle* h, int opA, int opB, std::vector<double>& a, std::vector<double>& b) {
    const size_t n = (size_t)h->d.M * h->d.M;
    const size_t es = h->prec == S2D_FP64 ? sizeof(double) : sizeof(float);
    void* dev = nullptr;
    IO_CUDA(cudaMalloc(&dev, 2 * n * es));
    int r = physical_pair(h, h->S0, opA, opB, dev, (char*)dev + n * es);
    std::vector<char> raw(2 * n * es);
    if (r == S2D_OK) {
        cudaError_t e = cudaMemcpyAsync(raw.data(), dev, raw.size(), cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) r = ioerr(S2D_ERR_CUDA, cudaGetErrorString(e));
    }
    cudaFree(dev);
    if (r != S2D_OK) return r;
    a.resize(n);
    b.resize(n);
    for (size_t i = 0; i < n; ++i) {
        if (h->prec == S2D_FP64) {
            a[i] = reinterpret_cast<const double*>(raw.data())[i];
            b[i] = reinterpret_cast<const double*>(raw.data())[n + i];
        } else {
            a[i] = reinterpret_cast<const float*>(raw.data())[i];
            b[i] = reinterpret_cast<const float*>(raw.data())[n + i];
        }
    }
    return S2D_OK;
}

std::string stem_of(const char* root, int num) {
    char buf[32];
    std::snprintf(buf, sizeof(buf), "_%08d", num);
    return std::string(root) + buf;
}

std::string base_name(const std::string& p) {
    const size_t s = p.find_last_of('/');
    return s == std::string::npos ? p : p.substr(s + 1);
}

}  // namespace

extern "C" {

S2D_API int s2d_checkpoint_write(s2d_handle* h, const char* path, int64_t nadv, double time) {
    if (!h || !path) return ioerr(S2D_ERR_INVALID, "null argument");
    IO_CUDA(cudaSetDevice(h->device));
    CkptHeader hd{};
    std::memcpy(hd.magic, "S2DCKPT1", 8);
    hd.nx = h->cfg.nx;
    hd.ny = h->cfg.ny;
    hd.precision = h->prec;
    hd.form = h->ph.form;
    hd.nu = h->cfg.nu;
    hd.alpha = h->cfg.alpha;
    hd.forcing_amp = h->cfg.forcing_amp;
    hd.forcing_k = h->cfg.forcing_k;
    hd.ldS = h->d.ldS;
    hd.nadv = nadv;
    hd.time = time;
    hd.bytes = (int64_t)h->d.KX * h->d.ldS * (int64_t)h->vsz;
    std::vector<char> st((size_t)hd.bytes);
    IO_CUDA(cudaMemcpyAsync(st.data(), h->S0, st.size(), cudaMemcpyDeviceToHost, h->stream));
    IO_CUDA(cudaStreamSynchronize(h->stream));
    FILE* f = std::fopen(path, "wb");
    if (!f) return ioerr(S2D_ERR_INVALID, std::string("cannot open ") + path);
    const bool ok = std::fwrite(&hd, sizeof(hd), 1, f) == 1 && std::fwrite(st.data(), 1, st.size(), f) == st.size();
    std::fclose(f);
    if (!ok) return ioerr(S2D_ERR_INVALID, std::string("write failed: ") + path);
    return S2D_OK;
}

S2D_API int s2d_checkpoint_read(s2d_handle* h, const char* path, int64_t* nadv, double* time) {
    if (!h || !path) return ioerr(S2D_ERR_INVALID, "null argument");
    IO_CUDA(cudaSetDevice(h->device));
    FILE* f = std::fopen(path, "rb");
    if (!f) return ioerr(S2D_ERR_INVALID, std::string("cannot open ") + path);
    CkptHeader hd{};
    bool ok = std::fread(&hd, sizeof(hd), 1, f) == 1;
    if (!ok || std::memcmp(hd.magic, "S2DCKPT1", 8) != 0) {
        std::fclose(f);
        return ioerr(S2D_ERR_INVALID, "not a checkpoint file");
    }
    const int64_t want = (int64_t)h->d.KX * h->d.ldS * (int64_t)h->vsz;
    if (hd.nx != h->cfg.nx || hd.ny != h->cfg.ny || hd.precision != h->prec || hd.ldS != h->d.ldS ||
        hd.bytes != want) {
        std::fclose(f);
        return ioerr(S2D_ERR_INVALID, "checkpoint grid or precision differs from the handle's");
    }
    std::vector<char> st((size_t)hd.bytes);
    ok = std::fread(st.data(), 1, st.size(), f) == st.size();
    std::fclose(f);
    if (!ok) return ioerr(S2D_ERR_INVALID, "truncated checkpoint");
    IO_CUDA(cudaMemcpyAsync(h->S0, st.data(), st.size(), cudaMemcpyHostToDevice, h->stream));
    IO_CUDA(cudaStreamSynchronize(h->stream));
    if (nadv) *nadv = hd.nadv;
    if (time) *time = hd.time;
    return S2D_OK;
}

S2D_API int s2d_write_restart(s2d_handle* h, const char* root, int32_t num, int64_t nadv, double time) {
    if (!h || !root) return ioerr(S2D_ERR_INVALID, "null argument");
    IO_CUDA(cudaSetDevice(h->device));
    std::vector<double> w, p, u, v;
    int r = fields_to_host(h, OP_W, OP_PSI, w, p);
    if (r == S2D_OK) r = fields_to_host(h, OP_U, OP_V, u, v);
    if (r != S2D_OK) return r;
    const int M = h->d.M;
    const std::string stem = stem_of(root, num);
    RestHeader hd{};
    std::memcpy(hd.magic, "S2DREST1", 8);
    hd.nx = h->cfg.nx;
    hd.ny = h->cfg.ny;
    hd.nxG = M;
    hd.nyG = M;
    hd.nadv = nadv;
    hd.time = time;
    hd.nu = h->cfg.nu;
    FILE* f = std::fopen((stem + ".bin").c_str(), "wb");
    if (!f) return ioerr(S2D_ERR_INVALID, "cannot open " + stem + ".bin");
    bool ok = std::fwrite(&hd, sizeof(hd), 1, f) == 1;
    for (const auto* a : {&w, &p, &u, &v}) ok = ok && std::fwrite(a->data(), sizeof(double), a->size(), f) == a->size();
    std::fclose(f);
    if (!ok) return ioerr(S2D_ERR_INVALID, "write failed: " + stem + ".bin");
    // XDMF sidecar: 2-D co-rectilinear mesh with the reference's 1-based origin
    f = std::fopen((stem + ".xmf").c_str(), "w");
    if (!f) return ioerr(S2D_ERR_INVALID, "cannot open " + stem + ".xmf");
    const double dx = 2.0 * M_PI / M;
    const std::string bin = base_name(stem + ".bin");
    std::fprintf(f, "<?xml version=\"1.0\" ?>\n<Xdmf Version=\"2.0\">\n <Domain>\n");
    std::fprintf(f, "  <Grid Name=\"FlowData\" GridType=\"Uniform\">\n   <Time Value=\"%.17g\"/>\n", time);
    std::fprintf(f, "   <Topology TopologyType=\"2DCoRectMesh\" Dimensions=\"%d %d\"/>\n", M, M);
    std::fprintf(f, "   <Geometry GeometryType=\"ORIGIN_DXDY\">\n");
    std::fprintf(f, "    <DataItem Dimensions=\"2\" NumberType=\"Float\" Precision=\"8\" Format=\"XML\">%.17g %.17g</DataItem>\n",
                 dx, dx);
    std::fprintf(f, "    <DataItem Dimensions=\"2\" NumberType=\"Float\" Precision=\"8\" Format=\"XML\">%.17g %.17g</DataItem>\n",
                 dx, dx);
    std::fprintf(f, "   </Geometry>\n");
    const char* names[4] = {"Omega", "Psi", "u", "v"};
    for (int k = 0; k < 4; ++k)
        std::fprintf(f,
                     "   <Attribute Name=\"%s\" AttributeType=\"Scalar\" Center=\"Node\">\n"
                     "    <DataItem Dimensions=\"%d %d\" NumberType=\"Float\" Precision=\"8\" Format=\"Binary\" "
                     "Endian=\"Little\" Seek=\"%lld\">%s</DataItem>\n   </Attribute>\n",
                     names[k], M, M, (long long)(64 + (long long)k * M * M * 8), bin.c_str());
    std::fprintf(f, "  </Grid>\n </Domain>\n</Xdmf>\n");
    std::fclose(f);
    return S2D_OK;
}

S2D_API int s2d_read_restart(s2d_handle* h, const char* path, int64_t* nadv, double* time) {
    if (!h || !path) return ioerr(S2D_ERR_INVALID, "null argument");
    IO_CUDA(cudaSetDevice(h->device));
    FILE* f = std::fopen(path, "rb");
    if (!f) return ioerr(S2D_ERR_INVALID, std::string("cannot open ") + path);
    RestHeader hd{};
    bool ok = std::fread(&hd, sizeof(hd), 1, f) == 1;
    const int M = h->d.M;
    if (!ok || std::memcmp(hd.magic, "S2DREST1", 8) != 0 || hd.nxG != M || hd.nyG != M || hd.nx != h->cfg.nx) {
        std::fclose(f);
        return ioerr(S2D_ERR_INVALID, "not a restart file of this grid");
    }
    std::vector<double> w((size_t)M * M);
    ok = std::fread(w.data(), sizeof(double), w.size(), f) == w.size();
    std::fclose(f);
    if (!ok) return ioerr(S2D_ERR_INVALID, "truncated restart file");
    // Omega -> forward transform (normalised, truncated) -> state
    const size_t es = h->prec == S2D_FP64 ? sizeof(double) : sizeof(float);
    std::vector<char> raw(w.size() * es);
    for (size_t i = 0; i < w.size(); ++i) {
        if (h->prec == S2D_FP64) reinterpret_cast<double*>(raw.data())[i] = w[i];
        else reinterpret_cast<float*>(raw.data())[i] = (float)w[i];
    }
    void* dev = nullptr;
    IO_CUDA(cudaMalloc(&dev, raw.size()));
    cudaError_t e = cudaMemcpyAsync(dev, raw.data(), raw.size(), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) {
        if (h->prec == S2D_FP64) {
            e = Kern<double>::xfwd_phys(h->d, dev, h->I[2], h->tw, h->stream, h->L_xrow);
            if (e == cudaSuccess) e = Kern<double>::yfwd_store(h->d, h->I[2], h->S0, h->tw, h->stream, h->L_ystore);
        } else {
            e = Kern<float>::xfwd_phys(h->d, dev, h->I[2], h->tw, h->stream, h->L_xrow);
            if (e == cudaSuccess) e = Kern<float>::yfwd_store(h->d, h->I[2], h->S0, h->tw, h->stream, h->L_ystore);
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(dev);
    if (e != cudaSuccess) return ioerr(S2D_ERR_CUDA, cudaGetErrorString(e));
    if (nadv) *nadv = hd.nadv;
    if (time) *time = hd.time;
    return S2D_OK;
}

}  // extern "C"
