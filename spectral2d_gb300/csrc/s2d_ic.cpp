// s2d_ic.cpp -- reproducible turbulent initial condition (host code).
//
// Follows SetTurbulentVelocity / FourierVelocity (src/SetIC.F90:125-151,
// :175-364): per stored mode a = sqrt(E(|k|) dk) exp(i theta),
// u = -a ky/|k|, v = a kx/|k| (:252-261), normalised by sqrt of the shell's
// mode count with Hermitian weights 1 (kx = 0 or kxMG) or 2 (:295-354),
// truncated (:357-358), then omega = i kx v - i ky u (src/Spectral.F90:624-647).
// Changes, each stated in the header s2d.h: theta comes from a counter-based
// hash of (seed, kx, ky) instead of the compiler RNG seeded from /dev/urandom
// (src/Random.F90:59-69); the kx = 0 column is made Hermitian; omega is scaled
// so that ComputeSpectrum's TKE equals the requested value.
// s2d_set_turbulent computes the same initial condition on the device
// (s2d_ic_dev.cu); this host generator serves callers without a GPU and
// checks the device one.
#include "s2d.h"
#include "s2d_internal.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ULL;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// phase in [0, 2 pi): top 53 bits of splitmix64(splitmix64(key)),
// key = seed<<42 ^ kx<<21 ^ (ky mod 2^21)
double mode_phase(uint64_t seed, int64_t kx, int64_t ky) {
    const uint64_t key = (seed << 42) ^ ((uint64_t)kx << 21) ^ ((uint64_t)ky & 0x1FFFFFULL);
    const uint64_t h = splitmix64(splitmix64(key));
    const double u = (double)(h >> 11) * (1.0 / 9007199254740992.0);
    return 2.0 * M_PI * u;
}

double shape(int kind, double k, double k0, double urms) {
    if (kind == S2D_SPECTRUM_SCHUMANN) return 1.5 * urms * urms * k / k0 * std::exp(-k / k0);
    return (k * k) * (k * k) * std::exp(-2.0 * ((k / k0) * (k / k0)));
}

// BinarySearch (src/Analysis.F90:475-513), 1-based result.
int binary_search(const std::vector<double>& f, double x) {
    int iL = 0, iU = (int)f.size();
    while (iU - iL > 1) {
        const int iM = (iL + iU) / 2;
        if (x >= f[iM - 1]) iL = iM;
        else iU = iM;
    }
    return iL;
}

}  // namespace

extern "C" {

S2D_API int s2d_turbulent_ic_host(int32_t nx, uint64_t seed, int32_t spectrum, double k0, double urms, double tke,
                                  double* wC) {
    if (!wC || nx < 8 || nx % 2) return S2D_ERR_INVALID;
    if (spectrum != S2D_SPECTRUM_SCHUMANN && spectrum != S2D_SPECTRUM_K4_GAUSS) return S2D_ERR_INVALID;
    if (!(k0 > 0.0)) return S2D_ERR_INVALID;
    s2d_grid g;
    if (s2d_get_grid_size(nx, nx, S2D_DEALIAS_3_2_RULE, &g) != S2D_OK) return S2D_ERR_INVALID;
    const int C = g.cISize, NY = g.nyG;
    const long n = (long)C * NY;
    const int K = nx / 2;
    auto kyof = [&](int j) { return j > NY / 2 ? j - NY : j; };
    auto kept = [&](int kx, int ky) { return (long)kx * kx + (long)ky * ky <= (long)K * K; };

    // bin edges (src/SetIC.F90:269-292)
    const double kMaxG = std::sqrt((double)(g.kxMG * g.kxMG + g.kyMG * g.kyMG));
    const int kIntMax = (int)(kMaxG + 1.0);
    const int numBin = kIntMax + 1;
    std::vector<double> edges(numBin + 1);
    edges[0] = 0.0;
    for (int i = 1; i <= kIntMax; ++i) edges[i] = 0.5 + (double)(i - 1) * 1.0;
    edges[numBin] = (double)kIntMax + 0.1;

    std::vector<long> cnt(numBin + 2, 0);
    std::vector<int> bin(n);
    for (int j = 0; j < NY; ++j) {
        const double ky = (double)kyof(j);
        for (int i = 0; i < C; ++i) {
            const double kx = (double)i;
            const double kmag = std::sqrt(kx * kx + ky * ky);
            const int b = binary_search(edges, kmag);
            bin[(long)j * C + i] = b;
            cnt[b] += (i == 0 || i == g.kxMG) ? 1 : 2;
        }
    }
    // velocity modes, normalised and truncated; omega = i kx v - i ky u
    std::vector<double> w(2 * n, 0.0);
    for (int j = 0; j < NY; ++j) {
        const int kyi = kyof(j);
        const double ky = (double)kyi;
        for (int i = 0; i < C; ++i) {
            const long o = (long)j * C + i;
            if (!kept(i, kyi) || (i == 0 && kyi == 0)) continue;
            const double kx = (double)i;
            const double kmag = std::sqrt(kx * kx + ky * ky);
            const double E = shape(spectrum, kmag, k0, urms);
            const double th = mode_phase(seed, i, kyi);
            const double amp = std::sqrt(E * 1.0);
            const double ar = amp * std::cos(th), ai = amp * std::sin(th);
            const double nrm = std::sqrt((double)cnt[bin[o]]);
            const double ur = ((-1.0 * ar) * ky / kmag) / nrm, ui = ((-1.0 * ai) * ky / kmag) / nrm;
            const double vr = (ar * kx / kmag) / nrm, vi = (ai * kx / kmag) / nrm;
            // i kx v - i ky u
            w[2 * o] = (-kx * vi) - (-ky * ui);
            w[2 * o + 1] = (kx * vr) - (ky * ur);
        }
    }
    // Hermitian kx = 0 column: w(0,-ky) = conj w(0,ky)
    for (int ky = 1; ky <= K; ++ky) {
        const long op = (long)ky * C, on = (long)(NY - ky) * C;
        w[2 * on] = w[2 * op];
        w[2 * on + 1] = -w[2 * op + 1];
    }
    if (tke > 0.0) {
        // ComputeSpectrum TKE with u = i ky psi, v = -i kx psi, psi = w/k^2
        std::vector<double> Ek(numBin + 2, 0.0);
        for (int j = 0; j < NY; ++j) {
            const double ky = (double)kyof(j);
            for (int i = 0; i < C; ++i) {
                const long o = (long)j * C + i;
                const double kx = (double)i;
                const double k2 = kx * kx + ky * ky;
                double pr = 0.0, pi = 0.0;
                if (k2 != 0.0) {
                    pr = w[2 * o] / k2;
                    pi = w[2 * o + 1] / k2;
                }
                const double ux = -ky * pi, uy = ky * pr, vx = kx * pi, vy = -kx * pr;
                const double e = ux * ux + uy * uy + vx * vx + vy * vy;
                Ek[bin[o]] += (i == 0 || i == g.kxMG) ? 0.5 * e : e;
            }
        }
        double t = 0.0;
        for (int b = 1; b <= numBin; ++b) t += Ek[b];
        if (t > 0.0) {
            const double s = std::sqrt(tke / t);
            for (auto& x : w) x *= s;
        }
    }
    std::memcpy(wC, w.data(), sizeof(double) * 2 * n);
    return S2D_OK;
}

}  // extern "C"
