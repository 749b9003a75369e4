// s2d_plan.h -- host-side FFT plan and twiddle-table builders, shared by the
// handle path (s2d_capi.cu) and the allocation-free entry point
// (s2d_noalloc.cu), so that both hand the FFT kernels the same tables in the
// same packed layout.  The builders write into caller-supplied buffers and
// allocate nothing.
#pragma once

#include <cmath>

#include "s2d_internal.h"

namespace s2d {

// exp(-2 pi i r / M) correctly rounded in practice: octant reduction with
// exact integer arithmetic, residual angle in [0, pi/4] in long double.
inline void twiddle(long long r, long long M, double* c, double* s) {
    const long double PI_4 = 0.785398163397448309615660845819875721L;
    r %= M;
    const long long n8 = 8 * r;
    const int oct = (int)(n8 / M);
    const long long rem = n8 - (long long)oct * M;
    const long double x = ((oct & 1) ? (long double)(M - rem) : (long double)rem) / (long double)M * PI_4;
    const long double cx = cosl(x), sx = sinl(x);
    long double C = 0, S = 0;
    switch (oct) {
        case 0: C = cx; S = sx; break;
        case 1: C = sx; S = cx; break;
        case 2: C = -sx; S = cx; break;
        case 3: C = -cx; S = sx; break;
        case 4: C = -cx; S = -sx; break;
        case 5: C = -sx; S = -cx; break;
        case 6: C = sx; S = -cx; break;
        default: C = cx; S = -sx; break;
    }
    *c = (double)C;
    *s = -(double)S;  // forward sign
}

// exp(-2 pi i m / M) = i^q * c * (1 + i t) with |t| <= 1 (needs 4 | M):
// q0 = nearest quarter turn of m, residual angle th in [-pi/4, pi/4].
inline void twiddle_fma(long long m, long long M, int* q, long double* c, long double* t) {
    const long double PI = 3.141592653589793238462643383279502884L;
    m %= M;
    if (m < 0) m += M;
    const long long q0 = (4 * m + M / 2) / M;
    const long long mr = m - q0 * (M / 4);
    const long double th = 2.0L * PI * (long double)mr / (long double)M;
    *q = (int)((4 - (q0 % 4)) % 4);   // (-i)^q0 = i^-q0
    *c = cosl(th);
    *t = -sinl(th) / cosl(th);
}

// Radix sequences of a length-M transform (M = 2^a 3^b, 12 | M):
//   plan 0: the radix-3 passes first (the first one is the pruned pass of
//           the inverse transforms), one radix-2 pass when a is odd, then
//           radix-4 passes;
//   plan 1: radix-3 passes first, radix-4 passes, the radix-2 pass last;
//   plan 2: the radix-2 pass first, radix-4 passes, radix-3 passes last
//           (no pruned first pass).
// Sets npass, radix[] and the per-pass constants.  False if M has another
// factor, the plan is unknown or needs more than kMaxPasses passes.
constexpr int kNumPlans = 3;
inline bool factor_plan(int M, Dims* d, int plan = 0) {
    int m = M, a = 0, b = 0;
    while (m % 2 == 0) { m /= 2; ++a; }
    while (m % 3 == 0) { m /= 3; ++b; }
    if (m != 1 || M % kElemsPerThread != 0 || plan < 0 || plan >= kNumPlans) return false;
    const int np = b + (a % 2) + a / 2;
    if (np > kMaxPasses) return false;
    int p = 0;
    auto put = [&](int r, int n) {
        for (int i = 0; i < n; ++i) d->radix[p++] = r;
    };
    if (plan == 0) {
        put(3, b);
        put(2, a % 2);
        put(4, a / 2);
    } else if (plan == 1) {
        put(3, b);
        put(4, a / 2);
        put(2, a % 2);
    } else {
        put(2, a % 2);
        put(4, a / 2);
        put(3, b);
    }
    d->npass = np;
    set_pass_constants(d);
    return true;
}

// Entries of the FMA-form twiddle blocks of a plan: one per butterfly
// position k < Ns of every radix-4 or radix-2 pass after the first.
inline int fma_table_entries(const Dims& d) {
    int n = 0, Ns = 1;
    for (int p = 0; p < d.npass; ++p) {
        if (p > 0 && (d.radix[p] == 4 || d.radix[p] == 2)) n += Ns;
        Ns *= d.radix[p];
    }
    return n;
}

// The FMA-form twiddle blocks (TwEnt) of every radix-4/2 pass after the
// first, written to out[0 .. fma_table_entries(*d)), and each pass's offset
// into them in d->twoff (-1 for passes that use the plain complex table).
// Returns the entry count, or -1 if it exceeds cap (nothing is written then).
template <typename T>
inline int fill_fma_tables(Dims* d, TwEnt<T>* out, int cap) {
    if (fma_table_entries(*d) > cap) return -1;
    int n = 0, Ns = 1;
    for (int p = 0; p < d->npass; ++p) {
        const int R = d->radix[p];
        d->twoff[p] = -1;
        if (p > 0 && (R == 4 || R == 2)) {
            d->twoff[p] = n;
            const long long step = d->M / (Ns * R);
            for (int k = 0; k < Ns; ++k) {
                TwEnt<T> e{};
                int qs[4] = {0, 0, 0, 0};
                long double cs[4] = {1, 1, 1, 1}, ts[4] = {0, 0, 0, 0};
                for (int r = 1; r < R; ++r) twiddle_fma((long long)r * k * step, d->M, &qs[r], &cs[r], &ts[r]);
                e.t1 = (T)ts[1];
                e.t2 = (T)ts[2];
                e.t3 = (T)ts[3];
                e.c1 = (T)cs[1];
                e.c2 = (T)cs[2];
                e.r31 = (T)(cs[3] / cs[1]);
                e.q = qs[1] | (qs[2] << 2) | (qs[3] << 4);
                out[n++] = e;
            }
        }
        Ns *= R;
    }
    return n;
}

// The plain complex twiddles exp(-2 pi i t / M), t < M, as (re, im) pairs.
inline void fill_twiddles(int M, double* out2M) {
    for (int t = 0; t < M; ++t) twiddle(t, M, &out2M[2 * t], &out2M[2 * t + 1]);
}

}  // namespace s2d
