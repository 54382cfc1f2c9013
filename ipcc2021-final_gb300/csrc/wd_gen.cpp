// wd_gen.cpp -- seeded synthetic gauge and source fields (host side).
//
// Every random number is a pure function of (seed, counter): a splitmix64
// hash feeds Box-Muller, so the fields do not depend on thread count or
// generation order.  The counter of a link is (mu, eo site); of a source
// entry its reference-layout index.  The reference itself ships no random
// gauge ("RANDOM" is an empty branch in src/load_gauge.cpp:53-57), so this
// generator defines the synthetic workloads:
//   U_mu(x) = exp(i eps H), H = traceless hermitian with N(0,1) diagonal and
//   N(0,1/2) real and imaginary off-diagonal parts, exponentiated by
//   scaling-and-squaring Taylor series, then re-unitarised (Gram-Schmidt of
//   rows 0 and 1, row 2 = conj(row0 x row1)) into SU(3).
//
// The CPU oracle compiles this same file, with the same flags, into its own
// host-only library under the names wo_gen_gauge / wo_gen_source
// (WD_GEN_ORACLE_NAMES), so that a CPU-only run of the reference's algorithm
// draws bit-identical inputs without loading the CUDA library.
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include "../../include/wilson_gb300.h"

namespace {

typedef std::complex<double> cd;

inline uint64_t splitmix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// uniform in (0, 1)
inline double uniform(uint64_t seed, uint64_t ctr)
{
    const uint64_t h = splitmix64(splitmix64(seed ^ 0x5DEECE66Dull) ^ ctr);
    return ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

inline void gauss2(uint64_t seed, uint64_t ctr, double *g0, double *g1)
{
    const double u1 = uniform(seed, 2 * ctr), u2 = uniform(seed, 2 * ctr + 1);
    const double r = std::sqrt(-2.0 * std::log(u1));
    const double th = 6.283185307179586476925286766559 * u2;
    *g0 = r * std::cos(th);
    *g1 = r * std::sin(th);
}

void matmul3(const cd *a, const cd *b, cd *c)
{
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            cd s = 0;
            for (int k = 0; k < 3; ++k) s += a[i * 3 + k] * b[k * 3 + j];
            c[i * 3 + j] = s;
        }
}

void make_link(uint64_t seed, uint64_t ctr, double eps, cd *U)
{
    double g[10];
    for (int k = 0; k < 5; ++k) gauss2(seed, ctr * 5 + k, &g[2 * k], &g[2 * k + 1]);
    cd H[9];
    const double tr = (g[0] + g[1] + g[2]) / 3.0;
    for (int i = 0; i < 3; ++i) H[i * 4] = g[i] - tr;
    const double s = std::sqrt(0.5);
    H[1] = cd(g[3], g[4]) * s;
    H[2] = cd(g[5], g[6]) * s;
    H[5] = cd(g[7], g[8]) * s;
    H[3] = std::conj(H[1]);
    H[6] = std::conj(H[2]);
    H[7] = std::conj(H[5]);
    // A = i eps H / 2^3; exp(A) by Taylor series to order 12, then square 3 times
    cd A[9], T[9], E[9], tmp[9];
    for (int k = 0; k < 9; ++k) A[k] = cd(0, eps / 8.0) * H[k];
    for (int k = 0; k < 9; ++k) E[k] = T[k] = (k % 4 == 0) ? 1.0 : 0.0;
    for (int n = 1; n <= 12; ++n) {
        matmul3(T, A, tmp);
        for (int k = 0; k < 9; ++k) {
            T[k] = tmp[k] / (double)n;
            E[k] += T[k];
        }
    }
    for (int sq = 0; sq < 3; ++sq) {
        matmul3(E, E, tmp);
        memcpy(E, tmp, sizeof(tmp));
    }
    // re-unitarise into SU(3)
    cd *r0 = E, *r1 = E + 3, *r2 = E + 6;
    double n0 = std::sqrt(std::norm(r0[0]) + std::norm(r0[1]) + std::norm(r0[2]));
    for (int k = 0; k < 3; ++k) r0[k] /= n0;
    cd d = std::conj(r0[0]) * r1[0] + std::conj(r0[1]) * r1[1] + std::conj(r0[2]) * r1[2];
    for (int k = 0; k < 3; ++k) r1[k] -= d * r0[k];
    double n1 = std::sqrt(std::norm(r1[0]) + std::norm(r1[1]) + std::norm(r1[2]));
    for (int k = 0; k < 3; ++k) r1[k] /= n1;
    r2[0] = std::conj(r0[1] * r1[2] - r0[2] * r1[1]);
    r2[1] = std::conj(r0[2] * r1[0] - r0[0] * r1[2]);
    r2[2] = std::conj(r0[0] * r1[1] - r0[1] * r1[0]);
    for (int k = 0; k < 9; ++k) U[k] = E[k];
}

bool dims_ok(const int *dims, int64_t *V)
{
    if (!dims) return false;
    int64_t v = 1;
    for (int i = 0; i < 4; ++i) {
        if (dims[i] <= 0) return false;
        v *= dims[i];
    }
    if (dims[0] % 2) return false;
    *V = v;
    return true;
}

}  // namespace

#ifdef WD_GEN_ORACLE_NAMES
#define WD_GEN_GAUGE wo_gen_gauge
#define WD_GEN_SOURCE wo_gen_source
#else
#define WD_GEN_GAUGE wd_gen_gauge
#define WD_GEN_SOURCE wd_gen_source
#endif

extern "C" wd_status WD_GEN_GAUGE(const int dims[4], uint64_t seed, double eps, double *const gauge[4])
{
    int64_t V;
    if (!dims_ok(dims, &V)) return WD_ERR_BAD_DIMS;
    if (!gauge) return WD_ERR_BAD_ARG;
    for (int mu = 0; mu < 4; ++mu)
        if (!gauge[mu]) return WD_ERR_BAD_ARG;
    for (int mu = 0; mu < 4; ++mu) {
        cd *out = reinterpret_cast<cd *>(gauge[mu]);
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < V; ++e) make_link(seed, (uint64_t)mu * (uint64_t)V + (uint64_t)e, eps, out + e * 9);
    }
    return WD_OK;
}

extern "C" wd_status WD_GEN_SOURCE(const int dims[4], uint64_t seed, double *src)
{
    int64_t V;
    if (!dims_ok(dims, &V)) return WD_ERR_BAD_DIMS;
    if (!src) return WD_ERR_BAD_ARG;
    const int64_t n = V * 12;
    // fixed chunking keeps the norm (and so every output bit) independent of
    // the number of threads
    const int64_t kChunks = 256;
    const int64_t chunk = (n + kChunks - 1) / kChunks;
    double part[kChunks];
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < kChunks; ++c) {
        double s = 0.0;
        const int64_t end = (c + 1) * chunk < n ? (c + 1) * chunk : n;
        for (int64_t i = c * chunk; i < end; ++i) {
            double g0, g1;
            gauss2(seed ^ 0xA5A5A5A5ull, (uint64_t)i, &g0, &g1);
            src[2 * i] = g0;
            src[2 * i + 1] = g1;
            s += g0 * g0 + g1 * g1;
        }
        part[c] = s;
    }
    double norm = 0.0;
    for (int64_t c = 0; c < kChunks; ++c) norm += part[c];
    const double inv = 1.0 / std::sqrt(norm);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < 2 * n; ++i) src[i] *= inv;
    return WD_OK;
}
