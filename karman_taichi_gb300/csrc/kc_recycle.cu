// Initial guesses for a sequence of pressure-correction systems by Galerkin
// projection onto the previous solutions.
//
// Within a time step the SIMPLE loop (karman_taichi.py:633-659;
// simple.py:270-281) solves one p' system per outer iteration, and the
// corrections keep their shape from one outer iteration to the next while
// their size shrinks.  With Z = [z_1 .. z_m] the last m solutions (newest
// first), the guess
//     x0 = Z y,   (Z^T A Z) y = Z^T b
// is the A-orthogonal projection of the new solution onto span(Z): it
// minimises the error's A-norm over that span (which contains x0 = 0), so it
// never starts the solve further from the solution than zero does.  Measured
// on the 320 x 64 channel's p' sequence (the NumPy restatement, time steps 4-6):
// with m = 4 the relative residual of the guess has median 6.7e-5 and
// geometric mean 1.8e-4, so one FP32 multigrid CG pass to 1e-4 reaches the
// required 1e-8 where two passes were needed from zero.
//
// One call: m SpMVs (A z_i), one pass summing the m (m + 1) / 2 products
// (z_i, A z_j) and the m products (z_i, b) per block, a one-block fixed-order
// fold, the m x m solve on the host (Cholesky; a vector whose pivot falls
// below 1e-12 of the diagonal is dropped together with the older ones), and
// one pass forming x0.  Everything FP64, bitwise reproducible.
#include "kc_common.cuh"
#include <algorithm>
#include <cmath>
#include <cstring>

namespace kc {
namespace {

constexpr int kRcThreads = 256;
constexpr int kRcMaxBlocks = 1024;
constexpr int kRcMaxM = KC_RECYCLE_MAX;
constexpr int kRcSums = kRcMaxM * (kRcMaxM + 1) / 2 + kRcMaxM;

struct RcLayout {
    size_t az, partials, out, total;
};
RcLayout rc_layout(long long n, int m) {
    RcLayout L{};
    size_t o = 0;
    L.az = o;
    o = align256(o + (size_t)m * n * 8);
    L.partials = o;
    o = align256(o + (size_t)kRcSums * kRcMaxBlocks * 8);
    L.out = o;
    o = align256(o + (size_t)kRcSums * 8);
    L.total = o;
    return L;
}

struct RcVecs {
    const double* z[kRcMaxM];
    const double* az[kRcMaxM];
};

template <int M>
__global__ void __launch_bounds__(kRcThreads) k_rc_gram(long long n, RcVecs V, const double* __restrict__ b,
                                                        double* partials) {
    constexpr int NS = M * (M + 1) / 2 + M;
    double v[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) v[s] = 0.0;
    for (long long k = blockIdx.x * (long long)kRcThreads + threadIdx.x; k < n; k += (long long)gridDim.x * kRcThreads) {
        double z[M], az[M];
#pragma unroll
        for (int i = 0; i < M; ++i) {
            z[i] = __ldg(V.z[i] + k);
            az[i] = __ldg(V.az[i] + k);
        }
        const double bk = __ldg(b + k);
        int s = 0;
#pragma unroll
        for (int i = 0; i < M; ++i)
#pragma unroll
            for (int j = i; j < M; ++j) {
                v[s] = fma(z[i], az[j], v[s]);
                ++s;
            }
#pragma unroll
        for (int i = 0; i < M; ++i) {
            v[s] = fma(z[i], bk, v[s]);
            ++s;
        }
    }
    block_sum<NS>(v);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int s = 0; s < NS; ++s) partials[s * kRcMaxBlocks + blockIdx.x] = v[s];
    }
}

template <int NS>
__global__ void __launch_bounds__(kRcThreads) k_rc_fold(const double* __restrict__ partials, int nb,
                                                        double* __restrict__ out) {
    double v[NS];
    reduce_partials<NS>(partials, kRcMaxBlocks, nb, v);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int s = 0; s < NS; ++s) out[s] = v[s];
    }
}

struct RcCoef {
    double y[kRcMaxM];
};

__global__ void __launch_bounds__(kRcThreads) k_rc_combine(long long n, RcVecs V, int m, RcCoef c,
                                                           double* __restrict__ x0) {
    for (long long k = blockIdx.x * (long long)kRcThreads + threadIdx.x; k < n; k += (long long)gridDim.x * kRcThreads) {
        double x = 0.0;
        for (int i = 0; i < m; ++i) x = fma(c.y[i], __ldg(V.z[i] + k), x);
        x0[k] = x;
    }
}

int rc_blocks(long long n) {
    return (int)std::max<long long>(1, std::min<long long>((n + kRcThreads * 4 - 1) / (kRcThreads * 4), kRcMaxBlocks));
}

template <int M>
int rc_gram(long long n, const RcVecs& V, const double* b, double* partials, double* out, int nb, cudaStream_t s) {
    constexpr int NS = M * (M + 1) / 2 + M;
    k_rc_gram<M><<<nb, kRcThreads, 0, s>>>(n, V, b, partials);
    KC_LAUNCH_CHECK("k_rc_gram");
    k_rc_fold<NS><<<1, kRcThreads, 0, s>>>(partials, nb, out);
    KC_LAUNCH_CHECK("k_rc_fold");
    return KC_OK;
}

// Cholesky of the leading k x k block of G (row-major m x m, symmetric):
// the largest k whose pivots stay above tol times the diagonal; y solves it.
int rc_solve(const double* G, const double* g, int m, double* y) {
    double Lm[kRcMaxM][kRcMaxM] = {};
    int k = 0;
    for (int i = 0; i < m; ++i) {
        double d = G[i * m + i];
        for (int p = 0; p < i; ++p) d -= Lm[i][p] * Lm[i][p];
        if (!(d > 1e-12 * std::fabs(G[i * m + i])) || !std::isfinite(d)) break;
        Lm[i][i] = std::sqrt(d);
        for (int r = i + 1; r < m; ++r) {
            double e = G[r * m + i];
            for (int p = 0; p < i; ++p) e -= Lm[r][p] * Lm[i][p];
            Lm[r][i] = e / Lm[i][i];
        }
        k = i + 1;
    }
    double w[kRcMaxM];
    for (int i = 0; i < k; ++i) {
        double e = g[i];
        for (int p = 0; p < i; ++p) e -= Lm[i][p] * w[p];
        w[i] = e / Lm[i][i];
    }
    for (int i = k - 1; i >= 0; --i) {
        double e = w[i];
        for (int p = i + 1; p < k; ++p) e -= Lm[p][i] * y[p];
        y[i] = e / Lm[i][i];
    }
    for (int i = k; i < m; ++i) y[i] = 0.0;
    return k;
}

}  // namespace
}  // namespace kc

using namespace kc;

extern "C" {

size_t kc_recycle_ws_bytes(long long n, int m) {
    if (n < 1 || m < 1 || m > KC_RECYCLE_MAX) return 0;
    return rc_layout(n, m).total;
}

int kc_recycle_guess(const kc_system* A64, const double* b, const double* const* Z, int m, double* x0, void* ws,
                     size_t ws_bytes, int* used, void* stream) {
    if (used) *used = 0;
    if (!A64 || !b || !x0 || (m > 0 && !Z)) return set_error("kc_recycle_guess: null argument"), KC_ERR_ARG;
    if (A64->dtype != KC_F64) return set_error("kc_recycle_guess: the system must be FP64"), KC_ERR_ARG;
    if (m < 0 || m > KC_RECYCLE_MAX)
        return set_error("kc_recycle_guess: m = %d outside [0, %d]", m, KC_RECYCLE_MAX), KC_ERR_ARG;
    const long long n = A64->n;
    cudaStream_t s = as_stream(stream);
    if (m == 0) {
        KC_CUDA(cudaMemsetAsync(x0, 0, (size_t)n * sizeof(double), s));
        return KC_OK;
    }
    const RcLayout L = rc_layout(n, m);
    if (!ws || ws_bytes < L.total || ((uintptr_t)ws & 255))
        return set_error("kc_recycle_guess: workspace %zu bytes (256-aligned) < required %zu", ws_bytes, L.total),
               KC_ERR_WORKSPACE;
    char* base = (char*)ws;
    RcVecs V{};
    for (int i = 0; i < m; ++i) {
        if (!Z[i]) return set_error("kc_recycle_guess: null vector %d", i), KC_ERR_ARG;
        V.z[i] = Z[i];
        double* az = (double*)(base + L.az) + (size_t)i * n;
        V.az[i] = az;
        int rc = kc_spmv(A64, Z[i], az, stream);
        if (rc) return rc;
    }
    double* partials = (double*)(base + L.partials);
    double* out = (double*)(base + L.out);
    const int nb = rc_blocks(n);
    int rc = KC_OK;
    switch (m) {
        case 1: rc = rc_gram<1>(n, V, b, partials, out, nb, s); break;
        case 2: rc = rc_gram<2>(n, V, b, partials, out, nb, s); break;
        case 3: rc = rc_gram<3>(n, V, b, partials, out, nb, s); break;
        default: rc = rc_gram<4>(n, V, b, partials, out, nb, s); break;
    }
    if (rc) return rc;
    const int ns = m * (m + 1) / 2 + m;
    double h[kRcSums];
    const void* hp = readback(out, (size_t)ns * sizeof(double), s);
    if (!hp) return KC_ERR_CUDA;
    memcpy(h, hp, (size_t)ns * sizeof(double));
    double G[kRcMaxM * kRcMaxM], g[kRcMaxM], y[kRcMaxM];
    int q = 0;
    for (int i = 0; i < m; ++i)
        for (int j = i; j < m; ++j) G[i * m + j] = G[j * m + i] = h[q++];
    for (int i = 0; i < m; ++i) g[i] = h[q++];
    const int k = rc_solve(G, g, m, y);
    RcCoef c{};
    for (int i = 0; i < m; ++i) c.y[i] = y[i];
    k_rc_combine<<<nb, kRcThreads, 0, s>>>(n, V, k, c, x0);
    KC_LAUNCH_CHECK("k_rc_combine");
    if (used) *used = k;
    return KC_OK;
}

}  // extern "C"
