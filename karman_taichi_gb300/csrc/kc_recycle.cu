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
// One call, three launches and no host round trip: one pass that forms A z_i
// on the fly (the FP64 stencil in kc_spmv's operation order, so the sums are
// those of separate SpMVs) and sums, per block, the m (m + 1) / 2 products
// (z_i, A z_j) and the m products (z_i, b); one block that folds the block
// sums in a fixed order and solves the m x m system (Cholesky; a vector whose
// pivot falls below 1e-12 of the diagonal is dropped together with the older
// ones); one pass forming x0 from the coefficients it left in device memory.
// On GB300 the pass is bound by the FP64 pipe (34 FMAs per cell at m = 4),
// not by its 80 bytes per cell.  Everything FP64, bitwise reproducible.
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
    size_t partials, out, coef, total;
};
RcLayout rc_layout() {
    RcLayout L{};
    size_t o = 0;
    L.partials = o;
    o = align256(o + (size_t)kRcSums * kRcMaxBlocks * 8);
    L.out = o;
    o = align256(o + (size_t)kRcSums * 8);
    L.coef = o;   // y[0 .. kRcMaxM), then the count kept (as a double)
    o = align256(o + (size_t)(kRcMaxM + 1) * 8);
    L.total = o;
    return L;
}

struct RcVecs {
    const double* z[kRcMaxM];
};
struct RcSys {
    const double* c;   // 5 planes: component q of cell k at c[q * cs + k * es]
    long long cs, es;
    int S, lap;
};

// (A x)[k]; reads outside [0, n) are 0 -- kc_spmv's FP64 arithmetic, operation for operation
__device__ __forceinline__ double rc_row(const RcSys& A, const double* __restrict__ x, long long n, long long k,
                                         double xk) {
    const long long e = k * A.es;
    const double c0 = __ldg(A.c + e), c1 = __ldg(A.c + A.cs + e), c2 = __ldg(A.c + 2 * A.cs + e),
                 c3 = __ldg(A.c + 3 * A.cs + e), c4 = __ldg(A.c + 4 * A.cs + e);
    const double xw = k >= A.S ? __ldg(x + k - A.S) : 0.0, xe = k + A.S < n ? __ldg(x + k + A.S) : 0.0;
    const double xs = k > 0 ? __ldg(x + k - 1) : 0.0, xn = k + 1 < n ? __ldg(x + k + 1) : 0.0;
    double v = c0 * xk;
    if (A.lap) {
        v = fma(c1, xw - xk, v);
        v = fma(c2, xe - xk, v);
        v = fma(c3, xn - xk, v);
        v = fma(c4, xs - xk, v);
    } else {
        v = fma(c1, xw, v);
        v = fma(c2, xe, v);
        v = fma(c3, xn, v);
        v = fma(c4, xs, v);
    }
    return v;
}

template <int M>
__global__ void __launch_bounds__(kRcThreads) k_rc_gram(long long n, RcSys A, RcVecs V, const double* __restrict__ b,
                                                        double* partials) {
    constexpr int NS = M * (M + 1) / 2 + M;
    double v[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) v[s] = 0.0;
    for (long long k = blockIdx.x * (long long)kRcThreads + threadIdx.x; k < n; k += (long long)gridDim.x * kRcThreads) {
        double z[M], az[M];
#pragma unroll
        for (int i = 0; i < M; ++i) z[i] = __ldg(V.z[i] + k);
#pragma unroll
        for (int i = 0; i < M; ++i) az[i] = rc_row(A, V.z[i], n, k, z[i]);
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

// Cholesky of the leading k x k block of G (m x m, symmetric): the largest k
// whose pivots stay above 1e-12 times their diagonal; y solves it, y[k..m) = 0.
__device__ int rc_solve(const double* G, const double* g, int m, double* y) {
    double Lm[kRcMaxM][kRcMaxM];
    int k = 0;
    for (int i = 0; i < m; ++i) {
        double d = G[i * m + i];
        for (int p = 0; p < i; ++p) d -= Lm[i][p] * Lm[i][p];
        if (!(d > 1e-12 * fabs(G[i * m + i])) || !isfinite(d)) break;
        Lm[i][i] = sqrt(d);
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

// fixed-order fold of the block sums, then (thread 0) the projected system's solve
template <int M>
__global__ void __launch_bounds__(kRcThreads) k_rc_fold_solve(const double* __restrict__ partials, int nb,
                                                              double* __restrict__ out, double* __restrict__ coef) {
    constexpr int NS = M * (M + 1) / 2 + M;
    double v[NS];
    reduce_partials<NS>(partials, kRcMaxBlocks, nb, v);
    if (threadIdx.x == 0) {
        double G[M * M], g[M], y[M];
        int q = 0;
#pragma unroll
        for (int i = 0; i < M; ++i)
#pragma unroll
            for (int j = i; j < M; ++j) {
                out[q] = v[q];
                G[i * M + j] = G[j * M + i] = v[q];
                ++q;
            }
#pragma unroll
        for (int i = 0; i < M; ++i) {
            out[q] = v[q];
            g[i] = v[q];
            ++q;
        }
        const int k = rc_solve(G, g, M, y);
#pragma unroll
        for (int i = 0; i < M; ++i) coef[i] = y[i];
        coef[kRcMaxM] = (double)k;
    }
}

template <int M>
__global__ void __launch_bounds__(kRcThreads) k_rc_combine(long long n, RcVecs V, const double* __restrict__ coef,
                                                           double* __restrict__ x0) {
    double y[M];
#pragma unroll
    for (int i = 0; i < M; ++i) y[i] = __ldg(coef + i);   // y[i] = 0 for a dropped vector
    for (long long k = blockIdx.x * (long long)kRcThreads + threadIdx.x; k < n; k += (long long)gridDim.x * kRcThreads) {
        double x = 0.0;
#pragma unroll
        for (int i = 0; i < M; ++i) x = fma(y[i], __ldg(V.z[i] + k), x);
        x0[k] = x;
    }
}

// cells per thread: 4 for the combine pass (memory-bound: many loads in flight), 16 for the
// Gram pass, which is bound by the FP64 pipe -- its per-thread block reduction of the
// m (m + 3) / 2 sums (70 FP64 adds at m = 4) then costs an eighth of the pass instead of half
int rc_blocks(long long n, int per_thread = 4) {
    const long long c = (long long)kRcThreads * per_thread;
    return (int)std::max<long long>(1, std::min<long long>((n + c - 1) / c, kRcMaxBlocks));
}

template <int M>
int rc_run(long long n, const RcSys& A, const RcVecs& V, const double* b, const RcLayout& L, char* base, double* x0,
           cudaStream_t s) {
    double* partials = (double*)(base + L.partials);
    double* out = (double*)(base + L.out);
    double* coef = (double*)(base + L.coef);
    const int nb = rc_blocks(n, 16);
    k_rc_gram<M><<<nb, kRcThreads, 0, s>>>(n, A, V, b, partials);
    KC_LAUNCH_CHECK("k_rc_gram");
    k_rc_fold_solve<M><<<1, kRcThreads, 0, s>>>(partials, nb, out, coef);
    KC_LAUNCH_CHECK("k_rc_fold_solve");
    k_rc_combine<M><<<rc_blocks(n), kRcThreads, 0, s>>>(n, V, coef, x0);
    KC_LAUNCH_CHECK("k_rc_combine");
    return KC_OK;
}

}  // namespace
}  // namespace kc

using namespace kc;

extern "C" {

size_t kc_recycle_ws_bytes(long long n, int m) {
    if (n < 1 || m < 1 || m > KC_RECYCLE_MAX) return 0;
    return rc_layout().total;
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
    if (!A64->coef || A64->stride < 1) return set_error("kc_recycle_guess: bad system"), KC_ERR_ARG;
    const RcLayout L = rc_layout();
    if (!ws || ws_bytes < L.total || ((uintptr_t)ws & 255))
        return set_error("kc_recycle_guess: workspace %zu bytes (256-aligned) < required %zu", ws_bytes, L.total),
               KC_ERR_WORKSPACE;
    RcVecs V{};
    for (int i = 0; i < m; ++i) {
        if (!Z[i]) return set_error("kc_recycle_guess: null vector %d", i), KC_ERR_ARG;
        V.z[i] = Z[i];
    }
    const RcSys A{(const double*)A64->coef, A64->cs, A64->es, A64->stride, A64->form == KC_FORM_LAPLACIAN};
    char* base = (char*)ws;
    int rc = KC_OK;
    switch (m) {
        case 1: rc = rc_run<1>(n, A, V, b, L, base, x0, s); break;
        case 2: rc = rc_run<2>(n, A, V, b, L, base, x0, s); break;
        case 3: rc = rc_run<3>(n, A, V, b, L, base, x0, s); break;
        default: rc = rc_run<4>(n, A, V, b, L, base, x0, s); break;
    }
    if (rc) return rc;
    if (used) {   // the count kept, when asked for, is the one host round trip
        const void* hp = readback(base + L.coef + kRcMaxM * sizeof(double), sizeof(double), s);
        if (!hp) return KC_ERR_CUDA;
        double k;
        memcpy(&k, hp, sizeof(double));
        *used = (int)k;
    }
    return KC_OK;
}

}  // extern "C"
