// Jacobi sweeps on a 5-point system (FP64): the smoother / solver paths
// jacobian_solve_u / jacobian_solve_p (pressure_valid.py:192-233) and
// quick_jacobian (debug/20210828_karman_taihi.py:375-393).
//
// The reference overwrites the iterate inside a parallel loop, so the order
// in which neighbours see new values is undefined there; this kernel does the
// iteration the names describe -- every cell reads the previous iterate:
//     x_mid = (b - sum_nb a_nb x_nb) / aP,   y = (1 - omega) x + omega x_mid
// on the cells of a rectangle of the [n/S][S] view (other cells: y = x), and
// reduces max |x_mid - x| over the rectangle (the residual the reference returns).
#include "kc_common.cuh"
#include <algorithm>

namespace kc {

constexpr int kJacThreads = 256;
constexpr int kJacMaxBlocks = 2048;

struct JacWs {
    unsigned ticket;
    unsigned pad[3];
    double part[kJacMaxBlocks];
};

__global__ void __launch_bounds__(kJacThreads)
    k_jacobi(const double* __restrict__ c, long long cs, long long es, long long n, int S, const double* __restrict__ b,
             const double* __restrict__ x, double* __restrict__ y, double omega, int i0, int i1, int j0, int j1,
             JacWs* ws, double* __restrict__ max_out) {
    double m = 0.0;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / S), j = (int)(k - (long long)i * S);
        const double xk = x[k];
        if (i < i0 || i >= i1 || j < j0 || j >= j1) {
            y[k] = xk;
            continue;
        }
        const long long e = k * es;
        const double aP = c[e];
        if (aP == 0.0) {
            y[k] = xk;
            continue;
        }
        double r = b[k];
        if (k >= S) r -= c[cs + e] * x[k - S];
        if (k + S < n) r -= c[2 * cs + e] * x[k + S];
        if (k + 1 < n) r -= c[3 * cs + e] * x[k + 1];
        if (k >= 1) r -= c[4 * cs + e] * x[k - 1];
        const double xm = r / aP;
        m = fmax(m, fabs(xm - xk));
        y[k] = (1.0 - omega) * xk + omega * xm;
    }
    double v[1] = {m};
    block_max<1>(v);   // non-negative values: the zero padding of block_max is the identity
    if (threadIdx.x == 0) ws->part[blockIdx.x] = v[0];
    if (!arrive_last(&ws->ticket, gridDim.x)) return;
    double t[1] = {0.0};
    for (unsigned q = threadIdx.x; q < gridDim.x; q += blockDim.x) t[0] = fmax(t[0], __ldcg(&ws->part[q]));
    block_max<1>(t);
    if (threadIdx.x == 0) {
        *max_out = t[0];
        ws->ticket = 0;
    }
}

}  // namespace kc

using namespace kc;

extern "C" {

size_t kc_jacobi_ws_bytes(void) { return sizeof(JacWs); }

int kc_jacobi(const kc_system* A, const double* b, const double* x, double* y, double omega, int i0, int i1, int j0,
              int j1, double* max_diff_dev, void* ws, size_t ws_bytes, void* stream) {
    if (!A || !A->coef || A->dtype != KC_F64 || A->form != KC_FORM_STANDARD || !b || !x || !y || !max_diff_dev)
        return set_error("kc_jacobi: need an FP64 standard-form system and b, x, y, max_diff"), KC_ERR_ARG;
    if (x == y) return set_error("kc_jacobi: x and y must differ (the sweep reads the previous iterate)"), KC_ERR_ARG;
    if (A->stride < 1 || A->n < 1) return set_error("kc_jacobi: bad system size"), KC_ERR_ARG;
    if (!ws || ws_bytes < sizeof(JacWs)) return set_error("kc_jacobi: workspace too small"), KC_ERR_WORKSPACE;
    const int nb = (int)std::max<long long>(1, std::min<long long>((A->n + kJacThreads - 1) / kJacThreads, kJacMaxBlocks));
    k_jacobi<<<nb, kJacThreads, 0, as_stream(stream)>>>((const double*)A->coef, A->cs, A->es, A->n, A->stride, b, x, y,
                                                         omega, i0, i1, j0, j1, (JacWs*)ws, max_diff_dev);
    KC_LAUNCH_CHECK("k_jacobi");
    return KC_OK;
}

}  // extern "C"
