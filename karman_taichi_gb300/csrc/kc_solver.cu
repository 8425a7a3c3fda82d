// Stencil linear algebra for the karman_taichi hot path on GB300 (sm_103a):
// matrix-free 5-point SpMV, deterministic FP64 dot products, and BiCGSTAB /
// CG with the vector updates fused into the stencil sweeps.
//
// Reference behaviour (file:line in houkensjtu/karman_taichi):
//   SpMV        bicgsolver.py:65-76, cgsolver.py:56-66, karman_taichi.py:362-366
//   reduce      cgsolver.py:49-54
//   BiCGSTAB    bicgsolver.py:88-135 (M = I, cold start),
//               karman_taichi.py:342-456 (right Jacobi, warm start, omega break)
//   CG          cgsolver.py:83-114
//
// Layout: every vector is a flat array of n elements; the stencil couples
// k +- 1 and k +- S.  A stencil block covers 32 consecutive columns (one per
// lane, so warp loads are fully coalesced along the contiguous index) and
// kWarps*kRows rows; each warp streams down kRows rows holding the operand of
// rows i-1, i, i+1 in registers, and takes the j +- 1 neighbours from the
// adjacent lanes with shuffles.  Only the two edge lanes and the strip ends
// recompute a neighbour from global memory.
//
// One BiCGSTAB iteration is three launches (27 words of traffic per cell):
//   A  p = r + beta (p - omega v) [x M^-1]  ->  v = A p^,   partial (r~, v)
//   B  s = r - alpha v [x M^-1]             ->  t = A s^,   partials (t, s), (t, t)
//   C  x += alpha p^ + omega s^,  r = s - omega t,          partials (r, r~), (r, r)
// The last block of each launch reduces the partials in a fixed order and
// advances the scalar recurrence on the device, so the host never waits on a
// dot product; it polls a "done" word once per chunk of iterations.
#include "kc_common.cuh"
#include <algorithm>
#include <mutex>
#include <map>
#include <tuple>

namespace kc {

constexpr int kWarps = 8;   // warps per stencil block (256 threads)
constexpr int kRows = 8;    // rows streamed by each warp
constexpr int kThreads = kWarps * kWarp;
constexpr int kPwThreads = 256;   // pointwise kernels
constexpr int kPwMaxBlocks = 2048;

struct SolverState {
    double rho, rho_1, alpha, omega, beta;
    double r0Tr, rTr, den, eps, old;
    double prev_rel;
    long long iter, max_iter;
    int status, done, omega_break, rel_to;
    unsigned ticket[4];
    double* hist;
    long long hist_len;
};

__device__ __forceinline__ void record_history(SolverState* st, long long k, double rr) {
    if (st->hist && k < st->hist_len) st->hist[k] = sqrt(rr);
}

template <typename T>
struct Coef {
    const T* c;
    long long cs, es;
    __device__ __forceinline__ T at(int comp, long long k) const { return __ldg(c + comp * cs + k * es); }
};

struct Geo {
    long long n;
    int S;
};

static inline dim3 stencil_grid(long long n, int S) {
    long long rows = (n + S - 1) / S;
    long long gx = (S + kWarp - 1) / kWarp;
    long long gy = (rows + kWarps * kRows - 1) / (kWarps * kRows);
    return dim3((unsigned)gx, (unsigned)gy);
}
static inline bool stencil_grid_ok(long long n, int S) {
    if (S < 1 || n < 1) return false;
    dim3 g = stencil_grid(n, S);
    return g.y <= 65535u && (long long)g.x * g.y <= (1ll << 31);
}
static inline int pw_blocks(long long n) {
    long long b = (n + kPwThreads * 4 - 1) / (kPwThreads * 4);
    return (int)std::max<long long>(1, std::min<long long>(b, kPwMaxBlocks));
}

template <typename T>
__device__ __forceinline__ T fmaT(T a, T b, T c) { return fma(a, b, c); }
template <>
__device__ __forceinline__ float fmaT<float>(float a, float b, float c) { return fmaf(a, b, c); }

// -----------------------------------------------------------------------------
// Streaming stencil strip.  Pol provides:
//   Val owner(k)   operand at k for the owning thread (may store side outputs)
//   T   halo(k)    operand at k recomputed for a neighbour (no side effects)
//   void sink(k, y, center, acc)   consumes y = (A operand)[k]
// -----------------------------------------------------------------------------
template <typename T, int NACC, class Pol>
__device__ __forceinline__ void stencil_strip(const Pol& pol, const Coef<T> A, long long n, int S,
                                              double (&acc)[NACC]) {
    using Val = typename Pol::Val;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long long j = (long long)blockIdx.x * kWarp + lane;
    const bool colok = j < S;
    const long long i0 = ((long long)blockIdx.y * kWarps + w) * kRows;
    if (i0 * (long long)S >= n) return;  // whole warp below the last row (warp-uniform)
    long long k = i0 * S + j;
    Val c = (colok && k < n) ? pol.owner(k) : Val::zero();
    T xm = (colok && i0 > 0 && k < n) ? pol.halo(k - S) : T(0);
#pragma unroll 2
    for (int r = 0; r < kRows; ++r) {
        const long long kn = k + S;
        const bool okc = colok && k < n;
        const bool okn = colok && kn < n;
        Val nxt = Val::zero();
        T xp;
        if (r + 1 < kRows) {
            if (okn) nxt = pol.owner(kn);
            xp = nxt.op;
        } else {
            xp = okn ? pol.halo(kn) : T(0);
        }
        T xl = __shfl_up_sync(kFull, c.op, 1);
        T xr = __shfl_down_sync(kFull, c.op, 1);
        if (lane == 0) xl = (okc && k >= 1) ? pol.halo(k - 1) : T(0);
        if (lane == kWarp - 1 || j == S - 1) xr = (okc && k + 1 < n) ? pol.halo(k + 1) : T(0);
        if (okc) {
            T y = A.at(0, k) * c.op;
            y = fmaT<T>(A.at(1, k), xm, y);
            y = fmaT<T>(A.at(2, k), xp, y);
            y = fmaT<T>(A.at(3, k), xr, y);
            y = fmaT<T>(A.at(4, k), xl, y);
            pol.sink(k, y, c, acc);
        }
        xm = c.op;
        c = nxt;
        k = kn;
    }
}

// ---- plain SpMV ---------------------------------------------------------------
template <typename T>
struct PolSpmv {
    const T* x;
    T* y;
    struct Val {
        T op;
        __device__ static Val zero() { return {T(0)}; }
    };
    __device__ Val owner(long long k) const { return {x[k]}; }
    __device__ T halo(long long k) const { return x[k]; }
    __device__ void sink(long long k, T v, const Val&, double (&)[1]) const { y[k] = v; }
};

template <typename T>
__global__ void __launch_bounds__(kThreads) k_spmv(Coef<T> A, Geo g, const T* x, T* y) {
    double acc[1] = {0.0};
    PolSpmv<T> pol{x, y};
    stencil_strip<T, 1>(pol, A, g.n, g.S, acc);
}

// ---- dot ----------------------------------------------------------------------
struct DotWs {
    unsigned ticket[4];
    double pad[2];
    double partials[kPwMaxBlocks];
};

template <typename T>
__global__ void __launch_bounds__(kPwThreads) k_dot(long long n, const T* p, const T* q, DotWs* ws,
                                                    double* out) {
    double acc[1] = {0.0};
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x)
        acc[0] += (double)p[k] * (double)q[k];
    block_sum<1>(acc);
    if (threadIdx.x == 0) ws->partials[blockIdx.x] = acc[0];
    if (arrive_last(&ws->ticket[0], gridDim.x)) {
        double s[1];
        reduce_partials<1>(ws->partials, 0, gridDim.x, s);
        if (threadIdx.x == 0) {
            *out = s[0];
            ws->ticket[0] = 0;
        }
    }
}

// =============================================================================
// BiCGSTAB
// =============================================================================
struct BicgPtrs {
    SolverState* st;
    double* partials;  // [4][ld]
    int ld;
};

__device__ __forceinline__ bool solver_done(const SolverState* st) {
    return __ldcg(&st->done) != 0;
}

// Called by thread 0 of the last block of pass C with (r, r~) and (r, r).
__device__ void bicg_finish_iteration(SolverState* st, double rho_new, double rTr) {
    st->iter += 1;
    st->rTr = rTr;
    record_history(st, st->iter, rTr);
    double rel = st->den > 0.0 ? sqrt(rTr / st->den) : 0.0;
    st->prev_rel = rel;
    if (rel < st->eps) {
        st->status = KC_OK;
        st->done = 1;
    } else if (!isfinite(rTr)) {
        st->status = KC_NONFINITE;
        st->done = 1;
    } else if (st->omega_break && st->omega == 0.0) {
        st->status = KC_BREAKDOWN_OMEGA;
        st->done = 1;
    } else if (st->iter >= st->max_iter) {
        st->status = KC_MAXITER;
        st->done = 1;
    } else if (rho_new == 0.0) {
        st->status = KC_BREAKDOWN_RHO;
        st->done = 1;
    } else {
        st->rho_1 = st->rho;
        st->rho = rho_new;
        st->beta = (st->rho / st->rho_1) * (st->alpha / st->omega);
    }
}

struct StartArgs {
    double eps;
    long long max_iter;
    int omega_break, rel_to;
    double* hist;
    long long hist_len;
};

__device__ void bicg_start(SolverState* st, double r0Tr, double bb, const StartArgs& a) {
    const double eps = a.eps;
    const long long max_iter = a.max_iter;
    const int omega_break = a.omega_break, rel_to = a.rel_to;
    st->hist = a.hist;
    st->hist_len = a.hist_len;
    record_history(st, 0, r0Tr);
    st->iter = 0;
    st->max_iter = max_iter;
    st->eps = eps;
    st->omega_break = omega_break;
    st->rel_to = rel_to;
    st->r0Tr = r0Tr;
    st->rTr = r0Tr;
    st->den = rel_to == KC_REL_B ? bb : r0Tr;
    st->rho = r0Tr;  // r~ = r0, so rho_0 = (r0, r0)
    st->rho_1 = st->alpha = st->omega = 1.0;
    st->beta = 0.0;
    st->old = r0Tr;
    st->status = KC_MAXITER;
    st->done = 0;
    st->prev_rel = st->den > 0.0 ? sqrt(r0Tr / st->den) : 0.0;
    if (r0Tr == 0.0) {  // x already solves the system exactly
        st->status = KC_OK;
        st->done = 1;
    } else if (!isfinite(r0Tr)) {
        st->status = KC_NONFINITE;
        st->done = 1;
    } else if (rel_to == KC_REL_B && st->prev_rel < eps) {
        st->status = KC_OK;
        st->done = 1;
    } else if (max_iter <= 0) {
        st->status = KC_MAXITER;
        st->done = 1;
    }
}

// cold start: r = r~ = b, x = 0; optional invM = 1/M
template <typename T>
__global__ void __launch_bounds__(kPwThreads)
    k_bicg_init_cold(long long n, const T* b, T* x, T* r, T* rt, const T* M, T* invM, BicgPtrs P,
                     StartArgs sa) {
    double acc[1] = {0.0};
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        T bk = b[k];
        r[k] = bk;
        rt[k] = bk;
        x[k] = T(0);
        if (M) invM[k] = T(1) / M[k];
        acc[0] += (double)bk * (double)bk;
    }
    block_sum<1>(acc);
    if (threadIdx.x == 0) P.partials[blockIdx.x] = acc[0];
    if (arrive_last(&P.st->ticket[0], gridDim.x)) {
        double s[1];
        reduce_partials<1>(P.partials, P.ld, gridDim.x, s);
        if (threadIdx.x == 0) {
            bicg_start(P.st, s[0], s[0], sa);
            P.st->ticket[0] = 0;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(kPwThreads) k_invdiag(long long n, const T* M, T* invM) {
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x)
        invM[k] = T(1) / M[k];
}

// warm start: r = r~ = b - A x
template <typename T>
struct PolWarm {
    const T* x;
    const T* b;
    T* r;
    T* rt;
    struct Val {
        T op;
        __device__ static Val zero() { return {T(0)}; }
    };
    __device__ Val owner(long long k) const { return {x[k]}; }
    __device__ T halo(long long k) const { return x[k]; }
    __device__ void sink(long long k, T y, const Val&, double (&acc)[2]) const {
        T bk = b[k];
        T rk = bk - y;
        r[k] = rk;
        rt[k] = rk;
        acc[0] += (double)rk * (double)rk;
        acc[1] += (double)bk * (double)bk;
    }
};

template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_bicg_init_warm(Coef<T> A, Geo g, const T* b, const T* x, T* r, T* rt, BicgPtrs P, StartArgs sa) {
    double acc[2] = {0.0, 0.0};
    PolWarm<T> pol{x, b, r, rt};
    stencil_strip<T, 2>(pol, A, g.n, g.S, acc);
    block_sum<2>(acc);
    const int nb = gridDim.x * gridDim.y;
    const int bid = blockIdx.y * gridDim.x + blockIdx.x;
    if (threadIdx.x == 0) {
        P.partials[bid] = acc[0];
        P.partials[P.ld + bid] = acc[1];
    }
    if (arrive_last(&P.st->ticket[0], nb)) {
        double s[2];
        reduce_partials<2>(P.partials, P.ld, nb, s);
        if (threadIdx.x == 0) {
            bicg_start(P.st, s[0], s[1], sa);
            P.st->ticket[0] = 0;
        }
    }
}

// pass A: p = r + beta (p_old - omega v_old); v = A p^; partial (r~, v)
template <typename T, bool PRE>
struct PolA {
    const T* r;
    const T* p_old;
    const T* v_old;
    T* p_new;
    const T* invM;
    const T* rt;
    T* v;
    T beta, omega;
    bool first;
    struct Val {
        T op;
        __device__ static Val zero() { return {T(0)}; }
    };
    __device__ __forceinline__ T pval(long long k) const {
        T rk = r[k];
        if (first) return rk;
        T d = fmaT<T>(-omega, v_old[k], p_old[k]);
        return fmaT<T>(beta, d, rk);
    }
    __device__ Val owner(long long k) const {
        T p = pval(k);
        p_new[k] = p;
        return {PRE ? p * invM[k] : p};
    }
    __device__ T halo(long long k) const {
        T p = pval(k);
        return PRE ? p * invM[k] : p;
    }
    __device__ void sink(long long k, T y, const Val&, double (&acc)[1]) const {
        v[k] = y;
        acc[0] += (double)rt[k] * (double)y;
    }
};

struct BicgVecs {
    void* r;
    void* rt;
    void* p[2];
    void* v[2];
    void* t;
    void* invM;
};

template <typename T, bool PRE>
__global__ void __launch_bounds__(kThreads) k_bicg_A(Coef<T> A, Geo g, BicgVecs V, BicgPtrs P) {
    SolverState* st = P.st;
    if (solver_done(st)) return;
    const long long it = __ldcg(&st->iter);
    const int cur = (int)(it & 1), nxt = cur ^ 1;
    PolA<T, PRE> pol;
    pol.r = (const T*)V.r;
    pol.p_old = (const T*)V.p[cur];
    pol.v_old = (const T*)V.v[cur];
    pol.p_new = (T*)V.p[nxt];
    pol.invM = (const T*)V.invM;
    pol.rt = (const T*)V.rt;
    pol.v = (T*)V.v[nxt];
    pol.beta = (T)__ldcg(&st->beta);
    pol.omega = (T)__ldcg(&st->omega);
    pol.first = it == 0;
    double acc[1] = {0.0};
    stencil_strip<T, 1>(pol, A, g.n, g.S, acc);
    block_sum<1>(acc);
    const int nb = gridDim.x * gridDim.y;
    const int bid = blockIdx.y * gridDim.x + blockIdx.x;
    if (threadIdx.x == 0) P.partials[bid] = acc[0];
    if (arrive_last(&st->ticket[0], nb)) {
        double s[1];
        reduce_partials<1>(P.partials, P.ld, nb, s);
        if (threadIdx.x == 0) {
            double alpha = st->rho / s[0];
            st->alpha = alpha;
            if (!isfinite(alpha)) {
                st->status = KC_NONFINITE;
                st->done = 1;
            }
            st->ticket[0] = 0;
        }
    }
}

// pass B: s = r - alpha v; t = A s^; partials (t, s), (t, t)
template <typename T, bool PRE>
struct PolB {
    const T* r;
    const T* v;
    const T* invM;
    T* t;
    T alpha;
    struct Val {
        T op, s;
        __device__ static Val zero() { return {T(0), T(0)}; }
    };
    __device__ __forceinline__ T sval(long long k) const { return fmaT<T>(-alpha, v[k], r[k]); }
    __device__ Val owner(long long k) const {
        T s = sval(k);
        return {PRE ? s * invM[k] : s, s};
    }
    __device__ T halo(long long k) const {
        T s = sval(k);
        return PRE ? s * invM[k] : s;
    }
    __device__ void sink(long long k, T y, const Val& c, double (&acc)[2]) const {
        t[k] = y;
        acc[0] += (double)y * (double)c.s;
        acc[1] += (double)y * (double)y;
    }
};

template <typename T, bool PRE>
__global__ void __launch_bounds__(kThreads) k_bicg_B(Coef<T> A, Geo g, BicgVecs V, BicgPtrs P) {
    SolverState* st = P.st;
    if (solver_done(st)) return;
    const long long it = __ldcg(&st->iter);
    const int nxt = (int)((it + 1) & 1);
    PolB<T, PRE> pol;
    pol.r = (const T*)V.r;
    pol.v = (const T*)V.v[nxt];
    pol.invM = (const T*)V.invM;
    pol.t = (T*)V.t;
    pol.alpha = (T)__ldcg(&st->alpha);
    double acc[2] = {0.0, 0.0};
    stencil_strip<T, 2>(pol, A, g.n, g.S, acc);
    block_sum<2>(acc);
    const int nb = gridDim.x * gridDim.y;
    const int bid = blockIdx.y * gridDim.x + blockIdx.x;
    if (threadIdx.x == 0) {
        P.partials[bid] = acc[0];
        P.partials[P.ld + bid] = acc[1];
    }
    if (arrive_last(&st->ticket[0], nb)) {
        double s[2];
        reduce_partials<2>(P.partials, P.ld, nb, s);
        if (threadIdx.x == 0) {
            double omega = s[0] / s[1];
            st->omega = omega;
            if (!isfinite(omega)) {
                st->status = KC_NONFINITE;
                st->done = 1;
            }
            st->ticket[0] = 0;
        }
    }
}

// pass C: x += alpha p^ + omega s^; r = s - omega t; partials (r, r~), (r, r)
template <typename T, bool PRE>
__global__ void __launch_bounds__(kPwThreads) k_bicg_C(long long n, T* x, BicgVecs V, BicgPtrs P) {
    SolverState* st = P.st;
    if (solver_done(st)) return;
    const long long it = __ldcg(&st->iter);
    const int nxt = (int)((it + 1) & 1);
    const T* p = (const T*)V.p[nxt];
    const T* v = (const T*)V.v[nxt];
    const T* t = (const T*)V.t;
    const T* rt = (const T*)V.rt;
    const T* invM = (const T*)V.invM;
    T* r = (T*)V.r;
    const T alpha = (T)__ldcg(&st->alpha), omega = (T)__ldcg(&st->omega);
    double acc[2] = {0.0, 0.0};
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        T rk = r[k];
        T s = fmaT<T>(-alpha, v[k], rk);
        T ph = p[k], sh = s;
        if (PRE) {
            T im = invM[k];
            ph = ph * im;
            sh = sh * im;
        }
        x[k] = x[k] + fmaT<T>(alpha, ph, omega * sh);
        T rn = fmaT<T>(-omega, t[k], s);
        r[k] = rn;
        acc[0] += (double)rn * (double)rt[k];
        acc[1] += (double)rn * (double)rn;
    }
    block_sum<2>(acc);
    if (threadIdx.x == 0) {
        P.partials[blockIdx.x] = acc[0];
        P.partials[P.ld + blockIdx.x] = acc[1];
    }
    if (arrive_last(&st->ticket[0], gridDim.x)) {
        double s[2];
        reduce_partials<2>(P.partials, P.ld, gridDim.x, s);
        if (threadIdx.x == 0) {
            bicg_finish_iteration(st, s[0], s[1]);
            st->ticket[0] = 0;
        }
    }
}

// =============================================================================
// CG (cgsolver.py:83-114), two passes per iteration
//   1  p = r + beta p_old  ->  Ap = A p,  partial (p, Ap)
//   2  x += alpha p, r -= alpha Ap,       partial (r, r)
// =============================================================================
template <typename T>
__global__ void __launch_bounds__(kPwThreads)
    k_cg_init(long long n, const T* b, T* x, T* r, BicgPtrs P, StartArgs sa) {
    double acc[1] = {0.0};
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        T bk = b[k];
        r[k] = bk;
        x[k] = T(0);
        acc[0] += (double)bk * (double)bk;
    }
    block_sum<1>(acc);
    if (threadIdx.x == 0) P.partials[blockIdx.x] = acc[0];
    if (arrive_last(&P.st->ticket[0], gridDim.x)) {
        double s[1];
        reduce_partials<1>(P.partials, P.ld, gridDim.x, s);
        if (threadIdx.x == 0) {
            bicg_start(P.st, s[0], s[0], sa);
            P.st->ticket[0] = 0;
        }
    }
}

template <typename T>
struct PolCg1 {
    const T* r;
    const T* p_old;
    T* p_new;
    T* Ap;
    T beta;
    bool first;
    struct Val {
        T op;
        __device__ static Val zero() { return {T(0)}; }
    };
    __device__ __forceinline__ T pval(long long k) const {
        return first ? r[k] : fmaT<T>(beta, p_old[k], r[k]);
    }
    __device__ Val owner(long long k) const {
        T p = pval(k);
        p_new[k] = p;
        return {p};
    }
    __device__ T halo(long long k) const { return pval(k); }
    __device__ void sink(long long k, T y, const Val& c, double (&acc)[1]) const {
        Ap[k] = y;
        acc[0] += (double)c.op * (double)y;
    }
};

template <typename T>
__global__ void __launch_bounds__(kThreads) k_cg_1(Coef<T> A, Geo g, BicgVecs V, BicgPtrs P) {
    SolverState* st = P.st;
    if (solver_done(st)) return;
    const long long it = __ldcg(&st->iter);
    const int cur = (int)(it & 1), nxt = cur ^ 1;
    PolCg1<T> pol;
    pol.r = (const T*)V.r;
    pol.p_old = (const T*)V.p[cur];
    pol.p_new = (T*)V.p[nxt];
    pol.Ap = (T*)V.v[0];
    pol.beta = (T)__ldcg(&st->beta);
    pol.first = it == 0;
    double acc[1] = {0.0};
    stencil_strip<T, 1>(pol, A, g.n, g.S, acc);
    block_sum<1>(acc);
    const int nb = gridDim.x * gridDim.y;
    const int bid = blockIdx.y * gridDim.x + blockIdx.x;
    if (threadIdx.x == 0) P.partials[bid] = acc[0];
    if (arrive_last(&st->ticket[0], nb)) {
        double s[1];
        reduce_partials<1>(P.partials, P.ld, nb, s);
        if (threadIdx.x == 0) {
            double alpha = st->old / s[0];
            st->alpha = alpha;
            if (!isfinite(alpha)) {
                st->status = KC_NONFINITE;
                st->done = 1;
            }
            st->ticket[0] = 0;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(kPwThreads) k_cg_2(long long n, T* x, BicgVecs V, BicgPtrs P) {
    SolverState* st = P.st;
    if (solver_done(st)) return;
    const long long it = __ldcg(&st->iter);
    const int nxt = (int)((it + 1) & 1);
    const T* p = (const T*)V.p[nxt];
    const T* Ap = (const T*)V.v[0];
    T* r = (T*)V.r;
    const T alpha = (T)__ldcg(&st->alpha);
    double acc[1] = {0.0};
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        x[k] = fmaT<T>(alpha, p[k], x[k]);
        T rn = fmaT<T>(-alpha, Ap[k], r[k]);
        r[k] = rn;
        acc[0] += (double)rn * (double)rn;
    }
    block_sum<1>(acc);
    if (threadIdx.x == 0) P.partials[blockIdx.x] = acc[0];
    if (arrive_last(&st->ticket[0], gridDim.x)) {
        double s[1];
        reduce_partials<1>(P.partials, P.ld, gridDim.x, s);
        if (threadIdx.x == 0) {
            double nw = s[0];
            st->iter += 1;
            st->rTr = nw;
            record_history(st, st->iter, nw);
            st->prev_rel = st->r0Tr > 0 ? sqrt(nw) / sqrt(st->r0Tr) : 0.0;
            if (sqrt(nw) < sqrt(st->r0Tr) * st->eps) {
                st->status = KC_OK;
                st->done = 1;
            } else if (!isfinite(nw)) {
                st->status = KC_NONFINITE;
                st->done = 1;
            } else if (st->iter >= st->max_iter) {
                st->status = KC_MAXITER;
                st->done = 1;
            } else {
                st->beta = nw / st->old;
                st->old = nw;
            }
            st->ticket[0] = 0;
        }
    }
}

// =============================================================================
// Mixed precision refinement helpers
// =============================================================================
struct PolResid {
    const double* x;
    const double* b;
    float* r32;
    struct Val {
        double op;
        __device__ static Val zero() { return {0.0}; }
    };
    __device__ Val owner(long long k) const { return {x[k]}; }
    __device__ double halo(long long k) const { return x[k]; }
    __device__ void sink(long long k, double y, const Val&, double (&acc)[2]) const {
        double bk = b[k];
        double rk = bk - y;
        r32[k] = (float)rk;
        acc[0] += rk * rk;
        acc[1] += bk * bk;
    }
};

__global__ void __launch_bounds__(kThreads)
    k_refine_resid(Coef<double> A, Geo g, const double* b, const double* x, float* r32, BicgPtrs P,
                   double* out2) {
    double acc[2] = {0.0, 0.0};
    PolResid pol{x, b, r32};
    stencil_strip<double, 2>(pol, A, g.n, g.S, acc);
    block_sum<2>(acc);
    const int nb = gridDim.x * gridDim.y;
    const int bid = blockIdx.y * gridDim.x + blockIdx.x;
    if (threadIdx.x == 0) {
        P.partials[bid] = acc[0];
        P.partials[P.ld + bid] = acc[1];
    }
    if (arrive_last(&P.st->ticket[0], nb)) {
        double s[2];
        reduce_partials<2>(P.partials, P.ld, nb, s);
        if (threadIdx.x == 0) {
            out2[0] = s[0];
            out2[1] = s[1];
            P.st->ticket[0] = 0;
        }
    }
}

__global__ void __launch_bounds__(kPwThreads) k_add_f32_to_f64(long long n, const float* d, double* x) {
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x)
        x[k] += (double)d[k];
}

__global__ void k_zero_f64(long long n, double* x) {
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x)
        x[k] = 0.0;
}

// =============================================================================
// Host side
// =============================================================================
static inline size_t esize(int dtype) { return dtype == KC_F64 ? 8 : 4; }

struct BicgLayout {
    size_t off_state, off_partials, off_vec[8], total;
    int ld;
};

// vectors: 0 r, 1 rt, 2 p0, 3 p1, 4 v0, 5 v1, 6 t, 7 invM
static BicgLayout bicg_layout(long long n, int S, int dtype) {
    BicgLayout L{};
    dim3 g = stencil_grid(n, std::max(S, 1));
    int nb = std::max<int>((int)(g.x * g.y), pw_blocks(n));
    L.ld = (int)align256((size_t)nb * 8) / 8;
    size_t off = 0;
    L.off_state = off;
    off = align256(off + sizeof(SolverState));
    L.off_partials = off;
    off = align256(off + (size_t)4 * L.ld * sizeof(double));
    for (int q = 0; q < 8; ++q) {
        L.off_vec[q] = off;
        off = align256(off + (size_t)n * esize(dtype));
    }
    L.total = off;
    return L;
}

static int check_system(const kc_system* A) {
    if (!A || !A->coef) return set_error("kc_system: null system or coefficients"), KC_ERR_ARG;
    if (A->n < 1) return set_error("kc_system: n = %lld < 1", A->n), KC_ERR_ARG;
    if (A->dtype != KC_F64 && A->dtype != KC_F32)
        return set_error("kc_system: dtype %d is neither KC_F64 nor KC_F32", A->dtype), KC_ERR_ARG;
    if (!stencil_grid_ok(A->n, A->stride))
        return set_error("kc_system: stride %d unsupported for n = %lld", A->stride, A->n), KC_ERR_ARG;
    if (A->cs < 0 || A->es < 1)
        return set_error("kc_system: bad coefficient strides cs=%lld es=%lld", A->cs, A->es), KC_ERR_ARG;
    return KC_OK;
}

template <typename T>
static Coef<T> coef_of(const kc_system* A) {
    return Coef<T>{(const T*)A->coef, A->cs, A->es};
}

struct HostState {
    int status, done;
    long long iter;
    double rTr, den, r0Tr, prev_rel;
};

static int read_state(const SolverState* st, HostState* h, cudaStream_t s) {
    SolverState tmp;
    KC_CUDA(cudaMemcpyAsync(&tmp, st, sizeof(SolverState), cudaMemcpyDeviceToHost, s));
    KC_CUDA(cudaStreamSynchronize(s));
    h->status = tmp.status;
    h->done = tmp.done;
    h->iter = tmp.iter;
    h->rTr = tmp.rTr;
    h->den = tmp.den;
    h->r0Tr = tmp.r0Tr;
    h->prev_rel = tmp.prev_rel;
    return KC_OK;
}

// ---- CUDA-graph cache for chunks of iterations --------------------------------
struct GraphKey {
    const void* ws;
    const void* coef;
    const void* x;
    long long n;
    int stride, dtype, pre, chunk, kind;
    long long cs, es;
    bool operator<(const GraphKey& o) const {
        return std::tie(ws, coef, x, n, stride, dtype, pre, chunk, kind, cs, es) <
               std::tie(o.ws, o.coef, o.x, o.n, o.stride, o.dtype, o.pre, o.chunk, o.kind, o.cs, o.es);
    }
};
static std::mutex g_graph_mu;
static std::map<std::pair<int, GraphKey>, cudaGraphExec_t> g_graphs;

template <typename T, bool PRE>
static void launch_bicg_iters(const kc_system* A, T* x, const BicgVecs& V, const BicgPtrs& P, int m,
                              cudaStream_t s) {
    Geo g{A->n, A->stride};
    dim3 sg = stencil_grid(A->n, A->stride);
    int pb = pw_blocks(A->n);
    Coef<T> C = coef_of<T>(A);
    for (int q = 0; q < m; ++q) {
        k_bicg_A<T, PRE><<<sg, kThreads, 0, s>>>(C, g, V, P);
        k_bicg_B<T, PRE><<<sg, kThreads, 0, s>>>(C, g, V, P);
        k_bicg_C<T, PRE><<<pb, kPwThreads, 0, s>>>(A->n, x, V, P);
    }
}

template <typename T>
static void launch_cg_iters(const kc_system* A, T* x, const BicgVecs& V, const BicgPtrs& P, int m,
                            cudaStream_t s) {
    Geo g{A->n, A->stride};
    dim3 sg = stencil_grid(A->n, A->stride);
    int pb = pw_blocks(A->n);
    Coef<T> C = coef_of<T>(A);
    for (int q = 0; q < m; ++q) {
        k_cg_1<T><<<sg, kThreads, 0, s>>>(C, g, V, P);
        k_cg_2<T><<<pb, kPwThreads, 0, s>>>(A->n, x, V, P);
    }
}

// Runs chunks of iterations (directly or as a cached CUDA graph) until the
// device marks the solve done.  Launcher(m, stream) enqueues m iterations.
template <class Launcher>
static int drive(const kc_solve_opts* o, const GraphKey& key, const SolverState* st, Launcher&& launch,
                 HostState* h, cudaStream_t s) {
    int rc = read_state(st, h, s);
    if (rc) return rc;
    long long launched = 0;
    const long long cap = h->done ? 0 : std::max<long long>(o->max_iter, 0);
    int chunk = o->check_every > 0 ? o->check_every : 4;
    const bool fixed = o->check_every > 0;
    const int gchunk = 16;
    while (!h->done && launched < cap) {
        int m = (int)std::min<long long>(chunk, cap - launched);
        if (o->use_graph && m == gchunk) {
            int dev = 0;
            KC_CUDA(cudaGetDevice(&dev));
            cudaGraphExec_t ex = nullptr;
            {
                std::lock_guard<std::mutex> lk(g_graph_mu);
                auto it = g_graphs.find({dev, key});
                if (it != g_graphs.end()) ex = it->second;
            }
            if (!ex) {
                cudaStream_t cap_s;
                KC_CUDA(cudaStreamCreateWithFlags(&cap_s, cudaStreamNonBlocking));
                cudaGraph_t graph;
                KC_CUDA(cudaStreamBeginCapture(cap_s, cudaStreamCaptureModeThreadLocal));
                launch(m, cap_s);
                cudaError_t e = cudaStreamEndCapture(cap_s, &graph);
                cudaStreamDestroy(cap_s);
                if (e != cudaSuccess) return cuda_status(e, "cudaStreamEndCapture");
                e = cudaGraphInstantiate(&ex, graph, 0);
                cudaGraphDestroy(graph);
                if (e != cudaSuccess) return cuda_status(e, "cudaGraphInstantiate");
                std::lock_guard<std::mutex> lk(g_graph_mu);
                if (g_graphs.size() >= 64) {  // bounded cache: drop everything when full
                    for (auto& kv : g_graphs) cudaGraphExecDestroy(kv.second);
                    g_graphs.clear();
                }
                g_graphs[{dev, key}] = ex;
            }
            KC_CUDA(cudaGraphLaunch(ex, s));
        } else {
            launch(m, s);
            KC_LAUNCH_CHECK("solver iteration launch");
        }
        launched += m;
        rc = read_state(st, h, s);
        if (rc) return rc;
        if (!fixed) chunk = std::min(chunk * 2, gchunk);
    }
    return KC_OK;
}

}  // namespace kc

using namespace kc;

extern "C" {

int kc_spmv(const kc_system* A, const void* x, void* y, void* stream) {
    int rc = check_system(A);
    if (rc) return rc;
    if (!x || !y) return set_error("kc_spmv: null x or y"), KC_ERR_ARG;
    cudaStream_t s = as_stream(stream);
    Geo g{A->n, A->stride};
    dim3 sg = stencil_grid(A->n, A->stride);
    if (A->dtype == KC_F64)
        k_spmv<double><<<sg, kThreads, 0, s>>>(coef_of<double>(A), g, (const double*)x, (double*)y);
    else
        k_spmv<float><<<sg, kThreads, 0, s>>>(coef_of<float>(A), g, (const float*)x, (float*)y);
    KC_LAUNCH_CHECK("k_spmv");
    return KC_OK;
}

size_t kc_dot_ws_bytes(long long n) {
    (void)n;
    return sizeof(DotWs);
}

int kc_dot(int dtype, long long n, const void* p, const void* q, double* out_dev, void* ws,
           size_t ws_bytes, void* stream) {
    if (n < 1 || !p || !q || !out_dev) return set_error("kc_dot: bad arguments"), KC_ERR_ARG;
    if (!ws || ws_bytes < sizeof(DotWs)) return set_error("kc_dot: workspace too small"), KC_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    int nb = pw_blocks(n);
    if (dtype == KC_F64)
        k_dot<double><<<nb, kPwThreads, 0, s>>>(n, (const double*)p, (const double*)q, (DotWs*)ws, out_dev);
    else if (dtype == KC_F32)
        k_dot<float><<<nb, kPwThreads, 0, s>>>(n, (const float*)p, (const float*)q, (DotWs*)ws, out_dev);
    else
        return set_error("kc_dot: bad dtype %d", dtype), KC_ERR_ARG;
    KC_LAUNCH_CHECK("k_dot");
    return KC_OK;
}

size_t kc_bicgstab_ws_bytes(long long n, int stride, int dtype) {
    if (n < 1 || stride < 1) return 0;
    return bicg_layout(n, stride, dtype).total;
}

size_t kc_cg_ws_bytes(long long n, int stride, int dtype) { return kc_bicgstab_ws_bytes(n, stride, dtype); }

static int bicg_impl(const kc_system* A, const void* b, void* x, const void* M, void* ws, size_t ws_bytes,
                     const kc_solve_opts* o, kc_solve_info* info, void* stream, bool is_cg) {
    int rc = check_system(A);
    if (rc) return rc;
    if (!b || !x || !o) return set_error("solver: null b, x or opts"), KC_ERR_ARG;
    if (o->precond == KC_PRECOND_JACOBI && !M)
        return set_error("solver: Jacobi preconditioner requested without M"), KC_ERR_ARG;
    if (o->precond != KC_PRECOND_NONE && o->precond != KC_PRECOND_JACOBI)
        return set_error("solver: unknown preconditioner %d", o->precond), KC_ERR_ARG;
    BicgLayout L = bicg_layout(A->n, A->stride, A->dtype);
    if (!ws || ws_bytes < L.total)
        return set_error("solver: workspace %zu bytes < required %zu", ws_bytes, L.total), KC_ERR_WORKSPACE;
    if (((uintptr_t)ws & 255) != 0) return set_error("solver: workspace not 256-byte aligned"), KC_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    char* base = (char*)ws;
    BicgPtrs P{(SolverState*)(base + L.off_state), (double*)(base + L.off_partials), L.ld};
    BicgVecs V{base + L.off_vec[0], base + L.off_vec[1], {base + L.off_vec[2], base + L.off_vec[3]},
               {base + L.off_vec[4], base + L.off_vec[5]}, base + L.off_vec[6], base + L.off_vec[7]};
    const bool pre = o->precond == KC_PRECOND_JACOBI;
    const int pb = pw_blocks(A->n);
    Geo g{A->n, A->stride};
    dim3 sg = stencil_grid(A->n, A->stride);
    const long long max_iter = o->max_iter;
    GraphKey key{ws, A->coef, x, A->n, A->stride, A->dtype, pre ? 1 : 0, 16, is_cg ? 1 : 0, A->cs, A->es};
    HostState h{};
    StartArgs sa{o->eps, max_iter, o->omega_break, o->rel_to, o->history, o->history ? o->history_len : 0};
    StartArgs sa_cg{o->eps, max_iter, 0, KC_REL_R0, o->history, o->history ? o->history_len : 0};
    KC_CUDA(cudaMemsetAsync(P.st, 0, sizeof(SolverState), s));
    if (A->dtype == KC_F64) {
        using T = double;
        if (is_cg) {
            k_cg_init<T><<<pb, kPwThreads, 0, s>>>(A->n, (const T*)b, (T*)x, (T*)V.r, P, sa_cg);
        } else if (o->x0 == KC_X0_WARM) {
            if (pre) k_invdiag<T><<<pb, kPwThreads, 0, s>>>(A->n, (const T*)M, (T*)V.invM);
            k_bicg_init_warm<T><<<sg, kThreads, 0, s>>>(coef_of<T>(A), g, (const T*)b, (const T*)x, (T*)V.r,
                                                        (T*)V.rt, P, sa);
        } else {
            k_bicg_init_cold<T><<<pb, kPwThreads, 0, s>>>(A->n, (const T*)b, (T*)x, (T*)V.r, (T*)V.rt,
                                                          pre ? (const T*)M : nullptr, (T*)V.invM, P, sa);
        }
        KC_LAUNCH_CHECK("solver init");
        if (is_cg)
            rc = drive(o, key, P.st, [&](int m, cudaStream_t ss) { launch_cg_iters<T>(A, (T*)x, V, P, m, ss); }, &h, s);
        else if (pre)
            rc = drive(o, key, P.st, [&](int m, cudaStream_t ss) { launch_bicg_iters<T, true>(A, (T*)x, V, P, m, ss); }, &h, s);
        else
            rc = drive(o, key, P.st, [&](int m, cudaStream_t ss) { launch_bicg_iters<T, false>(A, (T*)x, V, P, m, ss); }, &h, s);
    } else {
        using T = float;
        if (is_cg) {
            k_cg_init<T><<<pb, kPwThreads, 0, s>>>(A->n, (const T*)b, (T*)x, (T*)V.r, P, sa_cg);
        } else if (o->x0 == KC_X0_WARM) {
            if (pre) k_invdiag<T><<<pb, kPwThreads, 0, s>>>(A->n, (const T*)M, (T*)V.invM);
            k_bicg_init_warm<T><<<sg, kThreads, 0, s>>>(coef_of<T>(A), g, (const T*)b, (const T*)x, (T*)V.r,
                                                        (T*)V.rt, P, sa);
        } else {
            k_bicg_init_cold<T><<<pb, kPwThreads, 0, s>>>(A->n, (const T*)b, (T*)x, (T*)V.r, (T*)V.rt,
                                                          pre ? (const T*)M : nullptr, (T*)V.invM, P, sa);
        }
        KC_LAUNCH_CHECK("solver init");
        if (is_cg)
            rc = drive(o, key, P.st, [&](int m, cudaStream_t ss) { launch_cg_iters<T>(A, (T*)x, V, P, m, ss); }, &h, s);
        else if (pre)
            rc = drive(o, key, P.st, [&](int m, cudaStream_t ss) { launch_bicg_iters<T, true>(A, (T*)x, V, P, m, ss); }, &h, s);
        else
            rc = drive(o, key, P.st, [&](int m, cudaStream_t ss) { launch_bicg_iters<T, false>(A, (T*)x, V, P, m, ss); }, &h, s);
    }
    if (rc) return rc;
    if (info) {
        info->status = h.status;
        info->refinements = 0;
        info->iters = h.iter;
        info->rel_res = h.prev_rel;
        info->r0 = sqrt(h.r0Tr);
    }
    return h.status;
}

int kc_bicgstab(const kc_system* A, const void* b, void* x, const void* M, void* ws, size_t ws_bytes,
                const kc_solve_opts* opts, kc_solve_info* info, void* stream) {
    return bicg_impl(A, b, x, M, ws, ws_bytes, opts, info, stream, false);
}

int kc_cg(const kc_system* A, const void* b, void* x, void* ws, size_t ws_bytes, const kc_solve_opts* opts,
          kc_solve_info* info, void* stream) {
    return bicg_impl(A, b, x, nullptr, ws, ws_bytes, opts, info, stream, true);
}

// ---- mixed precision refinement ----------------------------------------------
struct RefineLayout {
    size_t off_state, off_partials, off_out, off_r32, off_d32, off_inner, total, inner_bytes;
    int ld;
};
static RefineLayout refine_layout(long long n, int S) {
    RefineLayout L{};
    dim3 g = stencil_grid(n, std::max(S, 1));
    int nb = (int)(g.x * g.y);
    L.ld = (int)align256((size_t)nb * 8) / 8;
    size_t off = 0;
    L.off_state = off;
    off = align256(off + sizeof(SolverState));
    L.off_partials = off;
    off = align256(off + (size_t)2 * L.ld * 8);
    L.off_out = off;
    off = align256(off + 4 * 8);
    L.off_r32 = off;
    off = align256(off + (size_t)n * 4);
    L.off_d32 = off;
    off = align256(off + (size_t)n * 4);
    L.off_inner = off;
    L.inner_bytes = bicg_layout(n, S, KC_F32).total;
    off = align256(off + L.inner_bytes);
    L.total = off;
    return L;
}

size_t kc_refined_ws_bytes(long long n, int stride) {
    if (n < 1 || stride < 1) return 0;
    return refine_layout(n, stride).total;
}

int kc_bicgstab_refined(const kc_system* A64, const kc_system* A32, const double* b, double* x, void* ws,
                        size_t ws_bytes, const kc_solve_opts* o, double eps_inner, int max_refine,
                        kc_solve_info* info, void* stream) {
    int rc = check_system(A64);
    if (rc) return rc;
    rc = check_system(A32);
    if (rc) return rc;
    if (A64->dtype != KC_F64 || A32->dtype != KC_F32 || A64->n != A32->n || A64->stride != A32->stride)
        return set_error("kc_bicgstab_refined: need matching FP64 and FP32 systems"), KC_ERR_ARG;
    if (!b || !x || !o) return set_error("kc_bicgstab_refined: null argument"), KC_ERR_ARG;
    RefineLayout L = refine_layout(A64->n, A64->stride);
    if (!ws || ws_bytes < L.total)
        return set_error("kc_bicgstab_refined: workspace %zu < %zu", ws_bytes, L.total), KC_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    char* base = (char*)ws;
    BicgPtrs P{(SolverState*)(base + L.off_state), (double*)(base + L.off_partials), L.ld};
    double* out2 = (double*)(base + L.off_out);
    float* r32 = (float*)(base + L.off_r32);
    float* d32 = (float*)(base + L.off_d32);
    const long long n = A64->n;
    Geo g{n, A64->stride};
    dim3 sg = stencil_grid(n, A64->stride);
    int pb = pw_blocks(n);
    KC_CUDA(cudaMemsetAsync(P.st, 0, sizeof(SolverState), s));
    k_zero_f64<<<pb, kPwThreads, 0, s>>>(n, x);
    kc_solve_opts io = *o;
    io.eps = eps_inner;
    io.x0 = KC_X0_ZERO;
    io.precond = KC_PRECOND_NONE;
    io.rel_to = KC_REL_R0;
    io.history = nullptr;
    io.history_len = 0;
    long long total = 0;
    int status = KC_MAXITER, sweeps = 0;
    double rel = 1.0, bb = 0.0;
    for (int it = 0; it <= max_refine; ++it) {
        k_refine_resid<<<sg, kThreads, 0, s>>>(coef_of<double>(A64), g, b, x, r32, P, out2);
        KC_LAUNCH_CHECK("k_refine_resid");
        double h2[2];
        KC_CUDA(cudaMemcpyAsync(h2, out2, sizeof(h2), cudaMemcpyDeviceToHost, s));
        KC_CUDA(cudaStreamSynchronize(s));
        bb = h2[1];
        rel = bb > 0 ? sqrt(h2[0] / bb) : 0.0;
        if (bb == 0.0 || rel < o->eps) {
            status = KC_OK;
            break;
        }
        if (!isfinite(rel)) {
            status = KC_NONFINITE;
            break;
        }
        if (it == max_refine || total >= o->max_iter) break;
        io.max_iter = o->max_iter - total;
        kc_solve_info ii{};
        int r2 = kc_bicgstab(A32, r32, d32, nullptr, base + L.off_inner, L.inner_bytes, &io, &ii, stream);
        if (r2 < 0) return r2;
        total += ii.iters;
        ++sweeps;
        k_add_f32_to_f64<<<pb, kPwThreads, 0, s>>>(n, d32, x);
        KC_LAUNCH_CHECK("k_add_f32_to_f64");
        if (r2 == KC_NONFINITE) {
            status = KC_NONFINITE;
            break;
        }
    }
    if (info) {
        info->status = status;
        info->refinements = sweeps;
        info->iters = total;
        info->rel_res = rel;
        info->r0 = sqrt(bb);
    }
    return status;
}

}  // extern "C"
