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
// k +- 1 and k +- S.  A stencil block (256 threads) owns a tile of kTI = 32
// rows x kTJ = 32 consecutive columns of the [rows][S] view.  It evaluates the
// stencil operand (e.g. p = r + beta (p - omega v), times M^-1) once for every
// point of the tile plus a one-point halo into shared memory -- owned points
// also store their side outputs -- then each thread applies the stencil to
// four cells from shared memory.  All global loads of a phase are issued
// before any is consumed (the loops are fully unrolled), warp loads are 32
// consecutive elements, read-only streams use the read-only path and every
// pointer is restrict-qualified.  Halo points use flat index arithmetic, so
// the k +- 1 neighbours across a row end follow the reference's 1-D gather.
//
// One BiCGSTAB iteration is three launches (27 words of traffic per cell):
//   A  p = r + beta (p - omega v) [x M^-1]  ->  v = A p^,   partial (r~, v)
//   B  s = r - alpha v [x M^-1]             ->  t = A s^,   partials (t, s), (t, t)
//   C  x += alpha p^ + omega s^,  r = s - omega t,          partials (r, r~), (r, r)
// The last block of each launch reduces the partials in a fixed order and
// advances the scalar recurrence on the device, so the host never waits on a
// dot product; it polls a "done" word once per chunk of iterations.
//
// Inner products: in FP64 mode every product and sum is FP64.  In FP32 mode
// each product of two floats is formed exactly as a (hi, lo) float pair
// (fmaf) and summed -- per thread, across the warp and across the block -- in
// double-float arithmetic (Knuth TwoSum, ~48-bit significand); each block's
// partial is then carried in FP64 and the partials are summed in FP64.
// GB300 issues FP64 at 1/60 of its FP32 rate (1.19 vs 72 TFLOP/s measured),
// so FP64 work per cell would make the FP32 solver compute bound.
#include "kc_common.cuh"
#include "kc_mg.h"
#include <algorithm>
#include <atomic>
#include <mutex>
#include <map>
#include <memory>
#include <tuple>
#include <initializer_list>
#include <cstring>
#include <cmath>

namespace kc {

constexpr int kTJ = 32;            // tile columns (one per lane)
constexpr int kTI = 32;            // tile rows
constexpr int kThreads = 256;      // 8 warps
constexpr int kCPT = kTI * kTJ / kThreads;            // cells per thread (4)
constexpr int kPts = (kTI + 2) * (kTJ + 2);           // operand points incl. halo
constexpr int kPtIters = (kPts + kThreads - 1) / kThreads;
constexpr int kPwThreads = 256;    // pointwise kernels
constexpr int kPwPer = 4;          // elements per thread per round
constexpr int kPwMaxBlocks = 4096;

struct SolverState {
    double rho, rho_1, alpha, omega, beta;
    double r0Tr, rTr, den, eps, old;
    double prev_rel, lim;
    float alpha_f, omega_f, beta_f, pad_f;
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
    const T* __restrict__ c;
    long long cs, es;
    int lap;   // KC_FORM_LAPLACIAN: component 0 holds the row sum
    __device__ __forceinline__ T at(int comp, int k) const { return __ldg(c + comp * cs + (long long)k * es); }
};

struct Geo {
    int n, S;
};

static inline dim3 stencil_grid(long long n, int S) {
    long long rows = (n + S - 1) / S;
    long long gx = (S + kTJ - 1) / kTJ;
    long long gy = (rows + kTI - 1) / kTI;
    return dim3((unsigned)gx, (unsigned)gy);
}
static inline bool stencil_grid_ok(long long n, int S) {
    if (S < 1 || n < 1 || n > (1ll << 31) - 4ll * S - 64) return false;
    dim3 g = stencil_grid(n, S);
    return g.y <= 65535u && (long long)g.x * g.y <= (1ll << 30);
}
static inline int pw_blocks(long long n) {
    long long b = (n + kPwThreads * kPwPer - 1) / (kPwThreads * kPwPer);
    return (int)std::max<long long>(1, std::min<long long>(b, kPwMaxBlocks));
}

template <typename T>
__device__ __forceinline__ T fmaT(T a, T b, T c) { return fma(a, b, c); }
template <>
__device__ __forceinline__ float fmaT<float>(float a, float b, float c) { return fmaf(a, b, c); }

// Loads of vectors that other blocks of the same (persistent) kernel wrote
// must bypass L1 (COH = true -> ld.global.cg); otherwise the read-only path.
template <bool COH, typename T>
__device__ __forceinline__ T ld(const T* p) {
    if constexpr (COH) return __ldcg(p);
    else return __ldg(p);
}

// scalars of the recurrence in the vector precision (float copies are written
// by the finalisers so FP32 kernels never convert)
template <typename T>
struct Scal;
template <>
struct Scal<double> {
    __device__ static double alpha(const SolverState* s) { return __ldcg(&s->alpha); }
    __device__ static double omega(const SolverState* s) { return __ldcg(&s->omega); }
    __device__ static double beta(const SolverState* s) { return __ldcg(&s->beta); }
};
template <>
struct Scal<float> {
    __device__ static float alpha(const SolverState* s) { return __ldcg(&s->alpha_f); }
    __device__ static float omega(const SolverState* s) { return __ldcg(&s->omega_f); }
    __device__ static float beta(const SolverState* s) { return __ldcg(&s->beta_f); }
};

// Thread 0 publishes the block's partials, fences, and takes a ticket; the
// last block to arrive gets true (no block ever waits on another).
__device__ __forceinline__ bool publish_and_arrive(unsigned* ticket, unsigned nb) {
    __shared__ bool last;
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(ticket, 1u) == nb - 1;
    }
    __syncthreads();
    if (last) __threadfence();
    return last;
}

// Block sums of NV accumulators into partials[q*ld + bid]; returns true in
// the last block, with the fixed-order totals in out[] (thread 0).
template <int NV>
__device__ __forceinline__ bool block_partials(const Acc<double> (&a)[NV], double* partials, int ld, int bid,
                                               int nb, unsigned* ticket, double (&out)[NV]) {
    double d[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) d[q] = a[q].s;
    block_sum<NV>(d);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) partials[q * ld + bid] = d[q];
    }
    if (!publish_and_arrive(ticket, nb)) return false;
    reduce_partials<NV>(partials, ld, nb, out);
    return true;
}

template <int NV>
__device__ __forceinline__ bool block_partials(const Acc<float> (&a)[NV], double* partials, int ld, int bid,
                                               int nb, unsigned* ticket, double (&out)[NV]) {
    __shared__ DF sh[NV][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        DF v = a[q].s;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            DF u{__shfl_down_sync(kFull, v.hi, o), __shfl_down_sync(kFull, v.lo, o)};
            v = df_add(v, u);
        }
        if (lane == 0) sh[q][w] = v;
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            DF v = lane < nw ? sh[q][lane] : DF{0.f, 0.f};
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                DF u{__shfl_down_sync(kFull, v.hi, o), __shfl_down_sync(kFull, v.lo, o)};
                v = df_add(v, u);
            }
            if (lane == 0) partials[q * ld + bid] = (double)v.hi + (double)v.lo;
        }
    }
    if (!publish_and_arrive(ticket, nb)) return false;
    reduce_partials<NV>(partials, ld, nb, out);
    return true;
}

// -----------------------------------------------------------------------------
// Tiled stencil.  Pol provides (all __device__):
//   T    pre(k)            operand before the diagonal scaling (loads)
//   T    scale(k, pre)     operand fed to the stencil (x M^-1 when preconditioned)
//   void own(k, pre)       side outputs of a point owned by this tile
//   void sink(k, y, pre_k, acc)   consumes y = (A operand)[k]
//   static constexpr bool kAux    whether sink needs pre_k
// -----------------------------------------------------------------------------
template <typename T, int NACC, class Pol>
__device__ __forceinline__ void stencil_tile_at(const Pol& pol, const Coef<T>& A, int n, int S, int i0, int j0,
                                                Acc<T> (&acc)[NACC]) {
    __shared__ T op[kTI + 2][kTJ + 2];
    __shared__ T aux[Pol::kAux ? kTI : 1][Pol::kAux ? kTJ : 1];
    // The coefficients of the owned points do not depend on the staged
    // operand: their loads are issued first, so they are in flight together
    // with the operand's and the tile waits on memory once.
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int j = j0 + tx;
    T c[kCPT][5];
    int kc[kCPT];
#pragma unroll
    for (int r = 0; r < kCPT; ++r) {
        const int a = ty + 8 * r;
        const long long kl = (long long)(i0 + a) * S + j;
        const bool ok = j < S && kl < n;
        kc[r] = ok ? (int)kl : -1;
#pragma unroll
        for (int q = 0; q < 5; ++q) c[r][q] = ok ? A.at(q, (int)kl) : T(0);
    }
    T pre[kPtIters];
    int kk[kPtIters];
#pragma unroll
    for (int q = 0; q < kPtIters; ++q) {
        const int e = threadIdx.x + q * kThreads;
        const int a = e / (kTJ + 2), b = e - a * (kTJ + 2);
        const long long kl = (long long)(i0 + a - 1) * S + (j0 + b - 1);
        const bool in = e < kPts && kl >= 0 && kl < n;
        kk[q] = in ? (int)kl : -1;
        pre[q] = in ? pol.pre((int)kl) : T(0);
    }
#pragma unroll
    for (int q = 0; q < kPtIters; ++q) {
        const int e = threadIdx.x + q * kThreads;
        if (e < kPts) {
            const int a = e / (kTJ + 2), b = e - a * (kTJ + 2);
            const int k = kk[q];
            T v = T(0);
            if (k >= 0) {
                v = pol.scale(k, pre[q]);
                if (a >= 1 && a <= kTI && b >= 1 && b <= kTJ && (j0 + b - 1) < S) {
                    pol.own(k, pre[q]);
                    if (Pol::kAux) aux[a - 1][b - 1] = pre[q];
                }
            }
            op[a][b] = v;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kCPT; ++r) {
        if (kc[r] >= 0) {
            const int a = ty + 8 * r;
            const T o = op[a + 1][tx + 1];
            T y = c[r][0] * o;
            if (A.lap) {
                y = fmaT<T>(c[r][1], op[a][tx + 1] - o, y);
                y = fmaT<T>(c[r][2], op[a + 2][tx + 1] - o, y);
                y = fmaT<T>(c[r][3], op[a + 1][tx + 2] - o, y);
                y = fmaT<T>(c[r][4], op[a + 1][tx] - o, y);
            } else {
                y = fmaT<T>(c[r][1], op[a][tx + 1], y);
                y = fmaT<T>(c[r][2], op[a + 2][tx + 1], y);
                y = fmaT<T>(c[r][3], op[a + 1][tx + 2], y);
                y = fmaT<T>(c[r][4], op[a + 1][tx], y);
            }
            pol.sink(kc[r], y, Pol::kAux ? aux[a][tx] : T(0), acc);
        }
    }
}

template <typename T, int NACC, class Pol>
__device__ __forceinline__ void stencil_tile(const Pol& pol, const Coef<T>& A, int n, int S,
                                             Acc<T> (&acc)[NACC]) {
    stencil_tile_at<T, NACC, Pol>(pol, A, n, S, blockIdx.y * kTI, blockIdx.x * kTJ, acc);
}

__device__ __forceinline__ int block_id() { return blockIdx.y * gridDim.x + blockIdx.x; }
__device__ __forceinline__ int block_count() { return gridDim.x * gridDim.y; }

// ---- plain SpMV ---------------------------------------------------------------
template <typename T>
struct PolSpmv {
    static constexpr bool kAux = false;
    const T* __restrict__ x;
    T* __restrict__ y;
    __device__ __forceinline__ T pre(int k) const { return __ldg(x + k); }
    __device__ __forceinline__ T scale(int, T p) const { return p; }
    __device__ __forceinline__ void own(int, T) const {}
    __device__ __forceinline__ void sink(int k, T v, T, Acc<T> (&)[1]) const { y[k] = v; }
};

template <typename T>
__global__ void __launch_bounds__(kThreads) k_spmv(Coef<T> A, Geo g, const T* __restrict__ x, T* __restrict__ y) {
    Acc<T> acc[1];
    PolSpmv<T> pol{x, y};
    stencil_tile<T, 1>(pol, A, g.n, g.S, acc);
}

// ---- flat vectorised stencil passes ----------------------------------------------------
// For SoA coefficient planes (es == 1) whose far stride S, plane stride cs and
// size n are multiples of V, with V-aligned pointers: each thread owns chunks of
// V consecutive cells and reads every coefficient, the operand and its +-S
// neighbours with one V-wide (8- or 16-byte) load each; the +-1 neighbours of a
// chunk are its own elements except one scalar load at each end.  No shared
// memory and no barrier, so a block's loads are all in flight at once and the
// launch runs at whatever occupancy the registers allow.  The arithmetic is
// that of stencil_tile_at operation for operation (same products, same FMA
// order), so the results are bitwise those of the tile kernels.
template <typename T, int V>
struct VecOf;
template <>
struct VecOf<double, 2> { using type = double2; };
template <>
struct VecOf<float, 4> { using type = float4; };
template <>
struct VecOf<float, 2> { using type = float2; };

template <typename T, int V>
__device__ __forceinline__ void ldg_vec(const T* __restrict__ p, T (&o)[V]) {
    using VT = typename VecOf<T, V>::type;
    const VT v = __ldg(reinterpret_cast<const VT*>(p));
    const T* e = reinterpret_cast<const T*>(&v);
#pragma unroll
    for (int i = 0; i < V; ++i) o[i] = e[i];
}
template <typename T, int V>
__device__ __forceinline__ void st_vec(T* __restrict__ p, const T (&o)[V]) {
    using VT = typename VecOf<T, V>::type;
    VT v;
    T* e = reinterpret_cast<T*>(&v);
#pragma unroll
    for (int i = 0; i < V; ++i) e[i] = o[i];
    *reinterpret_cast<VT*>(p) = v;
}

// y[k .. k+V) = (A x)[k .. k+V); reads outside [0, n) are 0
template <typename T, int V>
__device__ __forceinline__ void stencil_chunk(const Coef<T>& A, const T* __restrict__ x, int n, int S, int k,
                                              T (&y)[V]) {
    T c0[V], c1[V], c2[V], c3[V], c4[V], xc[V], xw[V], xe[V];
    ldg_vec<T, V>(A.c + k, c0);
    ldg_vec<T, V>(A.c + A.cs + k, c1);
    ldg_vec<T, V>(A.c + 2 * A.cs + k, c2);
    ldg_vec<T, V>(A.c + 3 * A.cs + k, c3);
    ldg_vec<T, V>(A.c + 4 * A.cs + k, c4);
    ldg_vec<T, V>(x + k, xc);
    if (k >= S) {
        ldg_vec<T, V>(x + k - S, xw);
    } else {
#pragma unroll
        for (int i = 0; i < V; ++i) xw[i] = T(0);
    }
    if (k + S < n) {
        ldg_vec<T, V>(x + k + S, xe);
    } else {
#pragma unroll
        for (int i = 0; i < V; ++i) xe[i] = T(0);
    }
    const T xl = k > 0 ? __ldg(x + k - 1) : T(0);
    const T xr = k + V < n ? __ldg(x + k + V) : T(0);
#pragma unroll
    for (int i = 0; i < V; ++i) {
        const T o = xc[i];
        const T xs = i > 0 ? xc[i - 1] : xl;
        const T xn = i < V - 1 ? xc[i + 1] : xr;
        T v = c0[i] * o;
        if (A.lap) {
            v = fmaT<T>(c1[i], xw[i] - o, v);
            v = fmaT<T>(c2[i], xe[i] - o, v);
            v = fmaT<T>(c3[i], xn - o, v);
            v = fmaT<T>(c4[i], xs - o, v);
        } else {
            v = fmaT<T>(c1[i], xw[i], v);
            v = fmaT<T>(c2[i], xe[i], v);
            v = fmaT<T>(c3[i], xn, v);
            v = fmaT<T>(c4[i], xs, v);
        }
        y[i] = v;
    }
}

template <typename T, int V>
__global__ void __launch_bounds__(kThreads) k_spmv_vec(Coef<T> A, int n, int S, const T* __restrict__ x,
                                                       T* __restrict__ y) {
    const int nc = n / V;
    for (int c = blockIdx.x * kThreads + threadIdx.x; c < nc; c += gridDim.x * kThreads) {
        T out[V];
        stencil_chunk<T, V>(A, x, n, S, c * V, out);
        st_vec<T, V>(y + c * V, out);
    }
}

// V for the flat vectorised passes on A with the given vector pointers (0: not applicable)
template <typename T>
static int vec_width(const kc_system* A, std::initializer_list<const void*> ptrs) {
    if (A->es != 1) return 0;
    for (int V : {int(16 / sizeof(T)), 2}) {
        const size_t bytes = V * sizeof(T);
        bool ok = A->stride % V == 0 && A->n % V == 0 && A->cs % V == 0 && ((uintptr_t)A->coef % bytes) == 0;
        for (const void* q : ptrs) ok = ok && ((uintptr_t)q % bytes) == 0;
        if (ok) return V;
    }
    return 0;
}

static int vec_blocks(long long chunks, int cap) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                       cudaSuccess)
            sms = 152;
    }
    const long long want = (chunks + kThreads - 1) / kThreads;
    return (int)std::max<long long>(1, std::min<long long>({want, (long long)sms * 8, (long long)cap}));
}

// Grid of a flat FP64 pass that also sums per thread and block (the refinement
// residual): about cpt chunks a thread.  Its block reduction costs each thread
// ten FP64 adds per summed value, a fixed price against the FP64 pipe that a
// thread handling only a few cells pays several times over.
static int red_blocks(long long chunks, int cpt, int cap) {
    const long long want = (chunks + (long long)kThreads * cpt - 1) / ((long long)kThreads * cpt);
    return (int)std::max<long long>(1, std::min<long long>({want, (long long)vec_blocks(chunks, cap)}));
}

// ---- dot ----------------------------------------------------------------------
struct DotWs {
    unsigned ticket[4];
    double pad[2];
    double partials[kPwMaxBlocks];
};

template <typename T>
__global__ void __launch_bounds__(kPwThreads) k_dot(long long n, const T* __restrict__ p, const T* __restrict__ q,
                                                    DotWs* ws, double* out) {
    double acc[1] = {0.0};
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x)
        acc[0] += (double)__ldg(p + k) * (double)__ldg(q + k);
    block_sum<1>(acc);
    if (threadIdx.x == 0) ws->partials[blockIdx.x] = acc[0];
    if (publish_and_arrive(&ws->ticket[0], gridDim.x)) {
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

__device__ __forceinline__ void set_alpha(SolverState* st, double a) {
    st->alpha = a;
    st->alpha_f = (float)a;
    if (!isfinite(a) || fabs(a) > st->lim) {
        st->status = KC_NONFINITE;
        st->done = 1;
    }
}
__device__ __forceinline__ void set_omega(SolverState* st, double w) {
    st->omega = w;
    st->omega_f = (float)w;
    if (!isfinite(w) || fabs(w) > st->lim) {
        st->status = KC_NONFINITE;
        st->done = 1;
    }
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
        const double beta = (st->rho / st->rho_1) * (st->alpha / st->omega);
        st->beta = beta;
        st->beta_f = (float)beta;
        if (!isfinite(beta) || fabs(beta) > st->lim) {
            st->status = KC_NONFINITE;
            st->done = 1;
        }
    }
}

struct StartArgs {
    double eps;
    long long max_iter;
    int omega_break, rel_to;
    double* hist;
    long long hist_len;
    double lim;   // largest scalar the vector precision can carry
};

__device__ void bicg_start(SolverState* st, double r0Tr, double bb, const StartArgs& a) {
    const double eps = a.eps;
    const long long max_iter = a.max_iter;
    st->hist = a.hist;
    st->hist_len = a.hist_len;
    st->lim = a.lim;
    record_history(st, 0, r0Tr);
    st->iter = 0;
    st->max_iter = max_iter;
    st->eps = eps;
    st->omega_break = a.omega_break;
    st->rel_to = a.rel_to;
    st->r0Tr = r0Tr;
    st->rTr = r0Tr;
    st->den = a.rel_to == KC_REL_B ? bb : r0Tr;
    st->rho = r0Tr;  // r~ = r0, so rho_0 = (r0, r0)
    st->rho_1 = st->alpha = st->omega = 1.0;
    st->alpha_f = st->omega_f = 1.f;
    st->beta = 0.0;
    st->beta_f = 0.f;
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
    } else if (a.rel_to == KC_REL_B && st->prev_rel < eps) {
        st->status = KC_OK;
        st->done = 1;
    } else if (max_iter <= 0) {
        st->status = KC_MAXITER;
        st->done = 1;
    }
}

// Pointwise driver: each block handles rounds of kPwThreads*kPwPer elements,
// every round issuing all its loads before computing.
#define KC_PW_LOOP(n, ...)                                                                  \
    for (int base_ = blockIdx.x * (kPwThreads * kPwPer); base_ < (n);                      \
         base_ += gridDim.x * (kPwThreads * kPwPer)) {                                      \
        _Pragma("unroll") for (int u_ = 0; u_ < kPwPer; ++u_) {                             \
            const int k = base_ + threadIdx.x + u_ * kPwThreads;                            \
            if (k < (n)) { __VA_ARGS__ }                                                           \
        }                                                                                   \
    }

// cold start: r = r~ = b, x = 0; optional invM = 1/M
template <typename T>
__global__ void __launch_bounds__(kPwThreads)
    k_bicg_init_cold(int n, const T* __restrict__ b, T* __restrict__ x, T* __restrict__ r, T* __restrict__ rt,
                     const T* __restrict__ M, T* __restrict__ invM, BicgPtrs P, StartArgs sa) {
    Acc<T> acc[1];
    KC_PW_LOOP(n, {
        const T bk = __ldg(b + k);
        r[k] = bk;
        rt[k] = bk;
        x[k] = T(0);
        if (M) invM[k] = T(1) / __ldg(M + k);
        acc[0].add(bk, bk);
    })
    double s[1];
    if (block_partials<1>(acc, P.partials, P.ld, blockIdx.x, gridDim.x, &P.st->ticket[0], s) && threadIdx.x == 0) {
        bicg_start(P.st, s[0], s[0], sa);
        P.st->ticket[0] = 0;
    }
}

template <typename T>
__global__ void __launch_bounds__(kPwThreads) k_invdiag(int n, const T* __restrict__ M, T* __restrict__ invM) {
    KC_PW_LOOP(n, { invM[k] = T(1) / __ldg(M + k); })
}

// warm start: r = r~ = b - A x
template <typename T>
struct PolWarm {
    static constexpr bool kAux = false;
    const T* __restrict__ x;
    const T* __restrict__ b;
    T* __restrict__ r;
    T* __restrict__ rt;
    __device__ __forceinline__ T pre(int k) const { return __ldg(x + k); }
    __device__ __forceinline__ T scale(int, T p) const { return p; }
    __device__ __forceinline__ void own(int, T) const {}
    __device__ __forceinline__ void sink(int k, T y, T, Acc<T> (&acc)[2]) const {
        const T bk = __ldg(b + k);
        const T rk = bk - y;
        r[k] = rk;
        rt[k] = rk;
        acc[0].add(rk, rk);
        acc[1].add(bk, bk);
    }
};

template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_bicg_init_warm(Coef<T> A, Geo g, const T* __restrict__ b, const T* __restrict__ x, T* __restrict__ r,
                     T* __restrict__ rt, BicgPtrs P, StartArgs sa) {
    Acc<T> acc[2];
    PolWarm<T> pol{x, b, r, rt};
    stencil_tile<T, 2>(pol, A, g.n, g.S, acc);
    double s[2];
    if (block_partials<2>(acc, P.partials, P.ld, block_id(), block_count(), &P.st->ticket[0], s) &&
        threadIdx.x == 0) {
        bicg_start(P.st, s[0], s[1], sa);
        P.st->ticket[0] = 0;
    }
}

// pass A: p = r + beta (p_old - omega v_old); v = A p^; partial (r~, v)
template <typename T, bool PRE, bool COH = false>
struct PolA {
    static constexpr bool kAux = false;
    const T* __restrict__ r;
    const T* __restrict__ p_old;
    const T* __restrict__ v_old;
    T* __restrict__ p_new;
    const T* __restrict__ invM;
    const T* __restrict__ rt;
    T* __restrict__ v;
    T beta, omega;
    bool first;
    __device__ __forceinline__ T pre(int k) const {
        const T rk = ld<COH>(r + k);
        if (first) return rk;
        const T d = fmaT<T>(-omega, ld<COH>(v_old + k), ld<COH>(p_old + k));
        return fmaT<T>(beta, d, rk);
    }
    __device__ __forceinline__ T scale(int k, T p) const { return PRE ? p * __ldg(invM + k) : p; }
    __device__ __forceinline__ void own(int k, T p) const { p_new[k] = p; }
    __device__ __forceinline__ void sink(int k, T y, T, Acc<T> (&acc)[1]) const {
        v[k] = y;
        acc[0].add(__ldg(rt + k), y);
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
    pol.p_old = (const T*)(cur ? V.p[1] : V.p[0]);
    pol.v_old = (const T*)(cur ? V.v[1] : V.v[0]);
    pol.p_new = (T*)(nxt ? V.p[1] : V.p[0]);
    pol.invM = (const T*)V.invM;
    pol.rt = (const T*)V.rt;
    pol.v = (T*)(nxt ? V.v[1] : V.v[0]);
    pol.beta = Scal<T>::beta(st);
    pol.omega = Scal<T>::omega(st);
    pol.first = it == 0;
    Acc<T> acc[1];
    stencil_tile<T, 1>(pol, A, g.n, g.S, acc);
    double s[1];
    if (block_partials<1>(acc, P.partials, P.ld, block_id(), block_count(), &st->ticket[0], s) &&
        threadIdx.x == 0) {
        set_alpha(st, st->rho / s[0]);
        st->ticket[0] = 0;
    }
}

// pass B: s = r - alpha v; t = A s^; partials (t, s), (t, t)
template <typename T, bool PRE, bool COH = false>
struct PolB {
    static constexpr bool kAux = true;
    const T* __restrict__ r;
    const T* __restrict__ v;
    const T* __restrict__ invM;
    T* __restrict__ t;
    T alpha;
    __device__ __forceinline__ T pre(int k) const { return fmaT<T>(-alpha, ld<COH>(v + k), ld<COH>(r + k)); }
    __device__ __forceinline__ T scale(int k, T s) const { return PRE ? s * __ldg(invM + k) : s; }
    __device__ __forceinline__ void own(int, T) const {}
    __device__ __forceinline__ void sink(int k, T y, T s, Acc<T> (&acc)[2]) const {
        t[k] = y;
        acc[0].add(y, s);
        acc[1].add(y, y);
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
    pol.v = (const T*)(nxt ? V.v[1] : V.v[0]);
    pol.invM = (const T*)V.invM;
    pol.t = (T*)V.t;
    pol.alpha = Scal<T>::alpha(st);
    Acc<T> acc[2];
    stencil_tile<T, 2>(pol, A, g.n, g.S, acc);
    double s[2];
    if (block_partials<2>(acc, P.partials, P.ld, block_id(), block_count(), &st->ticket[0], s) &&
        threadIdx.x == 0) {
        set_omega(st, s[0] / s[1]);
        st->ticket[0] = 0;
    }
}

// pass C: x += alpha p^ + omega s^; r = s - omega t; partials (r, r~), (r, r)
template <typename T, bool PRE>
__global__ void __launch_bounds__(kPwThreads) k_bicg_C(int n, T* __restrict__ x, BicgVecs V, BicgPtrs P) {
    SolverState* st = P.st;
    if (solver_done(st)) return;
    const long long it = __ldcg(&st->iter);
    const int nxt = (int)((it + 1) & 1);
    const T* __restrict__ p = (const T*)(nxt ? V.p[1] : V.p[0]);
    const T* __restrict__ v = (const T*)(nxt ? V.v[1] : V.v[0]);
    const T* __restrict__ t = (const T*)V.t;
    const T* __restrict__ rt = (const T*)V.rt;
    const T* __restrict__ invM = (const T*)V.invM;
    T* __restrict__ r = (T*)V.r;
    const T alpha = Scal<T>::alpha(st), omega = Scal<T>::omega(st);
    Acc<T> acc[2];
    KC_PW_LOOP(n, {
        const T rk = r[k];
        const T s = fmaT<T>(-alpha, __ldg(v + k), rk);
        T ph = __ldg(p + k), sh = s;
        if (PRE) {
            const T im = __ldg(invM + k);
            ph = ph * im;
            sh = sh * im;
        }
        x[k] = x[k] + fmaT<T>(alpha, ph, omega * sh);
        const T rn = fmaT<T>(-omega, __ldg(t + k), s);
        r[k] = rn;
        acc[0].add(rn, __ldg(rt + k));
        acc[1].add(rn, rn);
    })
    double s[2];
    if (block_partials<2>(acc, P.partials, P.ld, blockIdx.x, gridDim.x, &st->ticket[0], s) && threadIdx.x == 0) {
        bicg_finish_iteration(st, s[0], s[1]);
        st->ticket[0] = 0;
    }
}

// =============================================================================
// CG (cgsolver.py:83-114), two passes per iteration
//   1  p = r + beta p_old  ->  Ap = A p,  partial (p, Ap)
//   2  x += alpha p, r -= alpha Ap,       partial (r, r)
// =============================================================================
template <typename T>
__global__ void __launch_bounds__(kPwThreads)
    k_cg_init(int n, const T* __restrict__ b, T* __restrict__ x, T* __restrict__ r, BicgPtrs P, StartArgs sa) {
    Acc<T> acc[1];
    KC_PW_LOOP(n, {
        const T bk = __ldg(b + k);
        r[k] = bk;
        x[k] = T(0);
        acc[0].add(bk, bk);
    })
    double s[1];
    if (block_partials<1>(acc, P.partials, P.ld, blockIdx.x, gridDim.x, &P.st->ticket[0], s) && threadIdx.x == 0) {
        bicg_start(P.st, s[0], s[0], sa);
        P.st->ticket[0] = 0;
    }
}

template <typename T, bool COH = false>
struct PolCg1 {
    static constexpr bool kAux = true;
    const T* __restrict__ r;
    const T* __restrict__ p_old;
    T* __restrict__ p_new;
    T* __restrict__ Ap;
    T beta;
    bool first;
    __device__ __forceinline__ T pre(int k) const {
        return first ? ld<COH>(r + k) : fmaT<T>(beta, ld<COH>(p_old + k), ld<COH>(r + k));
    }
    __device__ __forceinline__ T scale(int, T p) const { return p; }
    __device__ __forceinline__ void own(int k, T p) const { p_new[k] = p; }
    __device__ __forceinline__ void sink(int k, T y, T p, Acc<T> (&acc)[1]) const {
        Ap[k] = y;
        acc[0].add(p, y);
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
    pol.p_old = (const T*)(cur ? V.p[1] : V.p[0]);
    pol.p_new = (T*)(nxt ? V.p[1] : V.p[0]);
    pol.Ap = (T*)V.v[0];
    pol.beta = Scal<T>::beta(st);
    pol.first = it == 0;
    Acc<T> acc[1];
    stencil_tile<T, 1>(pol, A, g.n, g.S, acc);
    double s[1];
    if (block_partials<1>(acc, P.partials, P.ld, block_id(), block_count(), &st->ticket[0], s) &&
        threadIdx.x == 0) {
        const double alpha = st->old / s[0];
        st->alpha = alpha;
        st->alpha_f = (float)alpha;
        if (!isfinite(alpha)) {
            st->status = KC_NONFINITE;
            st->done = 1;
        }
        st->ticket[0] = 0;
    }
}

template <typename T>
__global__ void __launch_bounds__(kPwThreads) k_cg_2(int n, T* __restrict__ x, BicgVecs V, BicgPtrs P) {
    SolverState* st = P.st;
    if (solver_done(st)) return;
    const long long it = __ldcg(&st->iter);
    const int nxt = (int)((it + 1) & 1);
    const T* __restrict__ p = (const T*)(nxt ? V.p[1] : V.p[0]);
    const T* __restrict__ Ap = (const T*)V.v[0];
    T* __restrict__ r = (T*)V.r;
    const T alpha = Scal<T>::alpha(st);
    Acc<T> acc[1];
    KC_PW_LOOP(n, {
        x[k] = fmaT<T>(alpha, __ldg(p + k), x[k]);
        const T rn = fmaT<T>(-alpha, __ldg(Ap + k), r[k]);
        r[k] = rn;
        acc[0].add(rn, rn);
    })
    double s[1];
    if (block_partials<1>(acc, P.partials, P.ld, blockIdx.x, gridDim.x, &st->ticket[0], s) && threadIdx.x == 0) {
        const double nw = s[0];
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
            st->beta_f = (float)st->beta;
            st->old = nw;
        }
        st->ticket[0] = 0;
    }
}

// =============================================================================
// Mixed precision refinement helpers
// =============================================================================
// r = b - A x in FP64, its FP32 copy, ||r||^2 and (with_b) ||b||^2: b does not
// change across the sweeps of one refinement, so only the first sums it.
struct PolResid {
    static constexpr bool kAux = false;
    const double* __restrict__ x;
    const double* __restrict__ b;
    float* __restrict__ r32;
    int with_b;
    __device__ __forceinline__ double pre(int k) const { return __ldg(x + k); }
    __device__ __forceinline__ double scale(int, double p) const { return p; }
    __device__ __forceinline__ void own(int, double) const {}
    __device__ __forceinline__ void sink(int k, double y, double, Acc<double> (&acc)[2]) const {
        const double bk = __ldg(b + k);
        const double rk = bk - y;
        r32[k] = f64_to_f32(rk);
        acc[0].add(rk, rk);
        if (with_b) acc[1].add(bk, bk);
    }
};

// A block walks the tiles t = blockIdx.x, + gridDim.x, ... (tiles_x per tile
// row): several tiles a block, so that the block reduction's FP64 adds are
// paid once per several tiles' cells.
__global__ void __launch_bounds__(kThreads)
    k_refine_resid(Coef<double> A, Geo g, int tiles_x, int ntiles, const double* __restrict__ b,
                   const double* __restrict__ x, float* __restrict__ r32, BicgPtrs P, double* out2, int with_b) {
    Acc<double> acc[2];
    PolResid pol{x, b, r32, with_b};
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        stencil_tile_at<double, 2>(pol, A, g.n, g.S, (t / tiles_x) * kTI, (t % tiles_x) * kTJ, acc);
        __syncthreads();   // the next tile restages the shared operand
    }
    double s[2];
    if (block_partials<2>(acc, P.partials, P.ld, blockIdx.x, gridDim.x, &P.st->ticket[0], s) && threadIdx.x == 0) {
        out2[0] = s[0];
        out2[1] = s[1];
        P.st->ticket[0] = 0;
    }
}

// The same pass in the flat vectorised form (SoA FP64 planes; see stencil_chunk):
// per chunk of V cells r = b - A x, its FP32 copy, ||r||^2 and ||b||^2.  The grid
// is capped at the partials the workspace holds (the tile grid's block count).
template <int V>
__global__ void __launch_bounds__(kThreads)
    k_refine_resid_vec(Coef<double> A, int n, int S, const double* __restrict__ b, const double* __restrict__ x,
                       float* __restrict__ r32, BicgPtrs P, double* out2, int with_b) {
    Acc<double> acc[2];
    const int nc = n / V;
    for (int c = blockIdx.x * kThreads + threadIdx.x; c < nc; c += gridDim.x * kThreads) {
        const int k = c * V;
        double y[V], bb[V];
        ldg_vec<double, V>(b + k, bb);
        stencil_chunk<double, V>(A, x, n, S, k, y);
        float rf[V];
#pragma unroll
        for (int i = 0; i < V; ++i) {
            const double rk = bb[i] - y[i];
            rf[i] = f64_to_f32(rk);
            acc[0].add(rk, rk);
            if (with_b) acc[1].add(bb[i], bb[i]);
        }
        if constexpr (V == 2) {
            *reinterpret_cast<float2*>(r32 + k) = make_float2(rf[0], rf[1]);
        } else {
#pragma unroll
            for (int i = 0; i < V; ++i) r32[k + i] = rf[i];
        }
    }
    double s[2];
    if (block_partials<2>(acc, P.partials, P.ld, blockIdx.x, gridDim.x, &P.st->ticket[0], s) && threadIdx.x == 0) {
        out2[0] = s[0];
        out2[1] = s[1];
        P.st->ticket[0] = 0;
    }
}

// x += d, applied only when every entry of d is finite (flag[0] == 0; set by
// k_flag_nonfinite), so a correction from a broken-down FP32 sweep is dropped.
__global__ void __launch_bounds__(kPwThreads)
    k_flag_nonfinite(int n, const float* __restrict__ d, int* __restrict__ flag) {
    int bad = 0;
    KC_PW_LOOP(n, { bad |= !isfinite(__ldg(d + k)); })
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

__global__ void __launch_bounds__(kPwThreads)
    k_flag_nonfinite_f64(int n, const double* __restrict__ d, int* __restrict__ flag) {
    int bad = 0;
    KC_PW_LOOP(n, { bad |= !isfinite(__ldg(d + k)); })
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

__global__ void __launch_bounds__(kPwThreads)
    k_add_f64(int n, const double* __restrict__ d, double* __restrict__ x, const int* __restrict__ flag) {
    if (__ldcg(flag)) return;
    KC_PW_LOOP(n, { x[k] += __ldg(d + k); })
}

__global__ void __launch_bounds__(kPwThreads) k_sub_f64(int n, const double* __restrict__ d, double* __restrict__ x) {
    KC_PW_LOOP(n, { x[k] -= __ldg(d + k); })
}

__global__ void __launch_bounds__(kPwThreads)
    k_add_f32_to_f64(int n, const float* __restrict__ d, double* __restrict__ x, const int* __restrict__ flag) {
    if (__ldcg(flag)) return;
    KC_PW_LOOP(n, { x[k] += (double)__ldg(d + k); })
}

__global__ void __launch_bounds__(kPwThreads)
    k_sub_f32_from_f64(int n, const float* __restrict__ d, double* __restrict__ x) {
    KC_PW_LOOP(n, { x[k] -= (double)__ldg(d + k); })
}

__global__ void k_zero_f64(int n, double* __restrict__ x) {
    KC_PW_LOOP(n, { x[k] = 0.0; })
}

// =============================================================================
// Persistent cooperative solvers: one launch runs the whole solve.
//
// Every block owns a fixed set of tiles for all passes of all iterations.
// After each pass the blocks meet at a grid barrier and every block sums the
// per-block partials itself (same data, same order -> identical scalars in
// every block), so no launch gap and no single-block tail sits between the
// passes.  The barrier spin is bounded: on timeout the block raises an error
// flag, every block leaves its loop, and the host reports KC_ERR_CUDA.
// Vectors written during the launch are read with ld.global.cg (L1 bypass).
// =============================================================================
// Block partial of NV accumulators -> partials[(slot+q)*ld + bid] (no ticket).
template <typename T, int NV>
__device__ __forceinline__ void store_block_partials(const Acc<T> (&a)[NV], double* partials, int ld, int slot,
                                                     int bid);
template <>
__device__ __forceinline__ void store_block_partials<double, 1>(const Acc<double> (&a)[1], double* partials, int ld,
                                                               int slot, int bid) {
    double d[1] = {a[0].s};
    block_sum<1>(d);
    if (threadIdx.x == 0) partials[slot * ld + bid] = d[0];
}
template <>
__device__ __forceinline__ void store_block_partials<double, 2>(const Acc<double> (&a)[2], double* partials, int ld,
                                                               int slot, int bid) {
    double d[2] = {a[0].s, a[1].s};
    block_sum<2>(d);
    if (threadIdx.x == 0) {
        partials[slot * ld + bid] = d[0];
        partials[(slot + 1) * ld + bid] = d[1];
    }
}
template <int NV>
__device__ __forceinline__ void store_block_partials_f(const Acc<float> (&a)[NV], double* partials, int ld, int slot,
                                                       int bid) {
    __shared__ DF sh[NV][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        DF v = a[q].s;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = df_add(v, DF{__shfl_down_sync(kFull, v.hi, o), __shfl_down_sync(kFull, v.lo, o)});
        if (lane == 0) sh[q][w] = v;
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            DF v = lane < nw ? sh[q][lane] : DF{0.f, 0.f};
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v = df_add(v, DF{__shfl_down_sync(kFull, v.hi, o), __shfl_down_sync(kFull, v.lo, o)});
            if (lane == 0) partials[(slot + q) * ld + bid] = (double)v.hi + (double)v.lo;
        }
    }
    __syncthreads();
}
template <>
__device__ __forceinline__ void store_block_partials<float, 1>(const Acc<float> (&a)[1], double* partials, int ld,
                                                              int slot, int bid) {
    store_block_partials_f<1>(a, partials, ld, slot, bid);
}
template <>
__device__ __forceinline__ void store_block_partials<float, 2>(const Acc<float> (&a)[2], double* partials, int ld,
                                                              int slot, int bid) {
    store_block_partials_f<2>(a, partials, ld, slot, bid);
}

// Fixed-order sum of NV partial vectors starting at slot; result in thread 0.
template <int NV>
__device__ __forceinline__ void sum_partials(const double* partials, int ld, int slot, int nb, double (&out)[NV]) {
    reduce_partials<NV>(partials + slot * ld, ld, nb, out);
}

// Visits the cells of tile (i0, j0) owned by this thread: rows ty + 8r.
template <class F>
__device__ __forceinline__ void for_tile_cells(int n, int S, int i0, int j0, F&& f) {
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int j = j0 + tx;
#pragma unroll
    for (int r = 0; r < kCPT; ++r) {
        const long long kl = (long long)(i0 + ty + 8 * r) * S + j;
        if (j < S && kl < n) f((int)kl);
    }
}

struct PersistGeo {
    int tiles_x, ntiles;
    unsigned spin_limit;   // polls a grid-barrier wait may take before it gives up
};

template <typename T, bool PRE>
__global__ void __launch_bounds__(kThreads)
    k_bicg_persist(Coef<T> A, Geo g, T* __restrict__ x, BicgVecs V, BicgPtrs P, GridBar* bar, PersistGeo pg) {
    SolverState* st = P.st;
    const int G = gridDim.x, bid = blockIdx.x;
    __shared__ double sc[8];      // rho, rho_1, alpha, omega, beta, den, eps, lim
    __shared__ long long siter, smax;
    __shared__ int sdone, sstatus, sobreak;
    __shared__ double q0, q1;     // scratch for parallel divisions
    if (threadIdx.x == 0) {
        sc[0] = st->rho; sc[1] = st->rho_1; sc[2] = st->alpha; sc[3] = st->omega; sc[4] = st->beta;
        sc[5] = st->den; sc[6] = st->eps; sc[7] = st->lim;
        siter = st->iter; smax = st->max_iter;
        sdone = st->done; sstatus = st->status; sobreak = st->omega_break;
    }
    __syncthreads();
    const T* __restrict__ rt = (const T*)V.rt;
    const T* __restrict__ invM = (const T*)V.invM;
    T* __restrict__ r = (T*)V.r;
    T* __restrict__ t = (T*)V.t;
    double rTr = st->rTr;
    while (!sdone) {
        const long long it = siter;
        const int cur = (int)(it & 1), nxt = cur ^ 1;
        T* p_new = (T*)(nxt ? V.p[1] : V.p[0]);
        T* v_new = (T*)(nxt ? V.v[1] : V.v[0]);
        // ---- pass A: p = r + beta (p - omega v); v = A p^; (r~, v)
        {
            PolA<T, PRE, true> pol;
            pol.r = r;
            pol.p_old = (const T*)(cur ? V.p[1] : V.p[0]);
            pol.v_old = (const T*)(cur ? V.v[1] : V.v[0]);
            pol.p_new = p_new;
            pol.invM = invM;
            pol.rt = rt;
            pol.v = v_new;
            pol.beta = (T)sc[4];
            pol.omega = (T)sc[3];
            pol.first = it == 0;
            Acc<T> acc[1];
            for (int tile = bid; tile < pg.ntiles; tile += G) {
                stencil_tile_at<T, 1>(pol, A, g.n, g.S, (tile / pg.tiles_x) * kTI, (tile % pg.tiles_x) * kTJ, acc);
                __syncthreads();
            }
            store_block_partials<T, 1>(acc, P.partials, P.ld, 0, bid);
        }
        if (!grid_sync(bar, G, pg.spin_limit)) return;
        {
            double s1[1];
            sum_partials<1>(P.partials, P.ld, 0, G, s1);
            if (threadIdx.x == 0) {
                const double alpha = sc[0] / s1[0];
                sc[2] = alpha;
                if (!isfinite(alpha) || fabs(alpha) > sc[7]) {
                    sdone = 1;
                    sstatus = KC_NONFINITE;
                }
            }
            __syncthreads();
            if (sdone) break;
        }
        // ---- pass B: s = r - alpha v; t = A s^; (t, s), (t, t)
        {
            PolB<T, PRE, true> pol;
            pol.r = r;
            pol.v = v_new;
            pol.invM = invM;
            pol.t = t;
            pol.alpha = (T)sc[2];
            Acc<T> acc[2];
            for (int tile = bid; tile < pg.ntiles; tile += G) {
                stencil_tile_at<T, 2>(pol, A, g.n, g.S, (tile / pg.tiles_x) * kTI, (tile % pg.tiles_x) * kTJ, acc);
                __syncthreads();
            }
            store_block_partials<T, 2>(acc, P.partials, P.ld, 1, bid);
        }
        if (!grid_sync(bar, G, pg.spin_limit)) return;
        {
            double s2[2];
            sum_partials<2>(P.partials, P.ld, 1, G, s2);
            if (threadIdx.x == 0) {
                const double omega = s2[0] / s2[1];
                sc[3] = omega;
                if (!isfinite(omega) || fabs(omega) > sc[7]) {
                    sdone = 1;
                    sstatus = KC_NONFINITE;
                }
            }
            __syncthreads();
            if (sdone) break;
        }
        // ---- pass C: x += alpha p^ + omega s^; r = s - omega t; (r, r~), (r, r)
        {
            const T alpha = (T)sc[2], omega = (T)sc[3];
            Acc<T> acc[2];
            for (int tile = bid; tile < pg.ntiles; tile += G) {
                for_tile_cells(g.n, g.S, (tile / pg.tiles_x) * kTI, (tile % pg.tiles_x) * kTJ, [&](int k) {
                    const T rk = __ldcg(r + k);
                    const T s = fmaT<T>(-alpha, __ldcg(v_new + k), rk);
                    T ph = __ldcg(p_new + k), sh = s;
                    if (PRE) {
                        const T im = __ldg(invM + k);
                        ph = ph * im;
                        sh = sh * im;
                    }
                    x[k] = __ldcg(x + k) + fmaT<T>(alpha, ph, omega * sh);
                    const T rn = fmaT<T>(-omega, __ldcg(t + k), s);
                    r[k] = rn;
                    acc[0].add(rn, __ldg(rt + k));
                    acc[1].add(rn, rn);
                });
            }
            store_block_partials<T, 2>(acc, P.partials, P.ld, 3, bid);
        }
        if (!grid_sync(bar, G, pg.spin_limit)) return;
        {
            double s3[2];
            sum_partials<2>(P.partials, P.ld, 3, G, s3);
            if (threadIdx.x == 0) {
                const double rho_new = s3[0];
                rTr = s3[1];
                siter = it + 1;
                q0 = rho_new;
                q1 = rTr;
            }
            __syncthreads();
            // beta = (rho_new / rho) * (alpha / omega): the two divisions run in two warps
            if (threadIdx.x == 0) q0 = q0 / sc[0];
            if (threadIdx.x == 32) sc[4] = sc[2] / sc[3];
            __syncthreads();
            if (threadIdx.x == 0) {
                const double rr = q1;
                const double den = sc[5], eps = sc[6];
                const long long itn = siter;
                if (rr < eps * eps * den) {
                    sdone = 1;
                    sstatus = KC_OK;
                } else if (!isfinite(rr)) {
                    sdone = 1;
                    sstatus = KC_NONFINITE;
                } else if (sobreak && sc[3] == 0.0) {
                    sdone = 1;
                    sstatus = KC_BREAKDOWN_OMEGA;
                } else if (itn >= smax) {
                    sdone = 1;
                    sstatus = KC_MAXITER;
                } else if (s3[0] == 0.0) {
                    sdone = 1;
                    sstatus = KC_BREAKDOWN_RHO;
                } else {
                    const double beta = q0 * sc[4];
                    sc[1] = sc[0];
                    sc[0] = s3[0];
                    sc[4] = beta;
                    if (!isfinite(beta) || fabs(beta) > sc[7]) {
                        sdone = 1;
                        sstatus = KC_NONFINITE;
                    }
                }
                if (bid == 0 && st->hist && itn < st->hist_len) st->hist[itn] = rr;  // squared; rooted after the solve
            }
            __syncthreads();
        }
    }
    if (bid == 0 && threadIdx.x == 0) {
        st->rho = sc[0];
        st->rho_1 = sc[1];
        st->alpha = sc[2];
        st->omega = sc[3];
        st->beta = sc[4];
        st->iter = siter;
        st->rTr = rTr;
        st->status = sstatus;
        st->done = 1;
        st->prev_rel = sc[5] > 0.0 ? sqrt(rTr / sc[5]) : 0.0;
    }
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_cg_persist(Coef<T> A, Geo g, T* __restrict__ x, BicgVecs V, BicgPtrs P, GridBar* bar, PersistGeo pg) {
    SolverState* st = P.st;
    const int G = gridDim.x, bid = blockIdx.x;
    __shared__ double sold, salpha, sbeta, sr0, seps;
    __shared__ long long siter, smax;
    __shared__ int sdone, sstatus;
    if (threadIdx.x == 0) {
        sold = st->old; salpha = st->alpha; sbeta = st->beta; sr0 = st->r0Tr; seps = st->eps;
        siter = st->iter; smax = st->max_iter; sdone = st->done; sstatus = st->status;
    }
    __syncthreads();
    T* __restrict__ r = (T*)V.r;
    T* __restrict__ Ap = (T*)V.v[0];
    double rTr = st->rTr;
    while (!sdone) {
        const long long it = siter;
        const int cur = (int)(it & 1), nxt = cur ^ 1;
        T* p_new = (T*)(nxt ? V.p[1] : V.p[0]);
        {
            PolCg1<T, true> pol;
            pol.r = r;
            pol.p_old = (const T*)(cur ? V.p[1] : V.p[0]);
            pol.p_new = p_new;
            pol.Ap = Ap;
            pol.beta = (T)sbeta;
            pol.first = it == 0;
            Acc<T> acc[1];
            for (int tile = bid; tile < pg.ntiles; tile += G) {
                stencil_tile_at<T, 1>(pol, A, g.n, g.S, (tile / pg.tiles_x) * kTI, (tile % pg.tiles_x) * kTJ, acc);
                __syncthreads();
            }
            store_block_partials<T, 1>(acc, P.partials, P.ld, 0, bid);
        }
        if (!grid_sync(bar, G, pg.spin_limit)) return;
        {
            double s1[1];
            sum_partials<1>(P.partials, P.ld, 0, G, s1);
            if (threadIdx.x == 0) {
                salpha = sold / s1[0];
                if (!isfinite(salpha)) {
                    sdone = 1;
                    sstatus = KC_NONFINITE;
                }
            }
            __syncthreads();
            if (sdone) break;
        }
        {
            const T alpha = (T)salpha;
            Acc<T> acc[1];
            for (int tile = bid; tile < pg.ntiles; tile += G) {
                for_tile_cells(g.n, g.S, (tile / pg.tiles_x) * kTI, (tile % pg.tiles_x) * kTJ, [&](int k) {
                    x[k] = fmaT<T>(alpha, __ldcg(p_new + k), __ldcg(x + k));
                    const T rn = fmaT<T>(-alpha, __ldcg(Ap + k), __ldcg(r + k));
                    r[k] = rn;
                    acc[0].add(rn, rn);
                });
            }
            store_block_partials<T, 1>(acc, P.partials, P.ld, 1, bid);
        }
        if (!grid_sync(bar, G, pg.spin_limit)) return;
        {
            double s2[1];
            sum_partials<1>(P.partials, P.ld, 1, G, s2);
            if (threadIdx.x == 0) {
                const double nw = s2[0];
                rTr = nw;
                siter = it + 1;
                if (nw < seps * seps * sr0) {
                    sdone = 1;
                    sstatus = KC_OK;
                } else if (!isfinite(nw)) {
                    sdone = 1;
                    sstatus = KC_NONFINITE;
                } else if (siter >= smax) {
                    sdone = 1;
                    sstatus = KC_MAXITER;
                } else {
                    sbeta = nw / sold;
                    sold = nw;
                }
                if (bid == 0 && st->hist && siter < st->hist_len) st->hist[siter] = nw;
            }
            __syncthreads();
        }
    }
    if (bid == 0 && threadIdx.x == 0) {
        st->old = sold;
        st->alpha = salpha;
        st->beta = sbeta;
        st->iter = siter;
        st->rTr = rTr;
        st->status = sstatus;
        st->done = 1;
        st->prev_rel = sr0 > 0.0 ? sqrt(rTr) / sqrt(sr0) : 0.0;
    }
}

// history[1..iters] hold squared norms after a persistent solve
__global__ void k_hist_sqrt(double* h, long long from, long long to) {
    for (long long k = from + blockIdx.x * blockDim.x + threadIdx.x; k < to; k += (long long)gridDim.x * blockDim.x)
        h[k] = sqrt(h[k]);
}

// =============================================================================
// Right-preconditioned BiCGSTAB (FP32 vectors, FP64 scalars) for a general
// preconditioner M applied between the passes (multigrid V-cycle):
//   P1  p = r + beta (p - omega v)           [pointwise]
//   M   p^ = M p
//   P2  v = A p^, partial (r~, v) -> alpha   [stencil]
//   P3  s = r - alpha v                      [pointwise]
//   M   s^ = M s
//   P4  t = A s^, partials (t, s), (t, t) -> omega
//   P5  x += alpha p^ + omega s^, r = s - omega t, (r, r~), (r, r)
// The iterate x is FP64: for the pressure correction of a long channel
// (cond ~ 1e7) an FP32 iterate carries rounding noise of relative size u32,
// and A applied to that noise is as large as the residual being solved for,
// so FP32 storage alone would stop the outer refinement.
// =============================================================================
struct PbVecs {
    float *r, *rt, *p, *ph, *v, *s, *sh, *t;
    double* x;
};

__global__ void __launch_bounds__(kPwThreads) k_pb_p(int n, PbVecs V, BicgPtrs P) {
    SolverState* st = P.st;
    if (solver_done(st)) return;
    const bool first = __ldcg(&st->iter) == 0;
    const float beta = __ldcg(&st->beta_f), omega = __ldcg(&st->omega_f);
    KC_PW_LOOP(n, {
        const float rk = V.r[k];
        V.p[k] = first ? rk : fmaf(beta, fmaf(-omega, V.v[k], V.p[k]), rk);
    })
}

template <bool TWO>
struct PolPb {
    static constexpr bool kAux = false;
    const float* __restrict__ x;     // operand (p^ or s^)
    float* __restrict__ y;           // output (v or t)
    const float* __restrict__ rt;
    const float* __restrict__ s;
    __device__ __forceinline__ float pre(int k) const { return __ldg(x + k); }
    __device__ __forceinline__ float scale(int, float p) const { return p; }
    __device__ __forceinline__ void own(int, float) const {}
    __device__ __forceinline__ void sink(int k, float v, float, Acc<float> (&acc)[TWO ? 2 : 1]) const {
        y[k] = v;
        if (TWO) {
            acc[0].add(v, __ldg(s + k));
            acc[TWO ? 1 : 0].add(v, v);
        } else {
            acc[0].add(__ldg(rt + k), v);
        }
    }
};

__global__ void __launch_bounds__(kThreads) k_pb_Av(Coef<float> A, Geo g, PbVecs V, BicgPtrs P) {
    SolverState* st = P.st;
    if (solver_done(st)) return;
    PolPb<false> pol{V.ph, V.v, V.rt, nullptr};
    Acc<float> acc[1];
    stencil_tile<float, 1>(pol, A, g.n, g.S, acc);
    double s[1];
    if (block_partials<1>(acc, P.partials, P.ld, block_id(), block_count(), &st->ticket[0], s) &&
        threadIdx.x == 0) {
        set_alpha(st, st->rho / s[0]);
        st->ticket[0] = 0;
    }
}

__global__ void __launch_bounds__(kPwThreads) k_pb_s(int n, PbVecs V, BicgPtrs P) {
    SolverState* st = P.st;
    if (solver_done(st)) return;
    const float alpha = __ldcg(&st->alpha_f);
    KC_PW_LOOP(n, { V.s[k] = fmaf(-alpha, V.v[k], V.r[k]); })
}

__global__ void __launch_bounds__(kThreads) k_pb_At(Coef<float> A, Geo g, PbVecs V, BicgPtrs P) {
    SolverState* st = P.st;
    if (solver_done(st)) return;
    PolPb<true> pol{V.sh, V.t, nullptr, V.s};
    Acc<float> acc[2];
    stencil_tile<float, 2>(pol, A, g.n, g.S, acc);
    double s[2];
    if (block_partials<2>(acc, P.partials, P.ld, block_id(), block_count(), &st->ticket[0], s) &&
        threadIdx.x == 0) {
        set_omega(st, s[0] / s[1]);
        st->ticket[0] = 0;
    }
}

__global__ void __launch_bounds__(kPwThreads) k_pb_x(int n, PbVecs V, BicgPtrs P) {
    SolverState* st = P.st;
    if (solver_done(st)) return;
    const float alpha = __ldcg(&st->alpha_f), omega = __ldcg(&st->omega_f);
    const double alpha_d = __ldcg(&st->alpha), omega_d = __ldcg(&st->omega);
    Acc<float> acc[2];
    KC_PW_LOOP(n, {
        V.x[k] = fma(alpha_d, (double)V.ph[k], fma(omega_d, (double)V.sh[k], V.x[k]));
        const float rn = fmaf(-omega, V.t[k], V.s[k]);
        V.r[k] = rn;
        acc[0].add(rn, __ldg(V.rt + k));
        acc[1].add(rn, rn);
    })
    double s[2];
    if (block_partials<2>(acc, P.partials, P.ld, blockIdx.x, gridDim.x, &st->ticket[0], s) && threadIdx.x == 0) {
        bicg_finish_iteration(st, s[0], s[1]);
        st->ticket[0] = 0;
    }
}

// =============================================================================
// Preconditioned CG (FP32 vectors, FP64 iterate and scalars) for symmetric
// systems with a symmetric preconditioner M (the multigrid V-cycle, whose
// post-smoother mirrors its pre-smoother):
//   K1  p = z + beta p (formed in the stencil tile), q = A p, (p, q) -> alpha
//   K2  x += alpha p, r -= alpha q, (r, r) -> convergence
//   M   z = M r
//   K3  (r, z) -> beta
// One operator and one V-cycle per iteration, half of BiCGSTAB's.  The start
// is K0 (r = b, x = 0, (r, r)), M, K3.
// =============================================================================
struct PcVecs {
    float *r[2], *z, *p[2], *q;   // r: ping-pong pair in the fused level-0 path, r[0] otherwise
    double* x;
    float* s[2];                  // fused path: s = A p (ping-pong); q holds w = A z there
};

// called by thread 0 of the last block once (r, r) of the new residual is known
__device__ __forceinline__ void pc_finish_iteration(SolverState* st, double nw) {
    st->iter += 1;
    st->rTr = nw;
    record_history(st, st->iter, nw);
    const double rel = st->den > 0.0 ? sqrt(nw / st->den) : 0.0;
    st->prev_rel = rel;
    if (rel < st->eps) {
        st->status = KC_OK;
        st->done = 1;
    } else if (!isfinite(nw)) {
        st->status = KC_NONFINITE;
        st->done = 1;
    } else if (st->iter >= st->max_iter) {
        st->status = KC_MAXITER;
        st->done = 1;
    }
}

// called by thread 0 of the last block once (r, z) is known
__device__ __forceinline__ void pc_finish_rz(SolverState* st, double rz) {
    if (!(rz > 0.0)) {  // (r, M r) <= 0: M is not positive definite
        st->status = isfinite(rz) ? KC_BREAKDOWN_RHO : KC_NONFINITE;
        st->done = 1;
    } else {
        if (st->iter > 0) {
            const double beta = rz / st->old;
            st->beta = beta;
            st->beta_f = (float)beta;
        }
        st->old = rz;
    }
}

struct PolPc1 {
    static constexpr bool kAux = true;
    const float* __restrict__ z;
    const float* __restrict__ p_old;
    float* __restrict__ p_new;
    float* __restrict__ q;
    float beta;
    bool first;
    __device__ __forceinline__ float pre(int k) const {
        return first ? __ldg(z + k) : fmaf(beta, __ldg(p_old + k), __ldg(z + k));
    }
    __device__ __forceinline__ float scale(int, float p) const { return p; }
    __device__ __forceinline__ void own(int k, float p) const { p_new[k] = p; }
    __device__ __forceinline__ void sink(int k, float y, float p, Acc<float> (&acc)[1]) const {
        q[k] = y;
        acc[0].add(p, y);
    }
};

__global__ void __launch_bounds__(kThreads) k_pc_1(Coef<float> A, Geo g, PcVecs V, BicgPtrs P) {
    pdl_wait();
    SolverState* st = P.st;
    if (solver_done(st)) return;
    const long long it = __ldcg(&st->iter);
    const int cur = (int)(it & 1);
    PolPc1 pol{V.z, V.p[cur], V.p[cur ^ 1], V.q, __ldcg(&st->beta_f), it == 0};
    Acc<float> acc[1];
    stencil_tile<float, 1>(pol, A, g.n, g.S, acc);
    pdl_trigger();
    double s[1];
    if (block_partials<1>(acc, P.partials, P.ld, block_id(), block_count(), &st->ticket[0], s) &&
        threadIdx.x == 0) {
        if (!(s[0] > 0.0)) {  // (p, A p) <= 0: the preconditioned operator is not positive definite
            st->status = isfinite(s[0]) ? KC_BREAKDOWN_RHO : KC_NONFINITE;
            st->done = 1;
        } else {
            set_alpha(st, st->old / s[0]);
        }
        st->ticket[0] = 0;
    }
}

__global__ void __launch_bounds__(kPwThreads) k_pc_2(int n, PcVecs V, BicgPtrs P) {
    SolverState* st = P.st;
    if (solver_done(st)) return;
    const long long it = __ldcg(&st->iter);
    const float* __restrict__ p = V.p[(int)((it + 1) & 1)];
    const float alpha = __ldcg(&st->alpha_f);
    const double alpha_d = __ldcg(&st->alpha);
    Acc<float> acc[1];
    float* __restrict__ r = V.r[0];
    KC_PW_LOOP(n, {
        const float pk = __ldg(p + k);
        V.x[k] = fma(alpha_d, (double)pk, V.x[k]);
        const float rn = fmaf(-alpha, __ldg(V.q + k), r[k]);
        r[k] = rn;
        acc[0].add(rn, rn);
    })
    double s[1];
    if (block_partials<1>(acc, P.partials, P.ld, blockIdx.x, gridDim.x, &st->ticket[0], s) && threadIdx.x == 0) {
        pc_finish_iteration(st, s[0]);
        st->ticket[0] = 0;
    }
}

// (r, z) -> beta = (r, z) / (r, z)_old; at the start it only records (r0, z0)
__global__ void __launch_bounds__(kPwThreads) k_pc_3(int n, PcVecs V, BicgPtrs P) {
    SolverState* st = P.st;
    if (solver_done(st)) return;
    Acc<float> acc[1];
    KC_PW_LOOP(n, { acc[0].add(__ldg(V.r[0] + k), __ldg(V.z + k)); })
    double s[1];
    if (block_partials<1>(acc, P.partials, P.ld, blockIdx.x, gridDim.x, &st->ticket[0], s) && threadIdx.x == 0) {
        pc_finish_rz(st, s[0]);
        st->ticket[0] = 0;
    }
}

// ---- fused level 0: CG's pointwise passes inside the V-cycle's level-0 tiles ----
// DOWN_0 with update: b = r_new = r_old - alpha q is formed per cell (halo
// included) from the previous residual, owned cells store r_new and
// accumulate (r_new, r_new), and x += alpha p runs while the tile is being
// staged -- pass K2.  r alternates between two buffers so no block reads a
// residual another block rewrote.  Without update (the start) b = r_0.
// ---- fused level-0 passes of the single-reduction preconditioned CG ----------------
// CG in the form of Chronopoulos and Gear: with z = M r and w = A z both
// inner products of an iteration come out of one pass,
//   gamma = (r, z), delta = (w, z),  beta = gamma / gamma_old,
//   alpha = gamma / (delta - beta gamma / alpha_old),
//   p = z + beta p,  s = w + beta s  (s = A p by recurrence),
//   x += alpha p,  r -= alpha s,
// so no separate pass forms A p: UP_0 (with a 3-cell halo, so that z is
// final on the 1-ring) writes z and w = A z and sums both products; DOWN_0
// forms s and the new r over its staged region, updates p and x on its own
// cells and hands b = r to the V-cycle.  Two level-0 launches per iteration.
template <int TI, int TJ, int NT>
struct PcMidCG {   // p = z + beta p, x += alpha p on the owned TI x TJ cells of the tile at (i0, j0)
    double* __restrict__ x;
    float* __restrict__ p;
    const float* __restrict__ z;
    double alpha;
    float beta;
    int NX, NY;
    bool on, first;
    __device__ __forceinline__ void operator()(int i0, int j0) const {
        if (!on) return;
        constexpr int R = (TI * TJ + NT - 1) / NT;
        float zv[R], pv[R];
        double xv[R];
        int kk[R];
        // all loads first (the cells are distinct, so no store can feed a later load)
#pragma unroll
        for (int m = 0; m < R; ++m) {
            const int t = threadIdx.x + m * NT;
            const int a = t / TJ, b = t - a * TJ;
            const int i = i0 + a, j = j0 + b;
            kk[m] = (t < TI * TJ && i < NX && j < NY) ? i * NY + j : -1;
            zv[m] = kk[m] >= 0 ? __ldcg(z + kk[m]) : 0.f;
            pv[m] = (kk[m] >= 0 && !first) ? __ldcg(p + kk[m]) : 0.f;
            xv[m] = kk[m] >= 0 ? __ldcg(x + kk[m]) : 0.0;
        }
#pragma unroll
        for (int m = 0; m < R; ++m)
            if (kk[m] >= 0) {
                const float pn = first ? zv[m] : fmaf(beta, pv[m], zv[m]);
                p[kk[m]] = pn;
                x[kk[m]] = fma(alpha, (double)pn, xv[m]);
            }
    }
};
// right-hand side of DOWN_0: s = w + beta s_old (staged sq = w, ss = s_old), b = r - alpha s;
// an owned cell also stores its s
struct PcPreCG {
    float alpha, beta;
    bool first;
    float* __restrict__ s_out;
    __device__ __forceinline__ float operator()(const MgStage& S, int u, int k) const {
        const float sv = first ? S.sq[u] : fmaf(beta, S.ss[u], S.sq[u]);
        if (k >= 0) s_out[k] = sv;
        return fmaf(-alpha, sv, S.sb[u]);
    }
};
struct PcOwnR {
    using Sum = Acc<float>;
    float* __restrict__ r_out;
    bool on;
    __device__ __forceinline__ void operator()(int k, float rn, Sum& acc) const {
        if (!on) return;
        r_out[k] = rn;
        acc.add(rn, rn);
    }
};

// DOWN_0 staging over the 2-cell-halo region, in two halves: W and the
// coefficients (the setup's), and r (sb), w (sq), s_old (ss) (the iteration's).
// Pairs: the row length is even, so 8-byte copies move two cells (see
// mg_stage_coef_pairs).
template <int TI, int AJ, int RY>
__device__ __forceinline__ void pcc_down_issue_fixed(int i0, int j0, const MgLvl& L, bool pairs, MgStage S) {
    using T = MgTile<TI, AJ, RY>;
    if (pairs && L.es == 1) {
        constexpr int PJ = AJ / 2;
        for (int e = threadIdx.x; e < T::AI * PJ; e += T::NT) {
            const int a = e / PJ, b = 2 * (e - a * PJ);
            const int i = i0 + a - 2, j = j0 + b - 2;
            const bool in = i >= 0 && i < L.NX && j >= 0 && j < L.NY;
            cp_async8f(S.sw + a * T::AJ + b, L.winv + (in ? i * L.NY + j : 0), in);
        }
        mg_stage_coef_pairs<TI, T>(L, i0, j0, S.sc);
        return;
    }
    const int b = T::tx(), j = j0 + b - 2;
    const bool jin = j >= 0 && j < L.NY;
    for (int a = T::ty(); a < T::AI; a += T::RY) {
        const int i = i0 + a - 2;
        const bool in = jin && i >= 0 && i < L.NX;
        cp_async4(S.sw + a * T::AJ + b, L.winv + (in ? i * L.NY + j : 0), in);
    }
    mg_stage_coef<TI, T>(L, i0, j0, S.sc);
}
template <int TI, int AJ, int RY>
__device__ __forceinline__ void pcc_down_issue_vec(int i0, int j0, const MgLvl& L, const float* __restrict__ r,
                                                   const float* __restrict__ w, const float* __restrict__ s_old,
                                                   bool update, bool first, bool pairs, MgStage S) {
    using T = MgTile<TI, AJ, RY>;
    if (pairs) {
        constexpr int PJ = AJ / 2;
        for (int e = threadIdx.x; e < T::AI * PJ; e += T::NT) {
            const int a = e / PJ, b = 2 * (e - a * PJ);
            const int i = i0 + a - 2, j = j0 + b - 2;
            const bool in = i >= 0 && i < L.NX && j >= 0 && j < L.NY;
            const int k = in ? i * L.NY + j : 0;
            const int u = a * T::AJ + b;
            cp_async8f(S.sb + u, r + k, in);
            if (update) cp_async8f(S.sq + u, w + k, in);
            if (update && !first) cp_async8f(S.ss + u, s_old + k, in);
        }
        return;
    }
    const int b = T::tx(), j = j0 + b - 2;
    const bool jin = j >= 0 && j < L.NY;
    for (int a = T::ty(); a < T::AI; a += T::RY) {
        const int i = i0 + a - 2;
        const bool in = jin && i >= 0 && i < L.NX;
        const int k = in ? i * L.NY + j : 0;
        const int u = a * T::AJ + b;
        cp_async4(S.sb + u, r + k, in);
        if (update) cp_async4(S.sq + u, w + k, in);
        if (update && !first) cp_async4(S.ss + u, s_old + k, in);
    }
}

// The level-0 kernels walk the tiles of the grid with a two-stage pipeline:
// a block (two per SM) stages tile t + G while it computes tile t, so the
// copies of one tile overlap the arithmetic and barriers of the other.
struct PcfGeo {
    int tiles_x, ntiles;
};
__device__ __forceinline__ int pcf_i0(const PcfGeo& g, int t, int TI) { return (t / g.tiles_x) * TI; }
__device__ __forceinline__ int pcf_j0(const PcfGeo& g, int t, int TJ) { return (t % g.tiles_x) * TJ; }

// update = 0: the start of a sweep (b = r, no CG vector updates)
template <int TI, int AJ, int RY>
__global__ void __launch_bounds__(AJ * RY, 2) k_pcc_down0(MgLvl L, float* __restrict__ x0pre, float* __restrict__ b1,
                                                          int NX1, int NY1, PcVecs V, BicgPtrs P, int update, PcfGeo g) {
    constexpr int TJ = AJ - 4, NT = AJ * RY;
    using T = MgTile<TI, AJ, RY>;
    constexpr int SA = 9 * T::A;   // staged floats per stage: sb, sq, ss, sw, sc[5]
    extern __shared__ __align__(16) float dsm[];
    const bool up = update != 0;
    auto stage = [&](int sidx) {
        float* b = dsm + sidx * SA;
        return MgStage{b, b + T::A, b + 3 * T::A, b + 4 * T::A, dsm + 2 * SA, nullptr, b + 2 * T::A};
    };
    // 8-byte staging copies: even row length and tile width, 8-byte aligned planes
    const bool even = (L.NY % 2 == 0) && (TJ % 2 == 0);
    const bool pairs_c = even && (L.cs % 2 == 0) &&
                         ((reinterpret_cast<unsigned long long>(L.c) | reinterpret_cast<unsigned long long>(L.winv)) %
                          8 == 0);
    int t = blockIdx.x, sidx = 0;
    // inside the iterations (update) the launch before this one is the previous iteration's
    // UP_0 or none, and the setup that wrote W and the coefficients ran launches earlier: the
    // first tile stages them before the grid dependency wait
    if (up && t < g.ntiles) pcc_down_issue_fixed<TI, AJ, RY>(pcf_i0(g, t, TI), pcf_j0(g, t, TJ), L, pairs_c, stage(0));
    pdl_wait();
    SolverState* st = P.st;
    if (solver_done(st)) {
        cp_async_wait_all();
        return;
    }
    const long long it = __ldcg(&st->iter);
    const int cur = (int)(it & 1);
    const bool first = it == 0;
    const float* r = cur ? V.r[1] : V.r[0];   // (selected, not indexed: no local copy of V)
    const float* s_old = cur ? V.s[1] : V.s[0];
    float* s_new = cur ? V.s[0] : V.s[1];
    const float alpha = up ? __ldcg(&st->alpha_f) : 0.f, beta = up ? __ldcg(&st->beta_f) : 0.f;
    const PcMidCG<TI, TJ, NT> mid{V.x, V.p[0], V.z, __ldcg(&st->alpha), beta, L.NX, L.NY, up, first};
    const PcOwnR own{cur ? V.r[0] : V.r[1], up};
    const bool pairs_v = even && ((reinterpret_cast<unsigned long long>(r) | reinterpret_cast<unsigned long long>(V.q) |
                                   reinterpret_cast<unsigned long long>(s_old)) % 8 == 0);
    Acc<float> acc[1];
    if (t < g.ntiles) {
        if (!up) pcc_down_issue_fixed<TI, AJ, RY>(pcf_i0(g, t, TI), pcf_j0(g, t, TJ), L, pairs_c, stage(0));
        pcc_down_issue_vec<TI, AJ, RY>(pcf_i0(g, t, TI), pcf_j0(g, t, TJ), L, r, V.q, s_old, up, first, pairs_v,
                                       stage(0));
    }
    cp_async_commit();
    for (; t < g.ntiles; t += gridDim.x) {
        const int tn = t + gridDim.x;
        if (tn < g.ntiles) {
            pcc_down_issue_fixed<TI, AJ, RY>(pcf_i0(g, tn, TI), pcf_j0(g, tn, TJ), L, pairs_c, stage(sidx ^ 1));
            pcc_down_issue_vec<TI, AJ, RY>(pcf_i0(g, tn, TI), pcf_j0(g, tn, TJ), L, r, V.q, s_old, up, first, pairs_v,
                                           stage(sidx ^ 1));
        }
        cp_async_commit();
        const int i0 = pcf_i0(g, t, TI), j0 = pcf_j0(g, t, TJ);
        mid(i0, j0);
        cp_async_wait_group<1>();
        __syncthreads();
        if (up)
            mg_down_compute_pre<TI, AJ, RY>(i0, j0, L, PcPreCG{alpha, beta, first, s_new}, own, stage(sidx), x0pre, b1,
                                            NX1, NY1, acc[0]);
        else
            mg_down_compute_pre<TI, AJ, RY>(i0, j0, L, MgPreB{}, own, stage(sidx), x0pre, b1, NX1, NY1, acc[0]);
        __syncthreads();   // the stage is refilled next
        sidx ^= 1;
    }
    pdl_trigger();
    if (!up) return;
    double sres[1];
    if (block_partials<1>(acc, P.partials, P.ld, blockIdx.x, gridDim.x, &st->ticket[0], sres) && threadIdx.x == 0) {
        pc_finish_iteration(st, sres[0]);
        st->ticket[0] = 0;
    }
}

// called by thread 0 of the last block once gamma = (r, z) and delta = (w, z) are known
__device__ __forceinline__ void pcc_finish(SolverState* st, double gamma, double delta) {
    if (!(gamma > 0.0)) {   // (r, M r) <= 0: M is not positive definite
        st->status = isfinite(gamma) ? KC_BREAKDOWN_RHO : KC_NONFINITE;
        st->done = 1;
        return;
    }
    double beta = 0.0, den = delta;
    if (st->iter > 0) {
        beta = gamma / st->old;
        den = delta - beta * gamma / st->alpha;
    }
    if (!(den > 0.0)) {   // (p, A p) <= 0: the operator is not positive definite
        st->status = isfinite(den) ? KC_BREAKDOWN_RHO : KC_NONFINITE;
        st->done = 1;
        return;
    }
    st->beta = beta;
    st->beta_f = (float)beta;
    st->old = gamma;
    set_alpha(st, gamma / den);
}

template <int TI, int AJ, int RY>
__global__ void __launch_bounds__(AJ * RY, 2) k_pcc_up0(MgLvl L, const float* __restrict__ x0pre,
                                                        const float* __restrict__ final1, int NX1, int NY1, float alpha0,
                                                        PcVecs V, BicgPtrs P, PcfGeo g) {
    using T = MgTile3<TI, AJ, RY>;
    constexpr int TJ = T::TJ, SA = 8 * T::A + T::XC;
    extern __shared__ __align__(16) float dsm[];
    auto stage = [&](int sidx) {
        float* b = dsm + sidx * SA;
        return MgStage{b + T::A, nullptr, b + 2 * T::A, b + 3 * T::A, b, b + 8 * T::A, nullptr};
    };
    int t = blockIdx.x, sidx = 0;
    // the launch before this one is the cycle's level-1 UP (or its tail), which waits for its
    // own predecessor before it lets this grid start: the pre-smoothed x0pre (DOWN_0's), W and
    // the coefficients are final, and the first tile stages them before the wait
    if (t < g.ntiles) mg_up3_issue_fixed<TI, AJ, RY>(pcf_i0(g, t, TI), pcf_j0(g, t, TJ), L, x0pre, stage(0));
    pdl_wait();
    SolverState* st = P.st;
    if (solver_done(st)) {
        cp_async_wait_all();
        return;
    }
    const long long it = __ldcg(&st->iter);
    const float* r = (it & 1) ? V.r[1] : V.r[0];
    Acc<float> acc[2];
    if (t < g.ntiles)
        mg_up3_issue_rest<TI, AJ, RY>(pcf_i0(g, t, TI), pcf_j0(g, t, TJ), L, final1, NX1, NY1, r, stage(0));
    cp_async_commit();
    for (; t < g.ntiles; t += gridDim.x) {
        const int tn = t + gridDim.x;
        if (tn < g.ntiles)
            mg_up3_issue<TI, AJ, RY>(pcf_i0(g, tn, TI), pcf_j0(g, tn, TJ), L, x0pre, final1, NX1, NY1, r, stage(sidx ^ 1));
        cp_async_commit();
        cp_async_wait_group<1>();
        __syncthreads();
        mg_up3_compute<TI, AJ, RY>(pcf_i0(g, t, TI), pcf_j0(g, t, TJ), L, alpha0, stage(sidx), V.z, V.q, acc[0], acc[1]);
        __syncthreads();
        sidx ^= 1;
    }
    pdl_trigger();
    double sres[2];
    if (block_partials<2>(acc, P.partials, P.ld, blockIdx.x, gridDim.x, &st->ticket[0], sres) && threadIdx.x == 0) {
        pcc_finish(st, sres[0], sres[1]);
        st->ticket[0] = 0;
    }
}

// Launch shape of the pipelined level-0 kernels: as many blocks as are
// resident (two per SM), at most one per tile; dynamic shared memory for two
// stages (and DOWN's scratch x).
struct PcfLaunch {
    PcfGeo gd, gu;
    int blocks;
    size_t smem_down, smem_up;
};
static int pcf_launch(const MgLvl& L0, PcfLaunch* out) {
    using TD = MgTile<kMgTI0, kMgAJ0, kMgRY0>;
    using TU = MgTile3<kMgTI0, kMgAJ0, kMgRY0>;
    constexpr size_t down = (2 * 9 * TD::A + TD::A) * sizeof(float), up = 2 * (8 * TU::A + TU::XC) * sizeof(float);
    static std::mutex mu;
    static int sms[64] = {0}, per[64] = {0};
    int dev = 0;
    KC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_error("device index %d out of range", dev), KC_ERR_ARG;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!sms[dev]) {
            int n = 0, pd = 0, pu = 0;
            KC_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
            KC_CUDA(cudaFuncSetAttribute(k_pcc_down0<kMgTI0, kMgAJ0, kMgRY0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)down));
            KC_CUDA(cudaFuncSetAttribute(k_pcc_up0<kMgTI0, kMgAJ0, kMgRY0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)up));
            KC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pd, k_pcc_down0<kMgTI0, kMgAJ0, kMgRY0>, kMgNT0, down));
            KC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pu, k_pcc_up0<kMgTI0, kMgAJ0, kMgRY0>, kMgNT0, up));
            per[dev] = std::max(1, std::min(pd, pu));
            sms[dev] = n;
        }
    }
    const dim3 td = mg_tile_grid(L0.NX, L0.NY, kMgTI0, TD::TJ), tu = mg_tile_grid(L0.NX, L0.NY, kMgTI0, TU::TJ);
    out->gd = PcfGeo{(int)td.x, (int)(td.x * td.y)};
    out->gu = PcfGeo{(int)tu.x, (int)(tu.x * tu.y)};
    out->blocks = std::max(1, std::min(std::min(out->gd.ntiles, out->gu.ntiles), per[dev] * sms[dev]));
    out->smem_down = down;
    out->smem_up = up;
    return KC_OK;
}

__global__ void k_copy_f64(int n, const double* __restrict__ a, double* __restrict__ b) {
    KC_PW_LOOP(n, { b[k] = a[k]; })
}

// =============================================================================
// Host side
// =============================================================================
static inline size_t esize(int dtype) { return dtype == KC_F64 ? 8 : 4; }

struct BicgLayout {
    size_t off_state, off_bar, off_partials, off_vec[8], total;
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
    L.off_bar = off;
    off = align256(off + sizeof(GridBar));
    L.off_partials = off;
    off = align256(off + (size_t)5 * L.ld * sizeof(double));
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
    if (A->form != KC_FORM_STANDARD && A->form != KC_FORM_LAPLACIAN)
        return set_error("kc_system: unknown coefficient form %d", A->form), KC_ERR_ARG;
    return KC_OK;
}

template <typename T>
static Coef<T> coef_of(const kc_system* A) {
    return Coef<T>{(const T*)A->coef, A->cs, A->es, A->form == KC_FORM_LAPLACIAN ? 1 : 0};
}

// r = b - A x and its sums: the flat vectorised pass when A's layout allows it,
// else the tile pass; both use at most the tile grid's block count of partials
static void launch_refine_resid(const kc_system* A64, Geo g, dim3 sg, const double* b, const double* x, float* r32,
                                BicgPtrs P, double* out2, bool with_b, cudaStream_t s) {
    if (vec_width<double>(A64, {b, x}) == 2 && ((uintptr_t)r32 % 8) == 0)
        k_refine_resid_vec<2><<<red_blocks(A64->n / 2, 8, (int)(sg.x * sg.y)), kThreads, 0, s>>>(
            coef_of<double>(A64), (int)A64->n, A64->stride, b, x, r32, P, out2, with_b ? 1 : 0);
    else {
        const int ntiles = (int)(sg.x * sg.y), nb = std::max(1, (ntiles + 3) / 4);   // four tiles a block
        k_refine_resid<<<nb, kThreads, 0, s>>>(coef_of<double>(A64), g, (int)sg.x, ntiles, b, x, r32, P, out2,
                                               with_b ? 1 : 0);
    }
}

struct HostState {
    int status, done;
    long long iter;
    double rTr, den, r0Tr, prev_rel;
};

static int read_state(const SolverState* st, HostState* h, cudaStream_t s) {
    const void* hp = readback(st, sizeof(SolverState), s);
    if (!hp) return KC_ERR_CUDA;
    SolverState tmp;
    memcpy(&tmp, hp, sizeof(SolverState));
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
// A captured chunk bakes in every pointer and parameter its launches take, so
// the key holds all of them: buffers can be freed and their addresses handed
// out again for a system of another form, size or multigrid configuration.
struct GraphKey {
    const void* ws;
    const void* coef;
    const void* x;
    long long n;
    int stride, dtype, pre, chunk, kind;
    long long cs, es;
    int form = 0;
    unsigned long long ohash = 0;   // hash of the multigrid options (0: none)
    const void* b = nullptr;        // a right-hand side the captured launches read (0: none)
    const void* c64 = nullptr;      // the FP64 system and iterate of a captured refinement (0: none)
    const void* x64 = nullptr;
    bool operator<(const GraphKey& o) const {
        return std::tie(ws, coef, x, n, stride, dtype, pre, chunk, kind, cs, es, form, ohash, b, c64, x64) <
               std::tie(o.ws, o.coef, o.x, o.n, o.stride, o.dtype, o.pre, o.chunk, o.kind, o.cs, o.es, o.form,
                        o.ohash, o.b, o.c64, o.x64);
    }
};

// FNV-1a over the bytes of an options struct
static unsigned long long bytes_hash(const void* p, size_t n) {
    unsigned long long h = 1469598103934665603ull;
    const unsigned char* b = (const unsigned char*)p;
    for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
    return h | 1ull;
}
// Cached executable graphs are reference counted: a caller takes a reference
// under the lock and launches outside it, so an entry evicted by another
// thread in between is destroyed only when the last holder drops it (and
// cudaGraphExecDestroy of a graph still in flight frees it on completion).
// When the cache is full the least recently used entry alone is evicted.
struct GraphExec {
    cudaGraphExec_t ex = nullptr;
    explicit GraphExec(cudaGraphExec_t e) : ex(e) {}
    ~GraphExec() {
        if (ex) cudaGraphExecDestroy(ex);
    }
    GraphExec(const GraphExec&) = delete;
    GraphExec& operator=(const GraphExec&) = delete;
};
struct GraphEntry {
    std::shared_ptr<GraphExec> g;
    unsigned long long last_use;
};
static size_t g_graph_cap = 1024;   // entries; set by kc_graph_cache_limit
static std::mutex g_graph_mu;
static std::map<std::pair<int, GraphKey>, GraphEntry> g_graphs;
static unsigned long long g_graph_clock = 0;

static std::shared_ptr<GraphExec> graph_lookup(int dev, const GraphKey& gk) {
    std::lock_guard<std::mutex> lk(g_graph_mu);
    auto it = g_graphs.find({dev, gk});
    if (it == g_graphs.end()) return nullptr;
    it->second.last_use = ++g_graph_clock;
    return it->second.g;
}

static void graph_insert(int dev, const GraphKey& gk, std::shared_ptr<GraphExec> g) {
    std::lock_guard<std::mutex> lk(g_graph_mu);
    if (!g_graphs.count({dev, gk})) {
        while (!g_graphs.empty() && g_graphs.size() >= g_graph_cap) {
            auto lru = g_graphs.begin();
            for (auto it = g_graphs.begin(); it != g_graphs.end(); ++it)
                if (it->second.last_use < lru->second.last_use) lru = it;
            g_graphs.erase(lru);
        }
    }
    g_graphs[{dev, gk}] = GraphEntry{std::move(g), ++g_graph_clock};
}

}  // namespace kc

extern "C" {
size_t kc_graph_cache_size(void) {
    std::lock_guard<std::mutex> lk(kc::g_graph_mu);
    return kc::g_graphs.size();
}

size_t kc_graph_cache_limit(size_t cap) {
    std::lock_guard<std::mutex> lk(kc::g_graph_mu);
    const size_t old = kc::g_graph_cap;
    if (cap > 0) {
        kc::g_graph_cap = cap;
        while (kc::g_graphs.size() > cap) {
            auto lru = kc::g_graphs.begin();
            for (auto it = kc::g_graphs.begin(); it != kc::g_graphs.end(); ++it)
                if (it->second.last_use < lru->second.last_use) lru = it;
            kc::g_graphs.erase(lru);
        }
    }
    return old;
}
}  // extern "C"

namespace kc {

template <typename T, bool PRE>
static void launch_bicg_iters(const kc_system* A, T* x, const BicgVecs& V, const BicgPtrs& P, int m,
                              cudaStream_t s) {
    Geo g{(int)A->n, A->stride};
    dim3 sg = stencil_grid(A->n, A->stride);
    int pb = pw_blocks(A->n);
    Coef<T> C = coef_of<T>(A);
    for (int q = 0; q < m; ++q) {
        k_bicg_A<T, PRE><<<sg, kThreads, 0, s>>>(C, g, V, P);
        k_bicg_B<T, PRE><<<sg, kThreads, 0, s>>>(C, g, V, P);
        k_bicg_C<T, PRE><<<pb, kPwThreads, 0, s>>>((int)A->n, x, V, P);
    }
}

template <typename T>
static void launch_cg_iters(const kc_system* A, T* x, const BicgVecs& V, const BicgPtrs& P, int m,
                            cudaStream_t s) {
    Geo g{(int)A->n, A->stride};
    dim3 sg = stencil_grid(A->n, A->stride);
    int pb = pw_blocks(A->n);
    Coef<T> C = coef_of<T>(A);
    for (int q = 0; q < m; ++q) {
        k_cg_1<T><<<sg, kThreads, 0, s>>>(C, g, V, P);
        k_cg_2<T><<<pb, kPwThreads, 0, s>>>((int)A->n, x, V, P);
    }
}

// Runs chunks of iterations (directly or as a cached CUDA graph) until the
// device marks the solve done.  Launcher(m, stream) enqueues m iterations.
template <class Launcher>
static int drive(const kc_solve_opts* o, const GraphKey& key, const SolverState* st, Launcher&& launch,
                 HostState* h, cudaStream_t s, int kernels_per_iter) {
    int rc = read_state(st, h, s);
    if (rc) return rc;
    long long launched = 0;
    const long long cap = h->done ? 0 : std::max<long long>(o->max_iter, 0);
    int chunk = o->check_every > 0 ? o->check_every : 4;
    const bool fixed = o->check_every > 0;
    const int gchunk = 16;
    while (!h->done && launched < cap) {
        int m = (int)std::min<long long>(chunk, cap - launched);
        if (o->use_graph && (fixed ? m == chunk : m == gchunk)) {
            int dev = 0;
            KC_CUDA(cudaGetDevice(&dev));
            GraphKey gk = key;
            gk.chunk = m;
            std::shared_ptr<GraphExec> gx = graph_lookup(dev, gk);
            if (!gx) {
                cudaStream_t cap_s;
                KC_CUDA(cudaStreamCreateWithFlags(&cap_s, cudaStreamNonBlocking));
                cudaGraph_t graph;
                KC_CUDA(cudaStreamBeginCapture(cap_s, cudaStreamCaptureModeThreadLocal));
                launch(m, cap_s);
                cudaError_t e = cudaStreamEndCapture(cap_s, &graph);
                cudaStreamDestroy(cap_s);
                if (e != cudaSuccess) return cuda_status(e, "cudaStreamEndCapture");
                cudaGraphExec_t ex = nullptr;
                e = cudaGraphInstantiate(&ex, graph, 0);
                cudaGraphDestroy(graph);
                if (e != cudaSuccess) return cuda_status(e, "cudaGraphInstantiate");
                gx = std::make_shared<GraphExec>(ex);
                graph_insert(dev, gk, gx);
            }
            KC_CUDA(cudaGraphLaunch(gx->ex, s));
        } else {
            launch(m, s);
            KC_LAUNCH_CHECK_NC("solver iteration launch");
        }
        count_launches((long long)m * kernels_per_iter);
        launched += m;
        rc = read_state(st, h, s);
        if (rc) return rc;
        if (!fixed) chunk = std::min(chunk * 2, gchunk);
    }
    return KC_OK;
}

// ---- device-side loop over whole iterations (conditional WHILE graph node) --------------------
// One captured iteration runs inside a WHILE node whose condition the last
// kernel of the body sets from the solver state: the loop ends when the solve
// is done (converged, capped, broken down) or after `cap` iterations, without
// a host round trip or a launch past convergence.  The body-execution count
// lives in st->ticket[3] (zero at the start of every solve), so the loop is
// bounded by construction.
__global__ void k_while_cond(SolverState* st, unsigned cap, cudaGraphConditionalHandle h) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const unsigned c = ++st->ticket[3];
    cudaGraphSetConditional(h, (__ldcg(&st->done) == 0 && c < cap) ? 1u : 0u);
}

constexpr unsigned kWhileCap = 1024;    // iterations one launch of the loop may run
static std::atomic<int> g_while_ok{1};  // cleared when the driver refuses conditional nodes
static std::atomic<int> g_refloop_ok{1};   // cleared when the nested conditional graph is refused

// Runs the solve's iterations as one graph launch; returns 1 when it ran (state in h), 0 when the
// caller should use the chunked loop instead, < 0 on a CUDA error.
template <class Launcher>
static int drive_while(const GraphKey& key, SolverState* st, Launcher&& launch1, HostState* h, cudaStream_t s,
                       int kernels_per_iter) {
    if (!g_while_ok.load(std::memory_order_relaxed)) return 0;
    int dev = 0;
    KC_CUDA(cudaGetDevice(&dev));
    GraphKey gk = key;
    gk.chunk = -1;
    gk.kind += 100;
    std::shared_ptr<GraphExec> gx = graph_lookup(dev, gk);
    if (!gx) {
        cudaGraph_t g = nullptr;
        KC_CUDA(cudaGraphCreate(&g, 0));
        cudaGraphConditionalHandle hnd;
        cudaGraphNodeParams cp{};
        cudaGraphNode_t node;
        cudaError_t e = cudaGraphConditionalHandleCreate(&hnd, g, 1, cudaGraphCondAssignDefault);
        if (e == cudaSuccess) {
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = hnd;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp);
        }
        if (e != cudaSuccess) {   // no conditional nodes here: the chunked loop
            cudaGetLastError();
            cudaGraphDestroy(g);
            g_while_ok.store(0);
            return 0;
        }
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        cudaStream_t cap_s;
        KC_CUDA(cudaStreamCreateWithFlags(&cap_s, cudaStreamNonBlocking));
        e = cudaStreamBeginCaptureToGraph(cap_s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            launch1(cap_s);
            k_while_cond<<<1, 32, 0, cap_s>>>(st, kWhileCap, hnd);
            cudaGraph_t out = nullptr;
            e = cudaStreamEndCapture(cap_s, &out);
        }
        cudaStreamDestroy(cap_s);
        cudaGraphExec_t ex = nullptr;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            cudaGetLastError();
            g_while_ok.store(0);
            return 0;
        }
        gx = std::make_shared<GraphExec>(ex);
        graph_insert(dev, gk, gx);
    }
    KC_CUDA(cudaGraphLaunch(gx->ex, s));
    int rc = read_state(st, h, s);
    if (rc) return rc;
    count_launches(h->iter * (long long)(kernels_per_iter + 1));
    return 1;
}

}  // namespace kc

using namespace kc;

// polls before a grid-barrier wait of the persistent solvers gives up (0: kSpinLimit);
// lowered only by tests, through kc_debug_barrier_spin_limit
static std::atomic<unsigned> g_spin_limit{0};

template <typename T, class K>
static int launch_persistent(K kernel, const kc_system* A, T* x, const BicgVecs& V, const BicgPtrs& P, GridBar* bar,
                             cudaStream_t s) {
    // device and occupancy queries once per (device, kernel): a solve that
    // takes a few iterations should not wait on host-side queries
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, std::pair<int, int>> cache;   // -> (SMs, blocks per SM)
    int dev = 0, sms = 0, per = 0;
    KC_CUDA(cudaGetDevice(&dev));
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find({dev, (const void*)kernel});
        if (it != cache.end()) {
            sms = it->second.first;
            per = it->second.second;
        } else {
            int coop = 0;
            KC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            KC_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
            if (!coop) return set_error("device %d does not support cooperative launches", dev), KC_ERR_UNSUPPORTED;
            KC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kThreads, 0));
            cache[{dev, (const void*)kernel}] = {sms, per};
        }
    }
    if (per < 1) return set_error("persistent solver kernel cannot be resident"), KC_ERR_UNSUPPORTED;
    dim3 sg = stencil_grid(A->n, A->stride);
    const unsigned lim = g_spin_limit.load(std::memory_order_relaxed);
    PersistGeo pg{(int)sg.x, (int)(sg.x * sg.y), lim ? lim : kSpinLimit};
    int G = std::max(1, std::min(pg.ntiles, sms * per));
    Coef<T> C = coef_of<T>(A);
    Geo g{(int)A->n, A->stride};
    BicgVecs Vc = V;
    BicgPtrs Pc = P;
    T* xx = x;
    void* args[] = {&C, &g, &xx, &Vc, &Pc, &bar, &pg};
    KC_CUDA(cudaMemsetAsync(bar, 0, sizeof(GridBar), s));
    KC_CUDA(cudaLaunchCooperativeKernel((const void*)kernel, dim3(G), dim3(kThreads), args, 0, s));
    count_launches(1);
    return KC_OK;
}

template <typename T>
static int run_solver(const kc_system* A, const void* b, void* x, const void* M, const kc_solve_opts* o, BicgPtrs P,
                      BicgVecs V, GridBar* bar, bool is_cg, bool pre, const GraphKey& key, StartArgs sa,
                      StartArgs sa_cg, HostState* h, cudaStream_t s) {
    const int pb = pw_blocks(A->n);
    Geo g{(int)A->n, A->stride};
    dim3 sg = stencil_grid(A->n, A->stride);
    if (is_cg) {
        k_cg_init<T><<<pb, kPwThreads, 0, s>>>((int)A->n, (const T*)b, (T*)x, (T*)V.r, P, sa_cg);
    } else if (o->x0 == KC_X0_WARM) {
        if (pre) k_invdiag<T><<<pb, kPwThreads, 0, s>>>((int)A->n, (const T*)M, (T*)V.invM);
        k_bicg_init_warm<T><<<sg, kThreads, 0, s>>>(coef_of<T>(A), g, (const T*)b, (const T*)x, (T*)V.r, (T*)V.rt, P,
                                                    sa);
    } else {
        k_bicg_init_cold<T><<<pb, kPwThreads, 0, s>>>((int)A->n, (const T*)b, (T*)x, (T*)V.r, (T*)V.rt,
                                                      pre ? (const T*)M : nullptr, (T*)V.invM, P, sa);
    }
    KC_LAUNCH_CHECK("solver init");
    if (!o->persistent) {
        if (is_cg)
            return drive(o, key, P.st, [&](int m, cudaStream_t ss) { launch_cg_iters<T>(A, (T*)x, V, P, m, ss); }, h, s, 2);
        if (pre)
            return drive(o, key, P.st, [&](int m, cudaStream_t ss) { launch_bicg_iters<T, true>(A, (T*)x, V, P, m, ss); },
                         h, s, 3);
        return drive(o, key, P.st, [&](int m, cudaStream_t ss) { launch_bicg_iters<T, false>(A, (T*)x, V, P, m, ss); },
                     h, s, 3);
    }
    int rc;
    if (is_cg)
        rc = launch_persistent<T>(k_cg_persist<T>, A, (T*)x, V, P, bar, s);
    else if (pre)
        rc = launch_persistent<T>(k_bicg_persist<T, true>, A, (T*)x, V, P, bar, s);
    else
        rc = launch_persistent<T>(k_bicg_persist<T, false>, A, (T*)x, V, P, bar, s);
    if (rc) return rc;
    // the state and the grid barrier (laid out right after it) in one readback
    const size_t span = (size_t)((const char*)bar - (const char*)P.st) + sizeof(GridBar);
    GridBar hb;
    if ((const char*)bar > (const char*)P.st && span <= 4096) {
        const void* hp = readback(P.st, span, s);
        if (!hp) return KC_ERR_CUDA;
        SolverState tmp;
        memcpy(&tmp, hp, sizeof(SolverState));
        memcpy(&hb, (const char*)hp + ((const char*)bar - (const char*)P.st), sizeof(GridBar));
        h->status = tmp.status;
        h->done = tmp.done;
        h->iter = tmp.iter;
        h->rTr = tmp.rTr;
        h->den = tmp.den;
        h->r0Tr = tmp.r0Tr;
        h->prev_rel = tmp.prev_rel;
    } else {
        rc = read_state(P.st, h, s);
        if (rc) return rc;
        KC_CUDA(cudaMemcpy(&hb, bar, sizeof(GridBar), cudaMemcpyDeviceToHost));
    }
    if (hb.err) return set_error("persistent solver: grid barrier timed out"), KC_ERR_CUDA;
    if (o->history && o->history_len > 1) {
        long long to = std::min<long long>(o->history_len, h->iter + 1);
        if (to > 1) {
            k_hist_sqrt<<<(unsigned)std::min<long long>((to + 255) / 256, 1024), 256, 0, s>>>(o->history, 1, to);
            KC_LAUNCH_CHECK("k_hist_sqrt");
        }
    }
    return KC_OK;
}

extern "C" {

unsigned kc_debug_barrier_spin_limit(unsigned polls) {
    return g_spin_limit.exchange(polls, std::memory_order_relaxed);
}

int kc_device_loop(int enable) {
    if (enable < 0)   // bit 0: the CG iteration loop, bit 1: the refinement loop (not refused by the driver)
        return g_while_ok.load(std::memory_order_relaxed) |
               (g_while_ok.load(std::memory_order_relaxed) && g_refloop_ok.load(std::memory_order_relaxed) ? 2 : 0);
    return g_while_ok.exchange(enable ? 1 : 0, std::memory_order_relaxed);
}

int kc_spmv(const kc_system* A, const void* x, void* y, void* stream) {
    int rc = check_system(A);
    if (rc) return rc;
    if (!x || !y) return set_error("kc_spmv: null x or y"), KC_ERR_ARG;
    cudaStream_t s = as_stream(stream);
    Geo g{(int)A->n, A->stride};
    dim3 sg = stencil_grid(A->n, A->stride);
    const int n = (int)A->n, S = A->stride;
    if (A->dtype == KC_F64) {
        const int V = vec_width<double>(A, {x, y});
        if (V == 2)
            k_spmv_vec<double, 2><<<vec_blocks(n / 2, 1 << 30), kThreads, 0, s>>>(coef_of<double>(A), n, S,
                                                                                   (const double*)x, (double*)y);
        else
            k_spmv<double><<<sg, kThreads, 0, s>>>(coef_of<double>(A), g, (const double*)x, (double*)y);
    } else {
        const int V = vec_width<float>(A, {x, y});
        if (V == 4)
            k_spmv_vec<float, 4><<<vec_blocks(n / 4, 1 << 30), kThreads, 0, s>>>(coef_of<float>(A), n, S,
                                                                                  (const float*)x, (float*)y);
        else if (V == 2)
            k_spmv_vec<float, 2><<<vec_blocks(n / 2, 1 << 30), kThreads, 0, s>>>(coef_of<float>(A), n, S,
                                                                                  (const float*)x, (float*)y);
        else
            k_spmv<float><<<sg, kThreads, 0, s>>>(coef_of<float>(A), g, (const float*)x, (float*)y);
    }
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
    Geo g{(int)A->n, A->stride};
    dim3 sg = stencil_grid(A->n, A->stride);
    const long long max_iter = o->max_iter;
    GraphKey key{ws, A->coef, x, A->n, A->stride, A->dtype, pre ? 1 : 0, 16, is_cg ? 1 : 0, A->cs, A->es};
    key.form = A->form;
    HostState h{};
    const double lim = A->dtype == KC_F64 ? 1e300 : 1e30;
    StartArgs sa{o->eps, max_iter, o->omega_break, o->rel_to, o->history, o->history ? o->history_len : 0, lim};
    StartArgs sa_cg{o->eps, max_iter, 0, KC_REL_R0, o->history, o->history ? o->history_len : 0, lim};
    KC_CUDA(cudaMemsetAsync(P.st, 0, sizeof(SolverState), s));
    GridBar* bar = (GridBar*)(base + L.off_bar);
    if (A->dtype == KC_F64)
        rc = run_solver<double>(A, b, x, M, o, P, V, bar, is_cg, pre, key, sa, sa_cg, &h, s);
    else
        rc = run_solver<float>(A, b, x, M, o, P, V, bar, is_cg, pre, key, sa, sa_cg, &h, s);
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

}  // extern "C"

// ---- red-black Gauss-Seidel (FP64) ------------------------------------------------------
// A block owns a kGsTI x kGsTJ tile and stages x over the tile plus a 2-cell
// halo (flat indices, as the stencil kernels: a link across the end of a row
// reaches the next row's cell).  Phase 1 forms b - A x of the incoming x on
// the owned cells (summed for the stopping test) and the new red values on
// the owned cells and their 1-ring (from the staged black values); phase 2
// updates the owned black cells from those red values.  Sweeps alternate
// between the caller's x and a workspace copy (sweep k reads the copy of
// parity k), so no block overwrites cells another block is still staging.
// FP64 arithmetic runs at a small fraction of the FP32 rate on GB300: the
// weights 1/d are formed once per solve, each update is one FMA.
namespace kc {
constexpr int kGsTI = 16, kGsAJ = 32, kGsRY = 8, kGsTJ = kGsAJ - 4, kGsNT = kGsAJ * kGsRY, kGsAI = kGsTI + 4;
// sweeps per captured graph of the inner FP32 Gauss-Seidel solve (sweeps after convergence return at once)
constexpr int kRbgsInnerChunk = 8;
constexpr int kGsR1 = (kGsTI + 2 + kGsRY - 1) / kGsRY;   // rows of phase 1 per thread (owned + 1-ring)
constexpr int kGsR2 = (kGsTI + kGsRY - 1) / kGsRY;       // rows of phase 2 per thread (owned)

__device__ __forceinline__ void cp_async8(double* smem, const double* gmem, bool valid) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(valid ? 8 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_t(double* smem, const double* gmem, bool valid) { cp_async8(smem, gmem, valid); }
__device__ __forceinline__ void cp_async_t(float* smem, const float* gmem, bool valid) { cp_async4(smem, gmem, valid); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }

// weights 1/d (0 on rows with a zero diagonal) and (b, b)
template <typename T>
__global__ void __launch_bounds__(kPwThreads) k_rbgs_init(Coef<T> A, int n, const T* __restrict__ b,
                                                          T* __restrict__ winv, BicgPtrs P, StartArgs sa) {
    Acc<T> acc[1];
    KC_PW_LOOP(n, {
        T d = A.at(0, k);
        if (A.lap) d = d - (((A.at(1, k) + A.at(2, k)) + A.at(3, k)) + A.at(4, k));
        winv[k] = d != T(0) ? T(1) / d : T(0);
        const T bk = __ldg(b + k);
        acc[0].add(bk, bk);
    })
    double s[1];
    if (block_partials<1>(acc, P.partials, P.ld, blockIdx.x, gridDim.x, &P.st->ticket[0], s) && threadIdx.x == 0) {
        SolverState* st = P.st;
        st->hist = sa.hist;
        st->hist_len = sa.hist_len;
        st->iter = 0;
        st->max_iter = sa.max_iter;
        st->eps = sa.eps;
        st->rel_to = sa.rel_to;
        st->den = s[0];   // ||b||^2; replaced by ||b - A x0||^2 at the first sweep for KC_REL_R0
        st->r0Tr = st->rTr = 0.0;
        st->status = KC_MAXITER;
        st->done = sa.max_iter <= 0 ? 1 : 0;
        st->prev_rel = 1.0;
        st->ticket[0] = 0;
    }
}

__device__ __forceinline__ void gs_finish(SolverState* st, double rr) {
    if (st->iter == 0) {
        st->r0Tr = rr;
        if (st->rel_to != KC_REL_B) st->den = rr;
    }
    record_history(st, st->iter, rr);
    st->iter += 1;
    st->rTr = rr;
    const double rel = st->den > 0.0 ? sqrt(rr / st->den) : 0.0;
    st->prev_rel = rel;
    if (rel < st->eps) {
        st->status = KC_OK;
        st->done = 1;
    } else if (!isfinite(rr)) {
        st->status = KC_NONFINITE;
        st->done = 1;
    } else if (st->iter >= st->max_iter) {
        st->status = KC_MAXITER;
        st->done = 1;
    }
}

// One sweep over a 16 x 28 tile: x, b, the weights and the five coefficients of
// the tile and its 2-cell halo are staged together by cp.async (every load of
// the sweep in flight at once; read from global memory phase by phase the
// sweep waited on memory latency twice), then both half-sweeps run from
// shared memory.
template <typename T>
__global__ void __launch_bounds__(kGsNT) k_rbgs_sweep(Coef<T> A, Geo g, const T* __restrict__ b,
                                                      const T* __restrict__ winv, T* __restrict__ x0,
                                                      T* __restrict__ x1, BicgPtrs P) {
    SolverState* st = P.st;
    if (solver_done(st)) return;
    const bool odd = (__ldcg(&st->iter) & 1) != 0;   // set by the previous launch: the same in every block
    const T* __restrict__ x = odd ? x1 : x0;
    T* __restrict__ xo = odd ? x0 : x1;
    __shared__ __align__(16) T sx[kGsAI][kGsAJ];
    __shared__ __align__(16) T sb[kGsAI][kGsAJ];
    __shared__ __align__(16) T sw[kGsAI][kGsAJ];
    __shared__ __align__(16) T sc[5][kGsAI][kGsAJ];
    const int n = g.n, S = g.S;
    const int i0 = blockIdx.y * kGsTI, j0 = blockIdx.x * kGsTJ;
    const int tx = threadIdx.x & (kGsAJ - 1), ty = threadIdx.x / kGsAJ;
    for (int a = ty; a < kGsAI; a += kGsRY) {
        const long long kl = (long long)(i0 + a - 2) * S + (j0 + tx - 2);
        const bool in = kl >= 0 && kl < n;
        const long long kk = in ? kl : 0;
        cp_async_t(&sx[a][tx], x + kk, in);
        cp_async_t(&sb[a][tx], b + kk, in);
        cp_async_t(&sw[a][tx], winv + kk, in);
#pragma unroll
        for (int q = 0; q < 5; ++q) cp_async_t(&sc[q][a][tx], A.c + q * A.cs + kk * A.es, in);
    }
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    // (A x) at staged position (a, t): diagonal first, then W, E, N, S by FMA
    auto ax = [&](int a, int t) -> T {
        const T xc = sx[a][t];
        T y = sc[0][a][t] * xc;
        if (A.lap) {
            y = fma_t(sc[1][a][t], sx[a - 1][t] - xc, y);
            y = fma_t(sc[2][a][t], sx[a + 1][t] - xc, y);
            y = fma_t(sc[3][a][t], sx[a][t + 1] - xc, y);
            y = fma_t(sc[4][a][t], sx[a][t - 1] - xc, y);
        } else {
            y = fma_t(sc[1][a][t], sx[a - 1][t], y);
            y = fma_t(sc[2][a][t], sx[a + 1][t], y);
            y = fma_t(sc[3][a][t], sx[a][t + 1], y);
            y = fma_t(sc[4][a][t], sx[a][t - 1], y);
        }
        return y;
    };
    const int j = j0 + tx - 2;
    const bool jown = tx >= 2 && tx < kGsTJ + 2 && j < S;
    // phase 1: residual of the incoming x (owned cells), new red values (owned cells and 1-ring)
    Acc<T> acc[1];
    T xr[kGsR1];
    bool wr[kGsR1];
#pragma unroll
    for (int m = 0; m < kGsR1; ++m) {
        const int a = 1 + ty + kGsRY * m;
        wr[m] = false;
        xr[m] = T(0);
        if (a > kGsTI + 2 || tx < 1 || tx > kGsAJ - 2) continue;
        const int i = i0 + a - 2;
        const long long kl = (long long)i * S + j;
        if (kl < 0 || kl >= n) continue;
        // a staged position past the end of a row holds the flat cell kl of the next
        // (previous) row; its neighbours are staged around it, so it is updated there
        // too, with the colour of its own (row, column).  (kl < n < 2^31: 32-bit division,
        // and only on those positions -- a 64-bit division per cell dominated the sweep.)
        int colour = (i + j) & 1;
        if (j < 0 || j >= S) {
            const int kk = (int)kl, row = kk / S;
            colour = (row + (kk - row * S)) & 1;
        }
        const T xc = sx[a][tx];
        const T r = sb[a][tx] - ax(a, tx);
        if (jown && a >= 2 && a < kGsTI + 2) acc[0].add(r, r);
        if (colour == 0) {
            xr[m] = fma_t(sw[a][tx], r, xc);
            wr[m] = true;
        }
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < kGsR1; ++m)
        if (wr[m]) sx[1 + ty + kGsRY * m][tx] = xr[m];
    __syncthreads();
    // phase 2: black values of the owned cells from the new red ones; write the owned cells
#pragma unroll
    for (int m = 0; m < kGsR2; ++m) {
        const int a = 2 + ty + kGsRY * m;
        if (a >= kGsTI + 2 || !jown) continue;
        const int i = i0 + a - 2;
        const long long kl = (long long)i * S + j;
        if (kl >= n) continue;
        T xc = sx[a][tx];
        if (((i + j) & 1) != 0) xc = fma_t(sw[a][tx], sb[a][tx] - ax(a, tx), xc);
        xo[kl] = xc;
    }
    double s[1];
    if (block_partials<1>(acc, P.partials, P.ld, block_id(), block_count(), &st->ticket[0], s) && threadIdx.x == 0) {
        gs_finish(st, s[0]);
        st->ticket[0] = 0;
    }
}

static dim3 gs_grid(long long n, int S) {
    const long long rows = (n + S - 1) / S;
    return dim3((unsigned)((S + kGsTJ - 1) / kGsTJ), (unsigned)((rows + kGsTI - 1) / kGsTI));
}

struct GsLayout {
    size_t off_state, off_partials, off_winv, off_x1, total;
    int ld;
};
// elem: bytes per vector element (8 for the FP64 solver, 4 for the FP32 inner solve of the refinement)
static GsLayout gs_layout(long long n, int S, size_t elem = sizeof(double)) {
    GsLayout L{};
    const dim3 g = gs_grid(n, std::max(S, 1));
    const int nb = std::max<int>((int)(g.x * g.y), pw_blocks(n));
    L.ld = (int)align256((size_t)nb * 8) / 8;
    size_t off = 0;
    L.off_state = off;
    off = align256(off + sizeof(SolverState));
    L.off_partials = off;
    off = align256(off + (size_t)L.ld * sizeof(double));
    L.off_winv = off;
    off = align256(off + (size_t)n * elem);
    L.off_x1 = off;
    off = align256(off + (size_t)n * elem);
    L.total = off;
    return L;
}

// ---- several Gauss-Seidel sweeps per launch (the inner solve of kc_rbgs_refined) ----
// A block stages its tile of b, the weights, the coefficients and the incoming
// x with a 2 NU-cell halo (the multigrid tiles' layout) and runs NU sweeps (red,
// black, ...) over shrinking rings in shared memory; half-sweep h covers the
// region less h rings, so the last one ends exactly on the tile.  Staging,
// launch and the absent per-sweep reduction are paid once per NU sweeps.  The
// tile treats a link across the end of a row as a link to zero: valid for
// systems whose rows never link across their ends (checked once per solve by
// k_rows_wrap_links; the padded SIMPLE systems qualify), else the one-sweep
// kernel above runs.  Ping-pong between two iterates: a block's halo reads
// cells that other blocks update in the same launch.
constexpr int kGsbNU = 2, kGsbTI = 12, kGsbAJ = 64, kGsbRY = 4;
constexpr int kGsbSweeps = 12;   // sweeps per refinement pass unless opts->check_every says otherwise

template <int TI, int AJ, int RY, int NU>
__global__ void __launch_bounds__(AJ * RY) k_gs_block_sweeps(MgLvl L, const float* __restrict__ b,
                                                             const float* __restrict__ xin, float* __restrict__ xout) {
    using T = MgTile<TI, AJ, RY, 2 * NU>;
    constexpr int H = T::H;
    // AJ / 2 threads to a staged row, thread m holding its columns 2m and 2m + 1 -- one cell of
    // each colour -- in RP rows a = a0, a0 + RP, ...; RP is even, so every row of a thread has
    // the same parity and its red cell is the same column in all of them.  Each half-sweep
    // then gives every thread one cell per row: no lane of a warp sits out.
    constexpr int HJ = AJ / 2, RP = T::NT / HJ;
    constexpr int R = (T::AI + RP - 1) / RP;   // staged rows per thread
    static_assert(T::NT % HJ == 0 && RP % 2 == 0, "whole rows per pass, an even row step");
    __shared__ __align__(16) float sx[T::A];
    const int i0 = blockIdx.y * TI, j0 = blockIdx.x * T::TJ;
    const int m = threadIdx.x & (HJ - 1), a0 = threadIdx.x / HJ;
    // the thread's red column ((a + b) even; i0 - H and j0 - H are even) and black column
    const int bcol[2] = {2 * m + (a0 & 1), 2 * m + 1 - (a0 & 1)};
    // A thread updates the same cells in every half-sweep: their coefficients, weights and
    // right-hand sides stay in registers (zero outside the grid), only x goes through shared
    // memory -- 5 shared-memory reads per cell update instead of 12.  [colour][row]
    float c0[2][R], c1[2][R], c2[2][R], c3[2][R], c4[2][R], wv[2][R], bv[2][R];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int j = j0 + bcol[q] - H;
        const bool jin = j >= 0 && j < L.NY;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int a = a0 + r * RP;
            const int i = i0 + a - H;
            const bool in = a < T::AI && jin && i >= 0 && i < L.NX;
            const long long k = in ? (long long)i * L.NY + j : 0;
            if (a < T::AI) cp_async4(sx + a * T::AJ + bcol[q], xin + k, in);
            const float* g = L.c + k * L.es;
            c0[q][r] = in ? __ldg(g) : 0.f;
            c1[q][r] = in ? __ldg(g + L.cs) : 0.f;
            c2[q][r] = in ? __ldg(g + 2 * L.cs) : 0.f;
            c3[q][r] = in ? __ldg(g + 3 * L.cs) : 0.f;
            c4[q][r] = in ? __ldg(g + 4 * L.cs) : 0.f;
            wv[q][r] = in ? __ldg(L.winv + k) : 0.f;
            bv[q][r] = in ? __ldg(b + k) : 0.f;
        }
    }
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
#pragma unroll
    for (int h = 1; h <= 2 * NU; ++h) {   // odd h: red ((i + j) even), even h: black
        const int q = (h & 1) ? 0 : 1;
        const int bc = bcol[q];
        if (bc >= h && bc < AJ - h) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int a = a0 + r * RP;
                if (a < h || a >= T::AI - h) continue;
                const int u = a * T::AJ + bc;
                const float xv = sx[u];
                const float y = mg_row(c0[q][r], c1[q][r], c2[q][r], c3[q][r], c4[q][r], L.lap, xv, sx[u - T::AJ],
                                       sx[u + T::AJ], sx[u + 1], sx[u - 1]);
                sx[u] = fmaf(wv[q][r], bv[q][r] - y, xv);
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int bc = bcol[q], j = j0 + bc - H;
        if (bc < H || bc >= T::TJ + H || j >= L.NY) continue;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int a = a0 + r * RP;
            const int i = i0 + a - H;
            if (a >= H && a < TI + H && i < L.NX) xout[i * L.NY + j] = sx[a * T::AJ + bc];
        }
    }
}

// weights 1/d of the red-black sweeps (0 on rows with a zero diagonal)
__global__ void __launch_bounds__(kPwThreads) k_gs_winv(Coef<float> A, int n, float* __restrict__ winv) {
    KC_PW_LOOP(n, {
        float d = A.at(0, k);
        if (A.lap) d = d - (((A.at(1, k) + A.at(2, k)) + A.at(3, k)) + A.at(4, k));
        winv[k] = d != 0.f ? 1.f / d : 0.f;
    })
}

// *flag = 1 when some row links across its end (north link of its last cell or
// south link of its first cell nonzero)
__global__ void __launch_bounds__(kPwThreads) k_rows_wrap_links(Coef<float> A, int NX, int NY, int* __restrict__ flag) {
    KC_PW_LOOP(NX, {
        const int i = k;
        if (A.at(3, i * NY + NY - 1) != 0.f || A.at(4, i * NY) != 0.f) *flag = 1;
    })
}

// NU-sweep launches from d = 0 on A32 d = r (r32); sweeps rounded up to whole launches
static int gs_blocked_run(const kc_system* A, const float* r, float* d, void* ws, size_t ws_bytes, int sweeps,
                          kc_solve_info* info, cudaStream_t s) {
    const GsLayout L = gs_layout(A->n, A->stride, sizeof(float));
    if (!ws || ws_bytes < L.total) return set_error("kc_rbgs_refined: inner workspace %zu < %zu", ws_bytes, L.total),
                                          KC_ERR_WORKSPACE;
    char* base = (char*)ws;
    float* winv = (float*)(base + L.off_winv);
    float* d1 = (float*)(base + L.off_x1);
    const int NY = A->stride, NX = (int)(A->n / A->stride);
    const Coef<float> C = coef_of<float>(A);
    k_gs_winv<<<pw_blocks(A->n), kPwThreads, 0, s>>>(C, (int)A->n, winv);
    KC_LAUNCH_CHECK("k_gs_winv");
    KC_CUDA(cudaMemsetAsync(d, 0, (size_t)A->n * sizeof(float), s));
    const MgLvl G{(const float*)A->coef, A->cs, A->es, NX, NY, A->form == KC_FORM_LAPLACIAN, winv, nullptr};
    const dim3 grid = mg_tile_grid(NX, NY, kGsbTI, kGsbAJ - 4 * kGsbNU);
    const int launches = std::max(1, (sweeps + kGsbNU - 1) / kGsbNU);
    float* cur = d;
    float* nxt = d1;
    for (int q = 0; q < launches; ++q) {
        k_gs_block_sweeps<kGsbTI, kGsbAJ, kGsbRY, kGsbNU><<<grid, kGsbAJ * kGsbRY, 0, s>>>(G, r, cur, nxt);
        KC_LAUNCH_CHECK("k_gs_block_sweeps");
        std::swap(cur, nxt);
    }
    if (cur != d) KC_CUDA(cudaMemcpyAsync(d, cur, (size_t)A->n * sizeof(float), cudaMemcpyDeviceToDevice, s));
    if (info) {
        info->status = KC_OK;   // no inner residual test: the refinement checks the true residual
        info->refinements = 0;
        info->iters = (long long)launches * kGsbNU;
        info->rel_res = 0.0;
        info->r0 = 0.0;
    }
    return KC_OK;
}

// Red-black Gauss-Seidel sweeps of A x = b (T = double: the FP64 solver; T = float: the
// inner solve of kc_rbgs_refined) until the residual of the incoming iterate meets o->eps,
// o->max_iter sweeps, or a non-finite residual.  Checked by the caller: A's dtype is T.
template <typename T>
static int rbgs_run(const kc_system* A, const T* b, T* x, void* ws, size_t ws_bytes, const kc_solve_opts* o,
                    kc_solve_info* info, cudaStream_t s) {
    const dim3 sg = gs_grid(A->n, A->stride);
    if (sg.y > 65535u) return set_error("kc_rbgs: %lld rows of stride %d exceed the launch grid", A->n, A->stride),
                              KC_ERR_ARG;
    const GsLayout L = gs_layout(A->n, A->stride, sizeof(T));
    if (!ws || ws_bytes < L.total) return set_error("kc_rbgs: workspace %zu < %zu", ws_bytes, L.total), KC_ERR_WORKSPACE;
    char* base = (char*)ws;
    BicgPtrs P{(SolverState*)(base + L.off_state), (double*)(base + L.off_partials), L.ld};
    T* winv = (T*)(base + L.off_winv);
    T* x1 = (T*)(base + L.off_x1);
    const int pb = pw_blocks(A->n);
    const Coef<T> C = coef_of<T>(A);
    const Geo g{(int)A->n, A->stride};
    KC_CUDA(cudaMemsetAsync(P.st, 0, sizeof(SolverState), s));
    if (o->x0 != KC_X0_WARM) KC_CUDA(cudaMemsetAsync(x, 0, (size_t)A->n * sizeof(T), s));   // all-zero bits: +0
    const StartArgs sa{o->eps, o->max_iter, 0, o->rel_to, o->history, o->history ? o->history_len : 0, 1e300};
    k_rbgs_init<T><<<pb, kPwThreads, 0, s>>>(C, (int)A->n, b, winv, P, sa);
    KC_LAUNCH_CHECK("k_rbgs_init");
    GraphKey key{ws, A->coef, x, A->n, A->stride, sizeof(T) == 8 ? KC_F64 : KC_F32, 0, 16, 9, A->cs, A->es};
    key.form = A->form;
    key.b = b;
    HostState h{};
    int rc = drive(o, key, P.st,
                   [&](int m, cudaStream_t ss) {
                       for (int q = 0; q < m; ++q) k_rbgs_sweep<T><<<sg, kGsNT, 0, ss>>>(C, g, b, winv, x, x1, P);
                   },
                   &h, s, 1);
    if (rc) return rc;
    if (h.iter & 1) {   // an odd number of sweeps left the iterate in the copy
        KC_CUDA(cudaMemcpyAsync(x, x1, (size_t)A->n * sizeof(T), cudaMemcpyDeviceToDevice, s));
    }
    if (info) {
        info->status = h.status;
        info->refinements = 0;
        info->iters = h.iter;
        info->rel_res = h.prev_rel;
        info->r0 = sqrt(h.r0Tr);
    }
    return h.status;
}
}  // namespace kc

extern "C" {

size_t kc_rbgs_ws_bytes(long long n, int stride) {
    if (n < 1 || stride < 1) return 0;
    return gs_layout(n, stride).total;
}

int kc_rbgs(const kc_system* A, const double* b, double* x, void* ws, size_t ws_bytes, const kc_solve_opts* o,
            kc_solve_info* info, void* stream) {
    int rc = check_system(A);
    if (rc) return rc;
    if (A->dtype != KC_F64) return set_error("kc_rbgs: the system must be FP64"), KC_ERR_ARG;
    if (!b || !x || !o) return set_error("kc_rbgs: null b, x or opts"), KC_ERR_ARG;
    if (o->precond != KC_PRECOND_NONE) return set_error("kc_rbgs: no preconditioner applies"), KC_ERR_ARG;
    return rbgs_run<double>(A, b, x, ws, ws_bytes, o, info, as_stream(stream));
}

}  // extern "C"

// ---- BiCGSTAB without caller-provided memory -------------------------------------
// Some callers cannot allocate device memory for a workspace: a plugin running
// inside a host framework whose device memory is owned by that framework's
// allocator, or a tight loop in which cudaMalloc/cudaFree (which can
// synchronise the whole device) are not acceptable.  kc_bicgstab_noalloc
// serves them from this file-scope scratch array instead.  It is sized for
// systems of up to KC_NOALLOC_MAX_N unknowns (about 4.5 MB, held by every GPU
// that loads the library until the process exits).  In host code the
// array's name is only a host-side stand-in, so its device address is looked
// up with cudaGetSymbolAddress, once per device, with that device current.
// That address is kept for the life of the process: it is not looked up again
// after a cudaDeviceReset or any other teardown of the device's context.
namespace kc {
constexpr size_t kNoallocBytes = 4718592;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];
static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[64] = {nullptr};

static int noalloc_scratch(void** out) {
    int dev = 0;
    KC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_error("kc_bicgstab_noalloc: device index %d out of range", dev), KC_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return KC_OK;
}
}  // namespace kc

extern "C" {

int kc_bicgstab_noalloc(const kc_system* A, const void* b, void* x, const void* M, const kc_solve_opts* opts,
                        kc_solve_info* info, void* stream) {
    int rc = check_system(A);
    if (rc) return rc;
    if (!opts) return set_error("kc_bicgstab_noalloc: null opts"), KC_ERR_ARG;
    if (A->n > KC_NOALLOC_MAX_N)
        return set_error("kc_bicgstab_noalloc: n = %lld exceeds the static scratch limit of %d unknowns; "
                         "use kc_bicgstab with a caller-allocated workspace",
                         A->n, KC_NOALLOC_MAX_N),
               KC_ERR_ARG;
    const size_t need = bicg_layout(A->n, A->stride, A->dtype).total;
    if (need > kNoallocBytes)
        return set_error("kc_bicgstab_noalloc: this system needs %zu bytes of scratch, the static array holds %zu",
                         need, kNoallocBytes),
               KC_ERR_ARG;
    void* scratch = nullptr;
    rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    // the graph path would instantiate graphs (allocations); launch directly
    kc_solve_opts o = *opts;
    o.use_graph = 0;
    // solver-state readbacks into a static pageable buffer: the pinned one is
    // allocated (cudaMallocHost) on a thread's first readback
    PageableReadbacks pageable;
    return bicg_impl(A, b, x, M, scratch, kNoallocBytes, &o, info, stream, false);
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
    L.off_inner = off;   // the inner FP32 solver's workspace: BiCGSTAB or red-black Gauss-Seidel
    L.inner_bytes = std::max(bicg_layout(n, S, KC_F32).total, gs_layout(n, S, sizeof(float)).total);
    off = align256(off + L.inner_bytes);
    L.total = off;
    return L;
}

size_t kc_refined_ws_bytes(long long n, int stride) {
    if (n < 1 || stride < 1) return 0;
    return refine_layout(n, stride).total;
}

}  // extern "C"

// FP64 iterative refinement around an FP32 inner solver: r = b - A64 x in FP64 (and its
// FP32 copy), inner(io, info, r32, d32, inner workspace, bytes, stream, aux) solves A32 d =
// r32 from d = 0 to io.eps relative to ||r32||, x += d; repeated until ||b - A64 x|| / ||b||
// < o->eps.  A sweep that raised the true residual is undone.  prep(slot, stream) may
// enqueue a device-side check that leaves an int in *slot; it comes back with the first
// residual (no extra synchronisation) and reaches every inner call as aux.
template <class Prep, class Inner>
static int refined_core(const char* who, const kc_system* A64, const kc_system* A32, const double* b, double* x,
                        void* ws, size_t ws_bytes, const kc_solve_opts* o, double eps_inner, int max_refine,
                        kc_solve_info* info, void* stream, Prep prep, Inner inner) {
    int rc = check_system(A64);
    if (rc) return rc;
    rc = check_system(A32);
    if (rc) return rc;
    if (A64->dtype != KC_F64 || A32->dtype != KC_F32 || A64->n != A32->n || A64->stride != A32->stride)
        return set_error("%s: need matching FP64 and FP32 systems", who), KC_ERR_ARG;
    if (!b || !x || !o) return set_error("%s: null argument", who), KC_ERR_ARG;
    RefineLayout L = refine_layout(A64->n, A64->stride);
    if (!ws || ws_bytes < L.total)
        return set_error("%s: workspace %zu < %zu", who, ws_bytes, L.total), KC_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    char* base = (char*)ws;
    BicgPtrs P{(SolverState*)(base + L.off_state), (double*)(base + L.off_partials), L.ld};
    double* out2 = (double*)(base + L.off_out);
    float* r32 = (float*)(base + L.off_r32);
    float* d32 = (float*)(base + L.off_d32);
    const long long n = A64->n;
    Geo g{(int)n, A64->stride};
    dim3 sg = stencil_grid(n, A64->stride);
    int pb = pw_blocks(n);
    KC_CUDA(cudaMemsetAsync(P.st, 0, sizeof(SolverState), s));
    if (o->x0 != KC_X0_WARM) k_zero_f64<<<pb, kPwThreads, 0, s>>>((int)n, x);   // warm: x is the initial guess
    KC_CUDA(cudaMemsetAsync(out2, 0, 4 * sizeof(double), s));
    {
        const int prc = prep((int*)(out2 + 3), s);
        if (prc < 0) return prc;
    }
    int aux = 0;
    kc_solve_opts io = *o;
    io.eps = eps_inner;
    io.x0 = KC_X0_ZERO;
    io.precond = KC_PRECOND_NONE;
    io.rel_to = KC_REL_R0;
    io.history = nullptr;
    io.history_len = 0;
    int* flag = (int*)(out2 + 2);
    long long total = 0;
    int status = KC_MAXITER, sweeps = 0, stalls = 0;
    double rel = 1.0, bb = 0.0, best = INFINITY;
    bool applied = false;
    for (int it = 0; it <= max_refine; ++it) {
        launch_refine_resid(A64, g, sg, b, x, r32, P, out2, it == 0, s);
        KC_LAUNCH_CHECK("k_refine_resid");
        double h2[4];
        {
            const void* hp = readback(out2, sizeof(h2), s);
            if (!hp) return KC_ERR_CUDA;
            memcpy(h2, hp, sizeof(h2));
        }
        if (it == 0) {
            bb = h2[1];
            memcpy(&aux, &h2[3], sizeof(int));
        }
        if (!std::isfinite(h2[0]) || !std::isfinite(bb)) {
            // a NaN or Inf in b, x or the system: ||b|| or ||b - A x|| is not finite
            rel = NAN;
            status = KC_NONFINITE;
            break;
        }
        rel = bb > 0 ? sqrt(h2[0] / bb) : 0.0;
        int skipped = 0;
        memcpy(&skipped, &h2[2], sizeof(int));
        if (applied && skipped == 0 && !(rel < best)) {
            // the last correction raised the true residual: undo it, keep the best iterate
            k_sub_f32_from_f64<<<pb, kPwThreads, 0, s>>>((int)n, d32, x);
            KC_LAUNCH_CHECK("undo correction");
            rel = best;
            status = KC_STALL;
            break;
        }
        applied = false;
        if (bb == 0.0 || rel < o->eps) {
            status = KC_OK;
            break;
        }
        if (!isfinite(rel)) {
            status = KC_NONFINITE;
            break;
        }
        // a sweep that does not lower the true residual twice in a row: stalled
        if (rel >= 0.9 * best) {
            if (++stalls >= 2) {
                status = KC_STALL;
                break;
            }
        } else {
            stalls = 0;
        }
        best = std::min(best, rel);
        if (it == max_refine || total >= o->max_iter) break;
        io.max_iter = o->max_iter - total;
        io.eps = std::max(eps_inner, 0.5 * o->eps / rel);   // no deeper than the target needs
        kc_solve_info ii{};
        int r2 = inner(io, &ii, r32, d32, base + L.off_inner, L.inner_bytes, stream, aux);
        if (r2 < 0) return r2;
        total += ii.iters;
        ++sweeps;
        // An inner breakdown (NONFINITE / BREAKDOWN_*) is caught before x is
        // touched in passes A and B; apply whatever finite correction the
        // sweep produced and restart from the FP64 residual.
        KC_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
        k_flag_nonfinite<<<pb, kPwThreads, 0, s>>>((int)n, d32, flag);
        k_add_f32_to_f64<<<pb, kPwThreads, 0, s>>>((int)n, d32, x, flag);
        KC_LAUNCH_CHECK("k_add_f32_to_f64");
        applied = true;
        if (r2 != KC_OK && ii.iters == 0) {
            status = r2;
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

extern "C" {

int kc_bicgstab_refined(const kc_system* A64, const kc_system* A32, const double* b, double* x, void* ws,
                        size_t ws_bytes, const kc_solve_opts* o, double eps_inner, int max_refine,
                        kc_solve_info* info, void* stream) {
    return refined_core("kc_bicgstab_refined", A64, A32, b, x, ws, ws_bytes, o, eps_inner, max_refine, info, stream,
                        [](int*, cudaStream_t) { return KC_OK; },
                        [&](const kc_solve_opts& io, kc_solve_info* ii, const float* r, float* d, void* iw,
                            size_t ib, void* st, int) { return kc_bicgstab(A32, r, d, nullptr, iw, ib, &io, ii, st); });
}

int kc_rbgs_refined(const kc_system* A64, const kc_system* A32, const double* b, double* x, void* ws,
                    size_t ws_bytes, const kc_solve_opts* o, double eps_inner, int max_refine, kc_solve_info* info,
                    void* stream) {
    // rows that never link across their ends (the padded SIMPLE systems): several sweeps per
    // launch, o->check_every of them per refinement pass (0: kGsbSweeps); otherwise one sweep per
    // launch with the residual tested every sweep
    return refined_core("kc_rbgs_refined", A64, A32, b, x, ws, ws_bytes, o, eps_inner, max_refine, info, stream,
                        [&](int* flag, cudaStream_t st) {
                            if (!A32 || A32->stride < 1 || A32->n % A32->stride) return KC_OK;   // checked later
                            const int NX = (int)(A32->n / A32->stride);
                            k_rows_wrap_links<<<pw_blocks(NX), kPwThreads, 0, st>>>(coef_of<float>(A32), NX,
                                                                                     A32->stride, flag);
                            KC_LAUNCH_CHECK("k_rows_wrap_links");
                            return KC_OK;
                        },
                        [&](const kc_solve_opts& io, kc_solve_info* ii, const float* r, float* d, void* iw,
                            size_t ib, void* st, int wraps) {
                            if (!wraps)
                                return gs_blocked_run(A32, r, d, iw, ib, o->check_every > 0 ? o->check_every : kGsbSweeps,
                                                      ii, as_stream(st));
                            kc_solve_opts g = io;
                            g.persistent = 0;
                            g.check_every = kRbgsInnerChunk;   // graph-captured chunks of sweeps
                            return rbgs_run<float>(A32, r, d, iw, ib, &g, ii, as_stream(st));
                        });
}

}  // extern "C"

// ---- multigrid-preconditioned refinement -------------------------------------------
namespace kc {
struct PbLayout {
    size_t off_state, off_partials, off_rstate, off_rpart, off_out, off_r32, off_vec[8], off_x, total;
    int ld;
};
static PbLayout pb_layout(long long n, int S) {
    PbLayout L{};
    dim3 g = stencil_grid(n, std::max(S, 1));
    int nb = std::max<int>((int)(g.x * g.y), pw_blocks(n));
    nb = std::max(nb, mg_fused_blocks0(n, std::max(S, 1)));
    L.ld = (int)align256((size_t)nb * 8) / 8;
    size_t off = 0;
    L.off_state = off;
    off = align256(off + sizeof(SolverState));
    L.off_partials = off;
    off = align256(off + (size_t)5 * L.ld * 8);
    L.off_rstate = off;
    off = align256(off + sizeof(SolverState));
    L.off_rpart = off;
    off = align256(off + (size_t)2 * L.ld * 8);
    L.off_out = off;
    off = align256(off + 64);
    L.off_r32 = off;
    off = align256(off + (size_t)n * 4);
    for (int q = 0; q < 8; ++q) {
        L.off_vec[q] = off;
        off = align256(off + (size_t)n * 4);
    }
    L.off_x = off;
    off = align256(off + (size_t)n * 8);
    L.total = off;
    return L;
}

// m iterations of the preconditioned BiCGSTAB; *kernels = launches per iteration
static int launch_pb_iters(const kc_system* A32, void* mg_ws, const kc_mg_opts* mo, const PbVecs& V, const BicgPtrs& P,
                           int m, cudaStream_t s, int* kernels) {
    Geo g{(int)A32->n, A32->stride};
    dim3 sg = stencil_grid(A32->n, A32->stride);
    const int pb = pw_blocks(A32->n);
    Coef<float> C = coef_of<float>(A32);
    const int* done = &P.st->done;
    int k1 = 0, k2 = 0;
    for (int q = 0; q < m; ++q) {
        k_pb_p<<<pb, kPwThreads, 0, s>>>(g.n, V, P);
        int rc = mg_enqueue(A32, mg_ws, mo, V.p, V.ph, done, s, &k1);
        if (rc) return rc;
        k_pb_Av<<<sg, kThreads, 0, s>>>(C, g, V, P);
        k_pb_s<<<pb, kPwThreads, 0, s>>>(g.n, V, P);
        rc = mg_enqueue(A32, mg_ws, mo, V.s, V.sh, done, s, &k2);
        if (rc) return rc;
        k_pb_At<<<sg, kThreads, 0, s>>>(C, g, V, P);
        k_pb_x<<<pb, kPwThreads, 0, s>>>(g.n, V, P);
        KC_LAUNCH_CHECK_NC("preconditioned iteration");
    }
    if (kernels) *kernels = 5 + k1 + k2;
    return KC_OK;
}

// m iterations of the preconditioned CG; *kernels = launches per iteration
static int launch_pc_iters(const kc_system* A32, void* mg_ws, const kc_mg_opts* mo, const PcVecs& V, const BicgPtrs& P,
                           int m, cudaStream_t s, int* kernels) {
    Geo g{(int)A32->n, A32->stride};
    dim3 sg = stencil_grid(A32->n, A32->stride);
    const int pb = pw_blocks(A32->n);
    Coef<float> C = coef_of<float>(A32);
    const int* done = &P.st->done;
    const MgFused F = mg_fused(A32, mg_ws, mo);
    int k1 = 0;
    for (int q = 0; q < m; ++q) {
        if (F.ok) {
            // the single-reduction CG: its vector updates ride in the V-cycle's level-0
            // launches; the chain is launched with programmatic dependencies (each kernel
            // waits on its predecessor in-kernel)
            PcfLaunch pl;
            int rc = pcf_launch(F.L0, &pl);
            if (rc) return rc;
            KC_CUDA(launch_chain(k_pcc_down0<kMgTI0, kMgAJ0, kMgRY0>, dim3(pl.blocks), dim3(kMgNT0), pl.smem_down, s,
                                 F.L0, F.x0pre, F.b1, F.NX1, F.NY1, V, P, 1, pl.gd));
            rc = mg_enqueue_coarse(A32, mg_ws, mo, done, s, &k1);
            if (rc) return rc;
            KC_CUDA(launch_chain(k_pcc_up0<kMgTI0, kMgAJ0, kMgRY0>, dim3(pl.blocks), dim3(kMgNT0), pl.smem_up, s, F.L0,
                                 (const float*)F.x0pre, F.final1, F.NX1, F.NY1, F.alpha0, V, P, pl.gu));
            k1 += 2;   // level 0's DOWN and UP: with the coarse levels, the whole iteration
        } else {
            k_pc_1<<<sg, kThreads, 0, s>>>(C, g, V, P);
            k_pc_2<<<pb, kPwThreads, 0, s>>>(g.n, V, P);
            int rc = mg_enqueue(A32, mg_ws, mo, V.r[0], V.z, done, s, &k1);
            if (rc) return rc;
            k_pc_3<<<pb, kPwThreads, 0, s>>>(g.n, V, P);
            KC_LAUNCH_CHECK_NC("preconditioned CG iteration");
            k1 += 2;
        }
    }
    if (kernels) *kernels = (F.ok ? 0 : 1) + k1;
    return KC_OK;
}

// number of kernels one preconditioned CG iteration launches
static int pc_iter_kernels(const kc_system* A32, void* mg_ws, const kc_mg_opts* mo) {
    return mg_fused(A32, mg_ws, mo).ok ? mg_cycle_kernels(A32, mo) : 1 + mg_cycle_kernels(A32, mo) + 2;
}
// Multigrid-preconditioned FP32 Krylov solve (BiCGSTAB or CG) inside FP64
// iterative refinement: r = b - A64 x in FP64, inner solve A32 d = r to
// eps_inner from d = 0 (d accumulated in FP64), x += d, until
// ||b - A64 x|| / ||b|| < eps.  A correction that raises the true residual is
// undone and ends the solve with KC_STALL, as do two sweeps in a row that
// gain less than 10 %.
// ---- the whole refinement on the device (the multigrid CG path) --------------------------
// The host loop of mg_refined reads the FP64 residual norms back after every
// refinement pass and decides there (converged, stalled, undo, next inner
// tolerance), and launches the next pass: a host round trip with the GPU idle
// per pass.  Here the same decisions run in a one-thread kernel, and the whole
// refinement is one graph launch: an outer WHILE node whose body is [FP64
// residual, decision, undo, inner start, first V-cycle, the inner CG loop (a
// nested WHILE node), correction], then one readback of the final state.  The
// decision kernel sets both loops' conditions and, when the refinement ends,
// marks the inner solver done, so the rest of that body pass does nothing.
// The arithmetic of every decision is the host loop's (IEEE sqrt and
// division), so the iterates, the iteration counts and the result are the
// same bit for bit.  (The host loop finishes an inner solve that reached the
// device loop's 1024-iteration cap with chunked graphs; here the refinement
// goes on from the true residual.)
struct RefState {
    double bb, best, rel, eps, eps_inner, eps_in;
    long long total, max_iter;
    int it, max_refine, stalls, applied, status, done, undo, sweeps;
};
static_assert(sizeof(RefState) <= 192, "the refinement state lives in the 256-byte output slot");

__global__ void k_ref_init(RefState* R, double eps, double eps_inner, long long max_iter, int max_refine) {
    if (threadIdx.x || blockIdx.x) return;
    R->bb = 0.0;
    R->best = INFINITY;
    R->rel = 1.0;
    R->eps = eps;
    R->eps_inner = eps_inner;
    R->eps_in = eps_inner;
    R->total = 0;
    R->max_iter = max_iter;
    R->it = 0;
    R->max_refine = max_refine;
    R->stalls = R->applied = R->done = R->undo = R->sweeps = 0;
    R->status = KC_MAXITER;
}

__global__ void k_ref_decide(RefState* R, const double* __restrict__ out2, int* flag, SolverState* st,
                             cudaGraphConditionalHandle ho, cudaGraphConditionalHandle hi) {
    if (threadIdx.x || blockIdx.x) return;
    bool stop = false;
    int status = KC_MAXITER;
    const double h0 = __ldcg(out2);
    const int skipped = __ldcg(flag);
    if (R->it == 0) R->bb = __ldcg(out2 + 1);
    const double bb = R->bb;
    double rel;
    if (!isfinite(h0) || !isfinite(bb)) {   // a NaN or Inf in b, x or the system
        rel = NAN;
        status = KC_NONFINITE;
        stop = true;
    } else {
        rel = bb > 0 ? sqrt(h0 / bb) : 0.0;
        if (R->applied && skipped == 0 && !(rel < R->best)) {   // the last correction raised the residual
            R->undo = 1;
            rel = R->best;
            status = KC_STALL;
            stop = true;
        } else {
            R->applied = 0;
            if (bb == 0.0 || rel < R->eps) {
                status = KC_OK;
                stop = true;
            } else if (!isfinite(rel)) {
                status = KC_NONFINITE;
                stop = true;
            } else {
                if (rel >= 0.9 * R->best) {
                    if (++R->stalls >= 2) {
                        status = KC_STALL;
                        stop = true;
                    }
                } else {
                    R->stalls = 0;
                }
                if (!stop) {
                    R->best = fmin(R->best, rel);
                    if (R->it == R->max_refine || R->total >= R->max_iter) stop = true;   // KC_MAXITER
                }
            }
        }
    }
    R->rel = rel;
    R->it += 1;
    if (stop) {
        R->status = status;
        R->done = 1;
        st->done = 1;   // the rest of this pass: every inner kernel returns at once
        cudaGraphSetConditional(hi, 0u);
        cudaGraphSetConditional(ho, 0u);
        return;
    }
    R->eps_in = fmax(R->eps_inner, 0.5 * R->eps / rel);
    *flag = 0;
    unsigned long long* w = reinterpret_cast<unsigned long long*>(st);   // the inner state from zero
    for (unsigned q = 0; q < sizeof(SolverState) / sizeof(unsigned long long); ++q) w[q] = 0ull;
    cudaGraphSetConditional(hi, 1u);
    cudaGraphSetConditional(ho, 1u);
}

__global__ void __launch_bounds__(kPwThreads) k_ref_undo(int n, const double* __restrict__ d, double* __restrict__ x,
                                                         const RefState* R) {
    if (!__ldcg(&R->undo)) return;
    KC_PW_LOOP(n, { x[k] -= __ldg(d + k); })
}

// k_bicg_init_cold for the inner pass, its tolerance and cap from the refinement state
__global__ void __launch_bounds__(kPwThreads)
    k_bicg_init_cold_ref(int n, const float* __restrict__ b, float* __restrict__ x, float* __restrict__ r,
                         float* __restrict__ rt, BicgPtrs P, const RefState* R) {
    if (__ldcg(&R->done)) return;
    Acc<float> acc[1];
    KC_PW_LOOP(n, {
        const float bk = __ldg(b + k);
        r[k] = bk;
        rt[k] = bk;
        x[k] = 0.f;
        acc[0].add(bk, bk);
    })
    double s[1];
    if (block_partials<1>(acc, P.partials, P.ld, blockIdx.x, gridDim.x, &P.st->ticket[0], s) && threadIdx.x == 0) {
        const StartArgs sa{__ldcg(&R->eps_in), __ldcg(&R->max_iter) - __ldcg(&R->total), 0, KC_REL_R0, nullptr, 0,
                           1e30};
        bicg_start(P.st, s[0], s[0], sa);
        P.st->ticket[0] = 0;
    }
}

__global__ void k_ref_after(RefState* R, const SolverState* st, cudaGraphConditionalHandle ho) {
    if (threadIdx.x || blockIdx.x || R->done) return;
    R->total += st->iter;
    R->sweeps += 1;
    R->applied = 1;
    if (st->status != KC_OK && st->iter == 0) {
        R->status = st->status;
        R->done = 1;
        cudaGraphSetConditional(ho, 0u);
    }
}


// The refinement of the multigrid CG as one graph launch; returns 1 when it ran (info filled),
// 0 when the caller should run the host loop, < 0 on a CUDA error.
template <class First, class Iter1>
static int refine_on_device(const GraphKey& key, const kc_system* A64, Geo g, dim3 sg, const double* b, double* x,
                            float* r32, BicgPtrs P, BicgPtrs Rr, double* out2, int* flag, PbVecs V, double* d64,
                            const kc_solve_opts* o, double eps_inner, int max_refine, First&& first, Iter1&& iter1,
                            int kernels_per_iter, kc_solve_info* info, int* status_out, cudaStream_t s) {
    if (!g_refloop_ok.load(std::memory_order_relaxed) || !g_while_ok.load(std::memory_order_relaxed)) return 0;
    const long long n = A64->n;
    const int pb = pw_blocks(n);
    RefState* R = reinterpret_cast<RefState*>(out2 + 8);
    int dev = 0;
    KC_CUDA(cudaGetDevice(&dev));
    GraphKey gk = key;
    gk.chunk = -2;
    gk.kind += 200;
    std::shared_ptr<GraphExec> gx = graph_lookup(dev, gk);
    if (!gx) {
        bool ok = true;
        cudaGraph_t gr = nullptr;
        cudaStream_t cs = nullptr, cs2 = nullptr;
        cudaGraphConditionalHandle ho{}, hi{};
        cudaGraphNodeParams cpo{}, cpi{};
        cudaGraphNode_t onode, inode;
        ok = cudaGraphCreate(&gr, 0) == cudaSuccess &&
             cudaGraphConditionalHandleCreate(&ho, gr, 1, cudaGraphCondAssignDefault) == cudaSuccess;
        if (ok) {
            cpo.type = cudaGraphNodeTypeConditional;
            cpo.conditional.handle = ho;
            cpo.conditional.type = cudaGraphCondTypeWhile;
            cpo.conditional.size = 1;
            ok = cudaGraphAddNode(&onode, gr, nullptr, nullptr, 0, &cpo) == cudaSuccess;
        }
        cudaGraph_t body = ok ? cpo.conditional.phGraph_out[0] : nullptr;
        ok = ok && cudaGraphConditionalHandleCreate(&hi, body, 0, cudaGraphCondAssignDefault) == cudaSuccess;
        ok = ok && cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) == cudaSuccess &&
             cudaStreamCreateWithFlags(&cs2, cudaStreamNonBlocking) == cudaSuccess;
        if (ok && cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
                      cudaSuccess) {
            launch_refine_resid(A64, g, sg, b, x, r32, Rr, out2, true, cs);   // ||b||^2 too: the first pass keeps it
            k_ref_decide<<<1, 32, 0, cs>>>(R, out2, flag, P.st, ho, hi);
            k_ref_undo<<<pb, kPwThreads, 0, cs>>>((int)n, d64, x, R);
            k_bicg_init_cold_ref<<<pb, kPwThreads, 0, cs>>>((int)n, r32, V.sh, V.r, V.rt, P, R);
            k_zero_f64<<<pb, kPwThreads, 0, cs>>>((int)n, d64);
            first(cs);   // the first V-cycle (returns at once when the refinement is done)
            // the inner CG loop: a WHILE node added to the capture by hand, its body captured on cs2
            cudaStreamCaptureStatus cst;
            cudaGraph_t cg = nullptr;
            const cudaGraphNode_t* deps = nullptr;
            size_t nd = 0;
            ok = cudaStreamGetCaptureInfo(cs, &cst, nullptr, &cg, &deps, nullptr, &nd) == cudaSuccess &&
                 cst == cudaStreamCaptureStatusActive;
            if (ok) {
                cpi.type = cudaGraphNodeTypeConditional;
                cpi.conditional.handle = hi;
                cpi.conditional.type = cudaGraphCondTypeWhile;
                cpi.conditional.size = 1;
                ok = cudaGraphAddNode(&inode, cg, deps, nullptr, nd, &cpi) == cudaSuccess &&
                     cudaStreamUpdateCaptureDependencies(cs, &inode, nullptr, 1, cudaStreamSetCaptureDependencies) ==
                         cudaSuccess;
            }
            if (ok && cudaStreamBeginCaptureToGraph(cs2, cpi.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                    cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
                iter1(cs2);
                k_while_cond<<<1, 32, 0, cs2>>>(P.st, kWhileCap, hi);
                cudaGraph_t o2 = nullptr;
                ok = cudaStreamEndCapture(cs2, &o2) == cudaSuccess;
            } else {
                ok = false;
            }
            k_flag_nonfinite_f64<<<pb, kPwThreads, 0, cs>>>((int)n, d64, flag);
            k_add_f64<<<pb, kPwThreads, 0, cs>>>((int)n, d64, x, flag);
            k_ref_after<<<1, 32, 0, cs>>>(R, P.st, ho);
            cudaGraph_t o1 = nullptr;
            ok = (cudaStreamEndCapture(cs, &o1) == cudaSuccess) && ok;
        } else {
            ok = false;
        }
        if (cs2) cudaStreamDestroy(cs2);
        if (cs) cudaStreamDestroy(cs);
        cudaGraphExec_t ex = nullptr;
        if (ok) ok = cudaGraphInstantiate(&ex, gr, 0) == cudaSuccess;
        if (gr) cudaGraphDestroy(gr);
        if (!ok) {
            cudaGetLastError();
            g_refloop_ok.store(0);
            return 0;
        }
        gx = std::make_shared<GraphExec>(ex);
        graph_insert(dev, gk, gx);
    }
    k_ref_init<<<1, 32, 0, s>>>(R, o->eps, eps_inner, o->max_iter, max_refine);
    KC_LAUNCH_CHECK("k_ref_init");
    KC_CUDA(cudaGraphLaunch(gx->ex, s));
    const void* hp = readback(R, sizeof(RefState), s);
    if (!hp) return KC_ERR_CUDA;
    RefState h;
    memcpy(&h, hp, sizeof(RefState));
    count_launches(h.total * (long long)(kernels_per_iter + 1) + 12ll * h.it);
    if (info) {
        info->status = h.status;
        info->refinements = h.sweeps;
        info->iters = h.total;
        info->rel_res = h.rel;
        info->r0 = sqrt(h.bb);
    }
    *status_out = h.status;
    return 1;
}

static int mg_refined(bool cg, const kc_system* A64, const kc_system* A32, const double* b, double* x, const double* x0,
                      void* mg_ws, const kc_mg_opts* mg_opts, void* ws, size_t ws_bytes, const kc_solve_opts* o,
                      double eps_inner, int max_refine, kc_solve_info* info, void* stream) {
    const char* name = cg ? "kc_pcg_refined" : "kc_pbicgstab_refined";
    int rc = check_system(A64);
    if (rc) return rc;
    rc = check_system(A32);
    if (rc) return rc;
    if (A64->dtype != KC_F64 || A32->dtype != KC_F32 || A64->n != A32->n || A64->stride != A32->stride)
        return set_error("%s: need matching FP64 and FP32 systems", name), KC_ERR_ARG;
    if (!b || !x || !o || !mg_ws || !mg_opts) return set_error("%s: null argument", name), KC_ERR_ARG;
    PbLayout L = pb_layout(A64->n, A64->stride);
    if (!ws || ws_bytes < L.total) return set_error("%s: workspace %zu < %zu", name, ws_bytes, L.total), KC_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    char* base = (char*)ws;
    BicgPtrs P{(SolverState*)(base + L.off_state), (double*)(base + L.off_partials), L.ld};
    BicgPtrs R{(SolverState*)(base + L.off_rstate), (double*)(base + L.off_rpart), L.ld};
    double* out2 = (double*)(base + L.off_out);
    int* flag = (int*)(out2 + 2);
    float* r32 = (float*)(base + L.off_r32);
    float* fv[8];
    for (int q = 0; q < 8; ++q) fv[q] = (float*)(base + L.off_vec[q]);
    double* d64 = (double*)(base + L.off_x);
    PbVecs V{fv[0], fv[1], fv[2], fv[3], fv[4], fv[5], fv[6], fv[7], d64};
    PcVecs W{{fv[0], fv[5]}, fv[1], {fv[2], fv[3]}, fv[4], d64, {fv[6], fv[7]}};
    const long long n = A64->n;
    Geo g{(int)n, A64->stride};
    dim3 sg = stencil_grid(n, A64->stride);
    const int pb = pw_blocks(n);
    KC_CUDA(cudaMemsetAsync(R.st, 0, sizeof(SolverState), s));
    KC_CUDA(cudaMemsetAsync(out2, 0, 4 * sizeof(double), s));
    if (x0) k_copy_f64<<<pb, kPwThreads, 0, s>>>((int)n, x0, x);
    else k_zero_f64<<<pb, kPwThreads, 0, s>>>((int)n, x);
    KC_LAUNCH_CHECK("x0");
    long long total = 0;
    int status = KC_MAXITER, sweeps = 0, stalls = 0;
    double rel = 1.0, bb = 0.0, best = INFINITY;
    bool applied = false;
    const StartArgs sa{eps_inner, 0, 0, KC_REL_R0, nullptr, 0, 1e30};
    GraphKey key{ws, A32->coef, mg_ws, n, A32->stride, KC_F32, cg ? 8 : 7, 4, 2, A32->cs, A32->es};
    key.form = A32->form;
    key.ohash = bytes_hash(mg_opts, sizeof(kc_mg_opts));
    if (cg && o->use_graph) {
        // the whole refinement as one graph launch (falls back to the host loop below where the
        // driver refuses nested conditional nodes)
        GraphKey rk = key;
        rk.x64 = x;
        rk.b = b;
        rk.c64 = A64->coef;
        const int per_iter = pc_iter_kernels(A32, mg_ws, mg_opts);
        int dst = KC_MAXITER;
        const int ran = refine_on_device(
            rk, A64, g, sg, b, x, r32, P, R, out2, flag, V, d64, o, eps_inner, max_refine,
            [&](cudaStream_t cs) {
                const MgFused F = mg_fused(A32, mg_ws, mg_opts);
                int mk = 0;
                if (F.ok) {
                    PcfLaunch pl;
                    if (pcf_launch(F.L0, &pl)) return;
                    k_pcc_down0<kMgTI0, kMgAJ0, kMgRY0><<<pl.blocks, kMgNT0, pl.smem_down, cs>>>(
                        F.L0, F.x0pre, F.b1, F.NX1, F.NY1, W, P, 0, pl.gd);
                    (void)mg_enqueue_coarse(A32, mg_ws, mg_opts, &P.st->done, cs, &mk);
                    k_pcc_up0<kMgTI0, kMgAJ0, kMgRY0><<<pl.blocks, kMgNT0, pl.smem_up, cs>>>(
                        F.L0, F.x0pre, F.final1, F.NX1, F.NY1, F.alpha0, W, P, pl.gu);
                } else {
                    (void)mg_enqueue(A32, mg_ws, mg_opts, W.r[0], W.z, &P.st->done, cs, &mk);
                    k_pc_3<<<pb, kPwThreads, 0, cs>>>((int)n, W, P);
                }
            },
            [&](cudaStream_t cs) { (void)launch_pc_iters(A32, mg_ws, mg_opts, W, P, 1, cs, nullptr); }, per_iter,
            info, &dst, s);
        if (ran < 0) return ran;
        if (ran) return dst;
    }
    for (int it = 0; it <= max_refine; ++it) {
        launch_refine_resid(A64, g, sg, b, x, r32, R, out2, it == 0, s);
        KC_LAUNCH_CHECK("k_refine_resid");
        double h2[3];
        {
            const void* hp = readback(out2, sizeof(h2), s);
            if (!hp) return KC_ERR_CUDA;
            memcpy(h2, hp, sizeof(h2));
        }
        if (it == 0) bb = h2[1];
        if (!std::isfinite(h2[0]) || !std::isfinite(bb)) {
            // a NaN or Inf in b, x or the system: ||b|| or ||b - A x|| is not finite
            rel = NAN;
            status = KC_NONFINITE;
            break;
        }
        rel = bb > 0 ? sqrt(h2[0] / bb) : 0.0;
        int skipped = 0;
        memcpy(&skipped, &h2[2], sizeof(int));
        if (applied && skipped == 0 && !(rel < best)) {
            // the last correction raised the true residual: undo it, keep the best iterate
            k_sub_f64<<<pb, kPwThreads, 0, s>>>((int)n, d64, x);
            KC_LAUNCH_CHECK("undo correction");
            rel = best;
            status = KC_STALL;
            break;
        }
        applied = false;
        if (bb == 0.0 || rel < o->eps) {
            status = KC_OK;
            break;
        }
        if (!isfinite(rel)) {
            status = KC_NONFINITE;
            break;
        }
        if (rel >= 0.9 * best) {
            if (++stalls >= 2) {
                status = KC_STALL;
                break;
            }
        } else {
            stalls = 0;
        }
        best = std::min(best, rel);
        if (it == max_refine || total >= o->max_iter) break;
        // inner FP32 solve of A d = r32 from d = 0, to eps_inner -- or less
        // far when that overshoots the target: a sweep that reduces its
        // residual by 0.5 eps / rel reaches ||r|| / ||b|| < eps
        StartArgs si = sa;
        si.max_iter = o->max_iter - total;
        si.eps = std::max(eps_inner, 0.5 * o->eps / rel);
        KC_CUDA(cudaMemsetAsync(P.st, 0, sizeof(SolverState), s));
        // the cold start zeroes an FP32 iterate and writes r~: both go to
        // slots that are scratch until a V-cycle writes them
        k_bicg_init_cold<float><<<pb, kPwThreads, 0, s>>>((int)n, r32, V.sh, V.r, V.rt, nullptr, nullptr, P, si);
        k_zero_f64<<<pb, kPwThreads, 0, s>>>((int)n, d64);
        KC_LAUNCH_CHECK("inner init");
        if (cg) {
            // z_0 = M r_0 and (r_0, z_0)
            const MgFused F = mg_fused(A32, mg_ws, mg_opts);
            int mk = 0;
            if (F.ok) {
                PcfLaunch pl;
                rc = pcf_launch(F.L0, &pl);
                if (rc) return rc;
                k_pcc_down0<kMgTI0, kMgAJ0, kMgRY0><<<pl.blocks, kMgNT0, pl.smem_down, s>>>(F.L0, F.x0pre, F.b1, F.NX1,
                                                                                            F.NY1, W, P, 0, pl.gd);
                KC_LAUNCH_CHECK("k_pcc_down0");
                rc = mg_enqueue_coarse(A32, mg_ws, mg_opts, &P.st->done, s, &mk);
                if (rc) return rc;
                k_pcc_up0<kMgTI0, kMgAJ0, kMgRY0><<<pl.blocks, kMgNT0, pl.smem_up, s>>>(F.L0, F.x0pre, F.final1, F.NX1,
                                                                                        F.NY1, F.alpha0, W, P, pl.gu);
                KC_LAUNCH_CHECK("k_pcc_up0");
            } else {
                rc = mg_enqueue(A32, mg_ws, mg_opts, W.r[0], W.z, &P.st->done, s, &mk);
                if (rc) return rc;
                k_pc_3<<<pb, kPwThreads, 0, s>>>((int)n, W, P);
                KC_LAUNCH_CHECK("pcg start");
            }
            count_launches(mk);
        }
        kc_solve_opts io = *o;
        io.max_iter = si.max_iter;
        io.check_every = o->check_every > 0 ? o->check_every : 4;
        const int per_iter = cg ? pc_iter_kernels(A32, mg_ws, mg_opts) : 5 + 2 * mg_cycle_kernels(A32, mg_opts);
        HostState h{};
        int ran = 0;
        if (cg && io.use_graph) {
            // the iterations loop on the device; the chunked loop below finishes a solve the
            // device loop left unfinished (its iteration cap) or runs where it is unavailable
            ran = drive_while(key, P.st,
                              [&](cudaStream_t ss) { (void)launch_pc_iters(A32, mg_ws, mg_opts, W, P, 1, ss, nullptr); },
                              &h, s, per_iter);
            if (ran < 0) return ran;
        }
        if (cg && (!ran || !h.done))
            rc = drive(&io, key, P.st,
                       [&](int m, cudaStream_t ss) { (void)launch_pc_iters(A32, mg_ws, mg_opts, W, P, m, ss, nullptr); },
                       &h, s, per_iter);
        else if (!cg)
            rc = drive(&io, key, P.st,
                       [&](int m, cudaStream_t ss) { (void)launch_pb_iters(A32, mg_ws, mg_opts, V, P, m, ss, nullptr); },
                       &h, s, per_iter);
        if (rc) return rc;
        total += h.iter;
        ++sweeps;
        KC_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
        k_flag_nonfinite_f64<<<pb, kPwThreads, 0, s>>>((int)n, d64, flag);
        k_add_f64<<<pb, kPwThreads, 0, s>>>((int)n, d64, x, flag);
        KC_LAUNCH_CHECK("correction");
        count_launches(1);
        applied = true;
        if (h.status != KC_OK && h.iter == 0) {
            status = h.status;
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

}  // namespace kc

extern "C" {

size_t kc_pbicgstab_ws_bytes(long long n, int stride) {
    if (n < 1 || stride < 1) return 0;
    return pb_layout(n, stride).total;
}

int kc_pbicgstab_refined(const kc_system* A64, const kc_system* A32, const double* b, double* x, const double* x0,
                         void* mg_ws, const kc_mg_opts* mg_opts, void* ws, size_t ws_bytes, const kc_solve_opts* o,
                         double eps_inner, int max_refine, kc_solve_info* info, void* stream) {
    return mg_refined(false, A64, A32, b, x, x0, mg_ws, mg_opts, ws, ws_bytes, o, eps_inner, max_refine, info, stream);
}

int kc_pcg_refined(const kc_system* A64, const kc_system* A32, const double* b, double* x, const double* x0,
                   void* mg_ws, const kc_mg_opts* mg_opts, void* ws, size_t ws_bytes, const kc_solve_opts* o,
                   double eps_inner, int max_refine, kc_solve_info* info, void* stream) {
    return mg_refined(true, A64, A32, b, x, x0, mg_ws, mg_opts, ws, ws_bytes, o, eps_inner, max_refine, info, stream);
}

}  // extern "C"
