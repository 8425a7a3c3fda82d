// The batched channel executor as one persistent launch.
//
// kc_channel_batch_fused advances n independent channel instances (uneven
// grid sizes) by `steps` time steps in ONE kernel launch: a group of threads
// owns an instance -- a whole 1024-thread block for an instance of at least
// 40k p cells, a quarter block (256 threads, four instances to a block)
// otherwise -- and runs its whole SIMPLE time steps (the outer loop of
// karman_taichi.py:633-659 / simple.py:270-281 with the stages of the mixed
// path), with a named barrier of its own between the phases and nothing on
// the host between them.  Instances never wait on each other, so the launch
// needs no grid-wide synchronisation and no instance can hold another up.
// Per outer iteration, per instance:
//
//   assemble_momentum   u_row / v_row (kc_simple.cuh) on every face: the
//                       FP64 systems and their FP32 copies, bit for bit the
//                       rows kc_assemble_momentum writes
//   u*, v*              FP32 red-black Gauss-Seidel (12 sweeps per pass) in
//                       FP64 refinement from the previous outer iteration's
//                       u*, v*, to ||b - A x|| / ||b|| < eps, at most 200
//                       sweeps (kc_rbgs_refined's method)
//   relax, outlet       u = a u* + (1 - a) u, v alike; the outlet column's
//                       zero gradient and mass-flow rescale
//   assemble_pcorr      the p' rows (FP64, the FP32 Laplacian-form copy) and
//                       the mass residual max |mdiv| over fluid cells
//   p'                  multigrid-preconditioned FP32 CG in FP64 refinement
//                       from p' = 0 to rel. tol eps (inner tol eps_inner_p);
//                       aggregation multigrid as kc_mg.cu (2x2 aggregates,
//                       Galerkin coarse rows in Laplacian form, isolated
//                       rows, red-black smoothing with the instance's
//                       mg_opts omega / alpha / nu_coarse), the coarsest
//                       level (<= 64 cells) solved by its dense inverse
//   correct             u, v, p corrections (kc_correct's arithmetic)
//
// and the outer loop stops when the mass residual is <= mass_tol or after
// max_outer iterations; then u0 = u, v0 = v.  Residual norms (FP64) and the
// CG inner products (double-float) are group reductions in a fixed order, and
// an instance's thread count depends on its size alone, so every instance
// computes bit for bit what it computes alone in a batch of one, whatever
// else shares the launch.  The reductions differ in order from the
// per-instance multi-block kernels of kc_channel_step, so the two agree to
// rounding, not bitwise.
//
// Why a block (or a quarter) per instance: an instance of the batched
// configuration has 4k-83k cells; as separate launches every stage is a few
// microseconds of launch latency for a fraction of a microsecond of work.
// Here the phases of one instance are separated by a barrier (~0.1 us), the
// large instances each get an SM of their own, and four small ones share
// one: the 256 instances of the batch fit in one wave of 141 blocks.  The
// launch ends with its slowest instance, so the sizes are balanced per
// thread: 83k cells on 1024 threads, at most 22k on 256.
//
// Loads use the coherent path throughout (no __ldg): every array is written
// by an earlier phase of the same launch.
#include "kc_simple.cuh"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

namespace kc {
namespace {

constexpr int kBBlock = 1024;            // threads per block
constexpr int kBGroups = 4;              // instances per block at most
constexpr int kBBigCells = 40000;        // instances of at least this many p cells get a whole block, the
                                         // others 256 threads (four to a block)
constexpr int kBLevels = 12;             // multigrid levels at most
constexpr int kBCoarse = 64;             // cells of the coarsest level at most (dense inverse in shared memory)
constexpr int kBGsSweeps = 12;           // Gauss-Seidel sweeps per momentum refinement pass
constexpr long long kBMomentumSweeps = 200;
constexpr int kBMaxRefine = 30;
constexpr int kBMaxCg = 1000;            // CG iterations per refinement pass at most
constexpr int kBCoarseFallbackSweeps = 64;
constexpr int kBMaxBicg = 4000;          // fallback BiCGSTAB iterations per refinement pass at most

// exact e / d for 0 <= e < 2^32 / d by a multiply-high (m = 0 stands for d = 1)
struct Div {
    unsigned m;
    __device__ __forceinline__ int q(int e) const { return m ? (int)__umulhi((unsigned)e, m) : e; }
};
inline Div div_of(int d) { return Div{d == 1 ? 0u : (unsigned)((1ull << 32) / (unsigned)d + 1)}; }

// The threads of one instance: a whole block (1024) or a quarter of one (256).  Its phases are
// separated by a named barrier of its own (id gi + 1, nt threads), so the instances sharing a
// block never wait on each other.
struct Grp {
    int tid, nt, gi;
    __device__ __forceinline__ void sync() const {
        asm volatile("bar.sync %0, %1;" ::"r"(gi + 1), "r"(nt) : "memory");
    }
    // barrier that also returns whether p was nonzero in any thread of the group
    __device__ __forceinline__ int any(int p) const {
        int r;
        asm volatile(
            "{\n\t.reg .pred q, o;\n\t"
            "setp.ne.s32 q, %1, 0;\n\t"
            "bar.red.or.pred o, %2, %3, q;\n\t"
            "selp.s32 %0, 1, 0, o;\n\t}"
            : "=r"(r)
            : "r"(p), "r"(gi + 1), "r"(nt)
            : "memory");
        return r;
    }
    __device__ __forceinline__ int warps() const { return nt >> 5; }
};

struct BLvl {
    float* c;             // 5 planes [NX][NY], Laplacian form (level 0: the FP32 p' copy)
    float* b;             // right-hand side (level 0: CG's residual)
    float* x;             // iterate (level 0: CG's z)
    float* w;             // smoother weights
    unsigned char* iso;   // rows without links
    int NX, NY;
    Div dy, dh;           // division by NY and by (NY + 1) / 2 (the cells of one colour in a row)
    float omega, alpha;   // smoother weight, weight of the coarse correction prolonged into this level
    int nu;               // red-black sweeps before and after the coarse correction
};

struct BInst {
    kc_phys P;
    SimpleK K;
    int max_outer;
    double mass_tol, eps, eps_inner_p;
    double *u, *v, *p, *u0, *v0, *pc, *um, *vm;
    const unsigned char* solid;
    double *cu, *bu, *cv, *bv, *cp, *bp;
    float *cu32, *bu32, *cv32, *bv32, *cp32, *bp32;
    float *gw, *r32, *d32;                 // momentum: Gauss-Seidel weights, FP32 residual, correction
    float *bt[5];                          // fallback BiCGSTAB: r~, p, v, s, t (the larger grid's size)
    double eps_inner;                      // inner tolerance of the fallback BiCGSTAB passes
    float *cr, *cz, *cpv, *cq, *cd;        // p' CG: r, z, p, q and the correction
    BLvl lv[kBLevels];
    int levels;
    Div du, dv, dp;                        // row lengths of the u, v and p grids
    Div dhu, dhv;                          // ... and their halves rounded up (the u and v grids)
    int nt;                                // threads of the instance (1024 or 256)
    kc_channel_stats* last;                // per instance: the last step's statistics
    kc_channel_stats* total;               // ... and the sums over the launch's steps
};

// ---- group reductions with the result in every thread (fixed order) ---------------
template <int NV>
__device__ __forceinline__ void bsum(const Grp& g, double (&v)[NV]) {
    __shared__ double sh[kBGroups][NV][32];
    const int lane = g.tid & 31, w = g.tid >> 5, nw = g.warps();
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        const double s = warp_sum(v[q]);
        if (lane == 0) sh[g.gi][q][w] = s;
    }
    g.sync();
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double s = 0.0;
        for (int i = 0; i < nw; ++i) s += sh[g.gi][q][i];
        v[q] = s;
    }
    g.sync();
}
// double-float sums of FP32 products (Acc<float>), as doubles in every thread
template <int NV>
__device__ __forceinline__ void bsum_df(const Grp& g, const Acc<float> (&a)[NV], double (&out)[NV]) {
    __shared__ DF sh[kBGroups][NV][32];
    const int lane = g.tid & 31, w = g.tid >> 5, nw = g.warps();
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        DF v = a[q].s;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v = df_add(v, DF{__shfl_down_sync(kFull, v.hi, o), __shfl_down_sync(kFull, v.lo, o)});
        if (lane == 0) sh[g.gi][q][w] = v;
    }
    g.sync();
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        DF v = sh[g.gi][q][0];
        for (int i = 1; i < nw; ++i) v = df_add(v, sh[g.gi][q][i]);
        out[q] = (double)v.hi + (double)v.lo;
    }
    g.sync();
}
__device__ __forceinline__ double bmax(const Grp& g, double v) {
    __shared__ double sh[kBGroups][32];
    const int lane = g.tid & 31, w = g.tid >> 5, nw = g.warps();
    v = warp_max(v);
    if (lane == 0) sh[g.gi][w] = v;
    g.sync();
    double m = 0.0;
    for (int i = 0; i < nw; ++i) m = fmax(m, sh[g.gi][i]);
    g.sync();
    return m;
}

// ---- 5-point stencils over [NX][NY] with zero values outside -------------------
// standard form (momentum rows): y = c0 x + c1 xW + c2 xE + c3 xN + c4 xS
template <typename T, typename X>
__device__ __forceinline__ X row_std(const T* c, long long n, const X* x, int NX, int NY, int k, int i, int j) {
    const X xk = x[k];
    const X xw = i > 0 ? x[k - NY] : X(0), xe = i + 1 < NX ? x[k + NY] : X(0);
    const X xn = j + 1 < NY ? x[k + 1] : X(0), xs = j > 0 ? x[k - 1] : X(0);
    X y = X(c[k]) * xk;
    y = fma(X(c[n + k]), xw, y);
    y = fma(X(c[2 * n + k]), xe, y);
    y = fma(X(c[3 * n + k]), xn, y);
    y = fma(X(c[4 * n + k]), xs, y);
    return y;
}
// Laplacian form (p' and coarse rows): y = c0 x + sum c_nb (x_nb - x)
__device__ __forceinline__ float row_lap(const float* c, int n, const float* x, int NX, int NY, int k, int i, int j) {
    const float xk = x[k];
    const float xw = i > 0 ? x[k - NY] : 0.f, xe = i + 1 < NX ? x[k + NY] : 0.f;
    const float xn = j + 1 < NY ? x[k + 1] : 0.f, xs = j > 0 ? x[k - 1] : 0.f;
    float y = c[k] * xk;
    y = fmaf(c[n + k], xw - xk, y);
    y = fmaf(c[2 * n + k], xe - xk, y);
    y = fmaf(c[3 * n + k], xn - xk, y);
    y = fmaf(c[4 * n + k], xs - xk, y);
    return y;
}

// One red-black half-sweep x += W (b - A x) over the cells (i, j) with (i + j) & 1 == col, in
// standard (LAP false) or Laplacian form.  A thread walks the cells of its colour only and keeps
// U of them in flight: every load of a group is issued before any of its stores, so the group's
// memory latencies overlap (the stores could alias the next cell's loads for all the compiler
// knows; they do not: a cell reads only cells of the other colour).
template <bool LAP, int U>
__device__ __forceinline__ void hs_sweep(const Grp& g, const float* c, const float* b, const float* w, float* x, int NX, int NY,
                                         Div dh, int col) {
    const int half = (NY + 1) >> 1, cnt = NX * half, n = NX * NY;
    for (int e0 = g.tid; e0 < cnt; e0 += g.nt * U) {
        int kk[U];
        float a0[U], a1[U], a2[U], a3[U], a4[U], xc[U], xw[U], xe[U], xn[U], xs[U], bk[U], wk[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int e = e0 + u * g.nt;
            int k = -1, i = 0, j = 0;
            if (e < cnt) {
                i = dh.q(e);
                j = 2 * (e - i * half) + ((i + col) & 1);
                if (j < NY) k = i * NY + j;
            }
            kk[u] = k;
            if (k >= 0) {
                xc[u] = x[k];
                xw[u] = i > 0 ? x[k - NY] : 0.f;
                xe[u] = i + 1 < NX ? x[k + NY] : 0.f;
                xn[u] = j + 1 < NY ? x[k + 1] : 0.f;
                xs[u] = j > 0 ? x[k - 1] : 0.f;
                a0[u] = c[k];
                a1[u] = c[n + k];
                a2[u] = c[2 * n + k];
                a3[u] = c[3 * n + k];
                a4[u] = c[4 * n + k];
                bk[u] = b[k];
                wk[u] = w[k];
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (kk[u] < 0) continue;
            const float o = xc[u];
            float y = a0[u] * o;
            if (LAP) {
                y = fmaf(a1[u], xw[u] - o, y);
                y = fmaf(a2[u], xe[u] - o, y);
                y = fmaf(a3[u], xn[u] - o, y);
                y = fmaf(a4[u], xs[u] - o, y);
            } else {
                y = fmaf(a1[u], xw[u], y);
                y = fmaf(a2[u], xe[u], y);
                y = fmaf(a3[u], xn[u], y);
                y = fmaf(a4[u], xs[u], y);
            }
            x[kk[u]] = fmaf(wk[u], bk[u] - y, o);
        }
    }
    g.sync();
}

// ---- stage 1: momentum assembly ------------------------------------------------
__device__ __noinline__ void b_assemble_momentum(const Grp& g, const BInst& I) {
    const kc_phys& P = I.P;
    const Dims D = dims_of(P);
    const Solid S{I.solid, D.NYp};
    {
        const int NX = D.nx + 3, NY = D.NYu, n = NX * NY;
        for (int k = g.tid; k < n; k += g.nt) {
            const int i = I.du.q(k), j = k - i * NY;
            double c[5], b;
            u_row(P, I.K, D, S, I.u, I.v, I.p, I.u0, i, j, c, b);
#pragma unroll
            for (int q = 0; q < 5; ++q) {
                I.cu[(long long)q * n + k] = c[q];
                I.cu32[(long long)q * n + k] = f64_to_f32(c[q]);
            }
            I.bu[k] = b;
            I.bu32[k] = f64_to_f32(b);
        }
    }
    {
        const int NX = D.nx + 2, NY = D.NYv, n = NX * NY;
        for (int k = g.tid; k < n; k += g.nt) {
            const int i = I.dv.q(k), j = k - i * NY;
            double c[5], b;
            v_row(P, I.K, D, S, I.u, I.v, I.p, I.v0, i, j, c, b);
#pragma unroll
            for (int q = 0; q < 5; ++q) {
                I.cv[(long long)q * n + k] = c[q];
                I.cv32[(long long)q * n + k] = f64_to_f32(c[q]);
            }
            I.bv[k] = b;
            I.bv32[k] = f64_to_f32(b);
        }
    }
    g.sync();
}

// ---- stage 2: a momentum system by FP32 red-black Gauss-Seidel in FP64 refinement ----
// r32 = b - A x in FP64, returns {||r||^2, ||b||^2}
__device__ __forceinline__ void b_resid64(const Grp& g, const double* c, const double* bvec, const double* x, float* r32, int NX,
                                          int NY, Div dy, double (&s)[2]) {
    const int n = NX * NY;
    double rr = 0.0, bb = 0.0;
    constexpr int U = 2;   // cells in flight per thread: loads before stores
    for (int k0 = g.tid; k0 < n; k0 += g.nt * U) {
        double bk[U], y[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int k = k0 + u * g.nt;
            if (k < n) {
                const int i = dy.q(k), j = k - i * NY;
                bk[u] = bvec[k];
                y[u] = row_std<double, double>(c, n, x, NX, NY, k, i, j);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int k = k0 + u * g.nt;
            if (k < n) {
                const double r = bk[u] - y[u];
                r32[k] = f64_to_f32(r);
                rr = fma(r, r, rr);
                bb = fma(bk[u], bk[u], bb);
            }
        }
    }
    s[0] = rr;
    s[1] = bb;
    bsum<2>(g, s);
}

// status of a refinement pass over {||r||^2, ||b||^2}, as refined_core in kc_solver.cu:
// 0 go on, 1 stop with *status set
struct Refine {
    double best = INFINITY, bb = 0.0, rel = 1.0;
    int stalls = 0;
    bool applied = false;
    __device__ int check(int it, const double (&s)[2], int* status, bool* undo) {
        *undo = false;
        if (it == 0) bb = s[1];
        if (!isfinite(s[0]) || !isfinite(bb)) {
            rel = NAN;
            *status = KC_NONFINITE;
            return 1;
        }
        rel = bb > 0 ? sqrt(s[0] / bb) : 0.0;
        if (applied && !(rel < best)) {   // the last correction raised the true residual: undo it
            *undo = true;
            rel = best;
            *status = KC_STALL;
            return 1;
        }
        applied = false;
        return 0;
    }
};

// ---- the fallback: FP32 BiCGSTAB in FP64 refinement (kc_bicgstab_refined's method) ----
// y = A32 x on cell k (standard or Laplacian form)
__device__ __forceinline__ float row32(bool lap, const float* c, int n, const float* x, int NX, int NY, int k, int i,
                                       int j) {
    return lap ? row_lap(c, n, x, NX, NY, k, i, j) : row_std<float, float>(c, n, x, NX, NY, k, i, j);
}
// A32 d = r from d = 0 to ||r_k|| <= eps_in ||r_0|| (r is overwritten); returns the iterations, *status
__device__ int b_bicg_inner(const Grp& g, const BInst& I, bool lap, const float* c, int NX, int NY, Div dy, float* r,
                            float* d, double eps_in, int max_it, int* status) {
    const int n = NX * NY;
    float* rt = I.bt[0];
    float* p = I.bt[1];
    float* v = I.bt[2];
    float* sv = I.bt[3];
    float* t = I.bt[4];
    double s1[1], s2[2];
    Acc<float> a1[1], a2[2];
    for (int k = g.tid; k < n; k += g.nt) {
        const float rk = r[k];
        rt[k] = rk;
        p[k] = 0.f;
        v[k] = 0.f;
        d[k] = 0.f;
        a1[0].add(rk, rk);
    }
    bsum_df<1>(g, a1, s1);
    const double rr0 = s1[0];
    *status = KC_OK;
    if (rr0 == 0.0) return 0;
    const double stop2 = eps_in * eps_in * rr0;
    double rho = 1.0, alpha = 1.0, omega = 1.0;
    int it = 0;
    *status = KC_MAXITER;
    while (it < max_it) {
        a1[0] = Acc<float>{};
        for (int k = g.tid; k < n; k += g.nt) a1[0].add(rt[k], r[k]);
        bsum_df<1>(g, a1, s1);
        const double rho_n = s1[0];
        if (rho_n == 0.0 || !isfinite(rho_n)) {
            *status = isfinite(rho_n) ? KC_BREAKDOWN_RHO : KC_NONFINITE;
            break;
        }
        const float beta = (float)((rho_n / rho) * (alpha / omega));
        const float om = (float)omega;
        for (int k = g.tid; k < n; k += g.nt) p[k] = fmaf(beta, fmaf(-om, v[k], p[k]), r[k]);
        g.sync();
        a1[0] = Acc<float>{};
        for (int k = g.tid; k < n; k += g.nt) {
            const int i = dy.q(k), j = k - i * NY;
            const float y = row32(lap, c, n, p, NX, NY, k, i, j);
            v[k] = y;
            a1[0].add(rt[k], y);
        }
        bsum_df<1>(g, a1, s1);
        if (s1[0] == 0.0 || !isfinite(s1[0])) {
            *status = isfinite(s1[0]) ? KC_BREAKDOWN_RHO : KC_NONFINITE;
            break;
        }
        alpha = rho_n / s1[0];
        const float af = (float)alpha;
        a1[0] = Acc<float>{};
        for (int k = g.tid; k < n; k += g.nt) {
            const float sk = fmaf(-af, v[k], r[k]);
            sv[k] = sk;
            a1[0].add(sk, sk);
        }
        bsum_df<1>(g, a1, s1);
        ++it;
        if (s1[0] <= stop2) {   // s is small enough: x += alpha p
            for (int k = g.tid; k < n; k += g.nt) d[k] = fmaf(af, p[k], d[k]);
            g.sync();
            *status = KC_OK;
            break;
        }
        a2[0] = Acc<float>{};
        a2[1] = Acc<float>{};
        for (int k = g.tid; k < n; k += g.nt) {
            const int i = dy.q(k), j = k - i * NY;
            const float y = row32(lap, c, n, sv, NX, NY, k, i, j);
            t[k] = y;
            a2[0].add(y, sv[k]);
            a2[1].add(y, y);
        }
        bsum_df<2>(g, a2, s2);
        if (!(s2[1] > 0.0) || !isfinite(s2[0])) {
            *status = isfinite(s2[1]) ? KC_BREAKDOWN_OMEGA : KC_NONFINITE;
            for (int k = g.tid; k < n; k += g.nt) d[k] = fmaf(af, p[k], d[k]);
            g.sync();
            break;
        }
        omega = s2[0] / s2[1];
        const float wf = (float)omega;
        a1[0] = Acc<float>{};
        for (int k = g.tid; k < n; k += g.nt) {
            d[k] = fmaf(wf, sv[k], fmaf(af, p[k], d[k]));
            const float rn = fmaf(-wf, t[k], sv[k]);
            r[k] = rn;
            a1[0].add(rn, rn);
        }
        bsum_df<1>(g, a1, s1);
        rho = rho_n;
        if (!isfinite(s1[0])) {
            *status = KC_NONFINITE;
            break;
        }
        if (s1[0] <= stop2) {
            *status = KC_OK;
            break;
        }
        if (omega == 0.0) {
            *status = KC_BREAKDOWN_OMEGA;
            break;
        }
    }
    return it;
}

// FP64 refinement with the FP32 BiCGSTAB inner passes, from the x given; the refinement
// rules of b_gs_refined
__device__ __noinline__ void b_bicg_refined(const Grp& g, const BInst& I, bool lap, const double* c,
                                            const double* bvec, const float* c32, double* x, int NX, int NY, Div dy,
                                            long long max_iter, long long* iters, int* status_out) {
    const int n = NX * NY;
    float* r = I.r32;
    float* d = I.d32;
    Refine R;
    int status = KC_MAXITER;
    long long total = 0;
    for (int it = 0; it <= kBMaxRefine; ++it) {
        double s[2];
        b_resid64(g, c, bvec, x, r, NX, NY, dy, s);
        bool undo = false;
        if (R.check(it, s, &status, &undo)) {
            if (undo) {
                for (int k = g.tid; k < n; k += g.nt) x[k] -= (double)d[k];
                g.sync();
            }
            break;
        }
        if (R.bb == 0.0 || R.rel < I.eps) {
            status = KC_OK;
            break;
        }
        if (R.rel >= 0.9 * R.best) {
            if (++R.stalls >= 2) {
                status = KC_STALL;
                break;
            }
        } else {
            R.stalls = 0;
        }
        R.best = fmin(R.best, R.rel);
        if (it == kBMaxRefine || total >= max_iter) break;
        int st = KC_OK;
        const int k_it = b_bicg_inner(g, I, lap, c32, NX, NY, dy, r, d, fmax(I.eps_inner, 0.5 * I.eps / R.rel),
                                      (int)(max_iter - total < kBMaxBicg ? max_iter - total : kBMaxBicg), &st);
        total += k_it;
        int bad = 0;
        for (int k = g.tid; k < n; k += g.nt) bad |= !isfinite(d[k]);
        bad = g.any(bad);
        if (!bad)
            for (int k = g.tid; k < n; k += g.nt) x[k] += (double)d[k];
        g.sync();
        R.applied = !bad;
        if ((st != KC_OK && k_it == 0) || bad) {
            status = bad ? KC_NONFINITE : st;
            break;
        }
    }
    g.sync();
    *iters += total;
    *status_out = status;
}

__device__ __noinline__ void b_gs_refined(const Grp& g, const double* c, const double* bvec, const float* c32, double* x, int NX, int NY, Div dy,
                             Div dh, const BInst& I, long long* iters, int* fallbacks, int* status_out) {
    const int n = NX * NY;
    float* gw = I.gw;
    float* r = I.r32;
    float* d = I.d32;
    for (int k = g.tid; k < n; k += g.nt) {
        const float a = c32[k];
        gw[k] = a != 0.f ? 1.f / a : 0.f;
    }
    Refine R;
    int status = KC_MAXITER;
    long long total = 0;
    for (int it = 0; it <= kBMaxRefine; ++it) {
        double s[2];
        b_resid64(g, c, bvec, x, r, NX, NY, dy, s);   // (its barrier also publishes gw and the last x)
        bool undo = false;
        if (R.check(it, s, &status, &undo)) {
            if (undo) {
                for (int k = g.tid; k < n; k += g.nt) x[k] -= (double)d[k];
                g.sync();
            }
            break;
        }
        if (R.bb == 0.0 || R.rel < I.eps) {
            status = KC_OK;
            break;
        }
        if (R.rel >= 0.9 * R.best) {
            if (++R.stalls >= 2) {
                status = KC_STALL;
                break;
            }
        } else {
            R.stalls = 0;
        }
        R.best = fmin(R.best, R.rel);
        if (it == kBMaxRefine || total >= kBMomentumSweeps) break;
        // kBGsSweeps red-black sweeps of A32 d = r from d = 0 (red first)
        for (int k = g.tid; k < n; k += g.nt) {   // the first (red) half-sweep from d = 0
            const int i = dy.q(k), j = k - i * NY;
            d[k] = ((i + j) & 1) == 0 ? gw[k] * r[k] : 0.f;
        }
        g.sync();
        for (int h = 1; h < 2 * kBGsSweeps; ++h) hs_sweep<false, 2>(g, c32, r, gw, d, NX, NY, dh, h & 1);
        total += kBGsSweeps;
        int bad = 0;
        for (int k = g.tid; k < n; k += g.nt) bad |= !isfinite(d[k]);
        bad = g.any(bad);
        if (bad) {
            status = KC_NONFINITE;
            break;
        }
        for (int k = g.tid; k < n; k += g.nt) x[k] += (double)d[k];
        g.sync();   // the next residual reads x's neighbours
        R.applied = true;
    }
    g.sync();
    *iters += total;
    if (status != KC_OK && status != KC_NONFINITE) {
        // the sweeps missed eps: the refined BiCGSTAB takes over from the best iterate, as the
        // native step does (kc_channel_step's solve_sys)
        ++*fallbacks;
        b_bicg_refined(g, I, false, c, bvec, c32, x, NX, NY, dy, 50ll * n, iters, &status);
    }
    *status_out = status;
}

// ---- stage 3: under-relaxation and the outlet column (k_relax, k_outlet_conserve) ----
__device__ __noinline__ void b_relax_outlet(const Grp& g, const BInst& I) {
    const kc_phys& P = I.P;
    const Dims D = dims_of(P);
    const Solid S{I.solid, D.NYp};
    const double a = P.alpha_m;
    {
        const int NY = D.NYu, n = (D.nx + 3) * NY;
        for (int k = g.tid; k < n; k += g.nt) {
            const int i = I.du.q(k), j = k - i * NY;
            if (unk_u(P, S, i, j)) I.u[k] = a * I.um[k] + I.K.one_m_am * I.u[k];
        }
    }
    {
        const int NY = D.NYv, n = (D.nx + 2) * NY;
        for (int k = g.tid; k < n; k += g.nt) {
            const int i = I.dv.q(k), j = k - i * NY;
            if (unk_v(P, S, i, j)) I.v[k] = a * I.vm[k] + I.K.one_m_am * I.v[k];
        }
    }
    g.sync();
    // outlet: zero gradient, then the outflow rescaled to the inflow
    double acc[2] = {0.0, 0.0};
    for (int j = 1 + g.tid; j <= D.ny; j += g.nt) {
        const double w = I.u[(long long)D.nx * D.NYu + j];
        I.u[(long long)(D.nx + 1) * D.NYu + j] = w;
        acc[0] += I.u[(long long)1 * D.NYu + j];
        acc[1] += w;
    }
    bsum<2>(g, acc);
    const double coef = acc[0] / acc[1];
    for (int j = 1 + g.tid; j <= D.ny; j += g.nt) {
        double* o = I.u + (long long)(D.nx + 1) * D.NYu + j;
        *o = coef * *o;
    }
    g.sync();
}

// ---- stage 4: p' rows and the mass residual (the channel branch of k_assemble_pcorr) ----
__device__ __noinline__ double b_assemble_pcorr(const Grp& g, const BInst& I) {
    const kc_phys& P = I.P;
    const Dims D = dims_of(P);
    const Solid S{I.solid, D.NYp};
    const int NX = D.nx + 2, NY = D.NYp, n = NX * NY;
    const int nx = D.nx, ny = D.ny;
    const double rho = P.rho, dx = P.dx, dy = P.dy;
    const double* u = I.u;
    const double* v = I.v;
    double mx = 0.0;
    for (int k = g.tid; k < n; k += g.nt) {
        const int i = I.dp.q(k), j = k - i * NY;
        double c[5] = {0, 0, 0, 0, 0}, b = 0.0, xs = 0.0;
        if (i >= 1 && i <= nx && j >= 1 && j <= ny) {
            const double md = rho * (u[(long long)i * D.NYu + j] - u[(long long)(i + 1) * D.NYu + j]) * dy +
                              rho * (v[(long long)i * D.NYv + j] - v[(long long)i * D.NYv + j + 1]) * dx;
            if (S.cell(i, j)) {
                c[0] = 1.0;
            } else {
                const double tw = I.K.nrdy2 / I.cu[(long long)i * D.NYu + j];
                const double te = I.K.nrdy2 / I.cu[(long long)(i + 1) * D.NYu + j];
                const double tv = I.K.nrdx2 / I.cv[(long long)i * D.NYv + j];
                const double tn = I.K.nrdx2 / I.cv[(long long)i * D.NYv + j + 1];
                double aW = 0.0, aE = 0.0, aN = 0.0, aS = 0.0;
                if (unk_u(P, S, i, j)) aW = tw;
                if (unk_u(P, S, i + 1, j)) aE = te;
                if (i == nx && unk_u(P, S, nx, j)) aE = tw;   // the outlet row links to face nx again
                if (unk_v(P, S, i, j + 1)) aN = tn;
                if (unk_v(P, S, i, j)) aS = tv;
                xs = aW + aE + aN + aS;
                c[0] = -xs;
                c[1] = aW;
                c[2] = aE;
                c[3] = aN;
                c[4] = aS;
                b = md;
                mx = fmax(mx, fabs(md));
            }
        }
#pragma unroll
        for (int q = 0; q < 5; ++q) I.cp[(long long)q * n + k] = c[q];
        I.bp[k] = b;
        I.cp32[k] = f64_to_f32(c[0] + xs);   // Laplacian form: component 0 is the row sum
#pragma unroll
        for (int q = 1; q < 5; ++q) I.cp32[(long long)q * n + k] = f64_to_f32(c[q]);
        I.bp32[k] = f64_to_f32(b);
    }
    return bmax(g, mx);   // (its barriers publish the rows)
}

// ---- stage 5: the p' solve --------------------------------------------------------
// hierarchy: smoother weights and isolation flags of level 0, then the Galerkin
// coarse rows level by level (k_mg_diag0, k_mg_coarsen), then the coarsest inverse
__device__ __noinline__ void b_mg_setup(const Grp& g, const BInst& I, float* inv, int* inv_bad) {
    {
        const BLvl& L = I.lv[0];
        const int n = L.NX * L.NY;
        for (int k = g.tid; k < n; k += g.nt) {
            const float w = L.c[n + k], ea = L.c[2 * n + k], no = L.c[3 * n + k], so = L.c[4 * n + k];
            const float d = L.c[k] - (w + ea + no + so);
            const bool linked = w != 0.f || ea != 0.f || no != 0.f || so != 0.f;
            L.iso[k] = linked ? 0 : 1;
            L.w[k] = d == 0.f ? 0.f : (linked ? L.omega / d : 1.f / d);
        }
        g.sync();
    }
    for (int l = 0; l + 1 < I.levels; ++l) {
        const BLvl& F = I.lv[l];
        const BLvl& Q = I.lv[l + 1];
        const int nf = F.NX * F.NY, nc = Q.NX * Q.NY;
        for (int kc = g.tid; kc < nc; kc += g.nt) {
            const int Ic = Q.dy.q(kc), Jc = kc - Ic * Q.NY;
            float rs = 0.f, aW = 0.f, aE = 0.f, aN = 0.f, aS = 0.f;
            for (int di = 0; di < 2; ++di) {
                const int i = 2 * Ic + di;
                if (i >= F.NX) continue;
                for (int dj = 0; dj < 2; ++dj) {
                    const int j = 2 * Jc + dj;
                    if (j >= F.NY) continue;
                    const int k = i * F.NY + j;
                    if (F.iso[k]) continue;
                    const float w = F.c[nf + k], ea = F.c[2 * nf + k], no = F.c[3 * nf + k], so = F.c[4 * nf + k];
                    float r = F.c[k];
                    if (i - 1 < 0 || F.iso[k - F.NY]) r -= w;
                    else if (di == 0) aW += w;
                    if (i + 1 >= F.NX || F.iso[k + F.NY]) r -= ea;
                    else if (di == 1) aE += ea;
                    if (j + 1 >= F.NY || F.iso[k + 1]) r -= no;
                    else if (dj == 1) aN += no;
                    if (j - 1 < 0 || F.iso[k - 1]) r -= so;
                    else if (dj == 0) aS += so;
                    rs += r;
                }
            }
            Q.c[kc] = rs;
            Q.c[nc + kc] = aW;
            Q.c[2 * nc + kc] = aE;
            Q.c[3 * nc + kc] = aN;
            Q.c[4 * nc + kc] = aS;
            const bool linked = aW != 0.f || aE != 0.f || aN != 0.f || aS != 0.f;
            const float d = rs - (aW + aE + aN + aS);
            Q.iso[kc] = linked ? 0 : 1;
            Q.w[kc] = d == 0.f ? 0.f : (linked ? Q.omega / d : 1.f / d);
        }
        g.sync();
    }
    // coarsest: Gauss-Jordan inversion in shared memory, no pivoting (the Galerkin operator of
    // the symmetric p' rows with the outlet folded into the row sums is positive definite; a row
    // without coupled children gets a unit diagonal and a zero right-hand side)
    const BLvl& C = I.lv[I.levels - 1];
    const int nc = C.NX * C.NY;
    for (int e = g.tid; e < nc * nc; e += g.nt) {
        const int i = e / nc, j = e - i * nc;
        const float w = C.c[nc + i], ea = C.c[2 * nc + i], no = C.c[3 * nc + i], so = C.c[4 * nc + i];
        float d = C.c[i] - (((w + ea) + no) + so);
        if (w == 0.f && ea == 0.f && no == 0.f && so == 0.f && d == 0.f) d = 1.f;
        const int jr = i % C.NY;
        float val = 0.f;
        if (j == i) val = d;
        else if (j == i - C.NY) val = w;
        else if (j == i + C.NY) val = ea;
        else if (j == i + 1 && jr + 1 < C.NY) val = no;
        else if (j == i - 1 && jr >= 1) val = so;
        inv[e] = val;
    }
    __shared__ float rowp_s[kBGroups][kBCoarse], colp_s[kBGroups][kBCoarse];
    __shared__ int bad_s[kBGroups];
    float* rowp = rowp_s[g.gi];
    float* colp = colp_s[g.gi];
    int& bad = bad_s[g.gi];
    if (g.tid == 0) bad = 0;
    g.sync();
    for (int p = 0; p < nc; ++p) {
        if (g.tid < nc) {
            rowp[g.tid] = inv[p * nc + g.tid];
            colp[g.tid] = inv[g.tid * nc + p];
        }
        g.sync();
        const float piv = rowp[p];
        if (!(piv > 0.f) || !isfinite(piv)) {   // uniform: every thread reads the same pivot
            if (g.tid == 0) bad = 1;
            break;
        }
        const float ip = 1.f / piv;
        for (int e = g.tid; e < nc * nc; e += g.nt) {
            const int i = e / nc, j = e - i * nc;
            const float sp = j == p ? ip : rowp[j] * ip;
            inv[e] = i == p ? sp : (j == p ? -colp[i] * ip : fmaf(-colp[i], sp, inv[e]));
        }
        g.sync();
    }
    g.sync();
    *inv_bad = bad;
    g.sync();
}

// one V-cycle z = M r on the hierarchy (level 0: b = r, x = z), kc_mg.cu's cycle:
// down: red start x = W b, 2 nu - 1 half-sweeps (black, red, ...), restriction of the
// residual over coupled cells; coarsest: x = A^-1 b; up: prolongation onto coupled cells
// scaled by alpha, 2 nu half-sweeps (black, red, ...)
__device__ __forceinline__ void b_half_sweep(const Grp& g, const BLvl& L, int col) {
    hs_sweep<true, 2>(g, L.c, L.b, L.w, L.x, L.NX, L.NY, L.dh, col);
}

__device__ __noinline__ void b_vcycle(const Grp& g, const BInst& I, const float* inv, int inv_bad) {
    const int Lc = I.levels - 1;
    for (int l = 0; l < Lc; ++l) {
        const BLvl& L = I.lv[l];
        const BLvl& Q = I.lv[l + 1];
        const int n = L.NX * L.NY;
        for (int k = g.tid; k < n; k += g.nt) {
            const int i = L.dy.q(k), j = k - i * L.NY;
            L.x[k] = ((i + j) & 1) == 0 ? L.w[k] * L.b[k] : 0.f;
        }
        g.sync();
        for (int h = 1; h < 2 * L.nu; ++h) b_half_sweep(g, L, h & 1);
        const int nc = Q.NX * Q.NY;
        for (int kc = g.tid; kc < nc; kc += g.nt) {
            const int Ic = Q.dy.q(kc), Jc = kc - Ic * Q.NY;
            float s = 0.f;
            for (int di = 0; di < 2; ++di) {
                const int i = 2 * Ic + di;
                if (i >= L.NX) continue;
                for (int dj = 0; dj < 2; ++dj) {
                    const int j = 2 * Jc + dj;
                    if (j >= L.NY) continue;
                    const int k = i * L.NY + j;
                    if (L.iso[k]) continue;
                    s += L.b[k] - row_lap(L.c, n, L.x, L.NX, L.NY, k, i, j);
                }
            }
            Q.b[kc] = s;
        }
        g.sync();
    }
    {
        const BLvl& C = I.lv[Lc];
        const int n = C.NX * C.NY;
        if (!inv_bad) {
            const int lane = g.tid & 31, wp = g.tid >> 5;
            for (int i = wp; i < n; i += g.warps()) {
                float s = 0.f;
                for (int j = lane; j < n; j += 32) s = fmaf(inv[i * n + j], C.b[j], s);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(kFull, s, o);
                if (lane == 0) C.x[i] = s;
            }
            g.sync();
        } else {   // Jacobi sweeps (the inverse failed)
            for (int k = g.tid; k < n; k += g.nt) C.x[k] = C.w[k] * C.b[k];
            g.sync();
            for (int sw = 1; sw < kBCoarseFallbackSweeps; ++sw) {
                float xn[2] = {0.f, 0.f};
                int q = 0;
                for (int k = g.tid; k < n; k += g.nt, ++q) {
                    const int i = C.dy.q(k), j = k - i * C.NY;
                    xn[q & 1] = C.x[k] + C.w[k] * (C.b[k] - row_lap(C.c, n, C.x, C.NX, C.NY, k, i, j));
                }
                g.sync();
                q = 0;
                for (int k = g.tid; k < n; k += g.nt, ++q) C.x[k] = xn[q & 1];
                g.sync();
            }
        }
    }
    for (int l = Lc - 1; l >= 0; --l) {
        const BLvl& L = I.lv[l];
        const BLvl& Q = I.lv[l + 1];
        const int n = L.NX * L.NY;
        for (int k = g.tid; k < n; k += g.nt) {
            if (L.iso[k]) continue;
            const int i = L.dy.q(k), j = k - i * L.NY;
            L.x[k] = fmaf(L.alpha, Q.x[(i >> 1) * Q.NY + (j >> 1)], L.x[k]);
        }
        g.sync();
        for (int h = 1; h <= 2 * L.nu; ++h) b_half_sweep(g, L, h & 1);
    }
}

// multigrid-preconditioned CG on the FP32 p' rows: A d = r from d = 0 to ||r_k|| <= eps_in ||r_0||
// (r is overwritten); inner products of the FP32 vectors in double-float accumulation (exact
// products, about 48-bit sums), the scalars in FP64.  Returns the iterations, *status.
__device__ __noinline__ int b_pcg(const Grp& g, const BInst& I, double eps_in, const float* inv, int inv_bad, int* status) {
    const BLvl& L0 = I.lv[0];
    const int NX = L0.NX, NY = L0.NY, n = NX * NY;
    const float* c = L0.c;
    float* r = I.cr;
    float* z = I.cz;
    float* p = I.cpv;
    float* q = I.cq;
    float* d = I.cd;
    double s1[1];
    Acc<float> a1[1];
    for (int k = g.tid; k < n; k += g.nt) {
        d[k] = 0.f;
        a1[0].add(r[k], r[k]);
    }
    bsum_df<1>(g, a1, s1);
    const double rr0 = s1[0];
    *status = KC_OK;
    if (rr0 == 0.0) return 0;
    const double stop2 = eps_in * eps_in * rr0;
    b_vcycle(g, I, inv, inv_bad);
    a1[0] = Acc<float>{};
    for (int k = g.tid; k < n; k += g.nt) {
        const float zk = z[k];
        p[k] = zk;
        a1[0].add(r[k], zk);
    }
    bsum_df<1>(g, a1, s1);
    double rho = s1[0];
    int it = 0;
    *status = KC_MAXITER;
    while (it < kBMaxCg) {
        if (!(rho > 0.0)) {   // (r, M r) <= 0: M is not positive definite
            *status = isfinite(rho) ? KC_BREAKDOWN_RHO : KC_NONFINITE;
            break;
        }
        a1[0] = Acc<float>{};
        for (int k0 = g.tid; k0 < n; k0 += g.nt * 2) {
            float y[2], pk[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int k = k0 + u * g.nt;
                if (k < n) {
                    const int i = L0.dy.q(k), j = k - i * NY;
                    y[u] = row_lap(c, n, p, NX, NY, k, i, j);
                    pk[u] = p[k];
                }
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int k = k0 + u * g.nt;
                if (k < n) {
                    q[k] = y[u];
                    a1[0].add(pk[u], y[u]);
                }
            }
        }
        bsum_df<1>(g, a1, s1);
        const double pq = s1[0];
        if (!(pq > 0.0)) {
            *status = isfinite(pq) ? KC_BREAKDOWN_RHO : KC_NONFINITE;
            break;
        }
        const double alpha = rho / pq;
        const float af = (float)alpha;
        a1[0] = Acc<float>{};
        for (int k0 = g.tid; k0 < n; k0 += g.nt * 4) {
            float pk[4], qk[4], rk[4], dk[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int k = k0 + u * g.nt;
                if (k < n) {
                    pk[u] = p[k];
                    qk[u] = q[k];
                    rk[u] = r[k];
                    dk[u] = d[k];
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int k = k0 + u * g.nt;
                if (k < n) {
                    d[k] = fmaf(af, pk[u], dk[u]);
                    const float rn = fmaf(-af, qk[u], rk[u]);
                    r[k] = rn;
                    a1[0].add(rn, rn);
                }
            }
        }
        bsum_df<1>(g, a1, s1);
        const double rr = s1[0];
        ++it;
        if (!isfinite(rr)) {
            *status = KC_NONFINITE;
            break;
        }
        if (rr <= stop2) {
            *status = KC_OK;
            break;
        }
        b_vcycle(g, I, inv, inv_bad);
        a1[0] = Acc<float>{};
        for (int k = g.tid; k < n; k += g.nt) a1[0].add(r[k], z[k]);
        bsum_df<1>(g, a1, s1);
        const float beta = (float)(s1[0] / rho);
        rho = s1[0];
        for (int k0 = g.tid; k0 < n; k0 += g.nt * 4) {
            float pk[4], zk[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int k = k0 + u * g.nt;
                if (k < n) {
                    pk[u] = p[k];
                    zk[u] = z[k];
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int k = k0 + u * g.nt;
                if (k < n) p[k] = fmaf(beta, pk[u], zk[u]);
            }
        }
        g.sync();
    }
    return it;
}

// p' = 0, then FP32 CG passes on the FP64 residual until ||b - A p'|| / ||b|| < eps
__device__ __noinline__ void b_pcorr_solve(const Grp& g, const BInst& I, float* inv, int* inv_bad_s, long long* iters, int* status_out) {
    const Dims D = dims_of(I.P);
    const int NX = D.nx + 2, NY = D.NYp, n = NX * NY;
    double* x = I.pc;
    for (int k = g.tid; k < n; k += g.nt) x[k] = 0.0;
    b_mg_setup(g, I, inv, inv_bad_s);
    const int inv_bad = *inv_bad_s;
    Refine R;
    int status = KC_MAXITER;
    long long total = 0;
    for (int it = 0; it <= kBMaxRefine; ++it) {
        double s[2];
        b_resid64(g, I.cp, I.bp, x, I.cr, NX, NY, I.dp, s);
        bool undo = false;
        if (R.check(it, s, &status, &undo)) {
            if (undo) {
                for (int k = g.tid; k < n; k += g.nt) x[k] -= (double)I.cd[k];
                g.sync();
            }
            break;
        }
        if (R.bb == 0.0 || R.rel < I.eps) {
            status = KC_OK;
            break;
        }
        if (R.rel >= 0.9 * R.best) {
            if (++R.stalls >= 2) {
                status = KC_STALL;
                break;
            }
        } else {
            R.stalls = 0;
        }
        R.best = fmin(R.best, R.rel);
        if (it == kBMaxRefine) break;
        int st = KC_OK;
        const int k_it = b_pcg(g, I, fmax(I.eps_inner_p, 0.5 * I.eps / R.rel), inv, inv_bad, &st);
        total += k_it;
        int bad = 0;
        for (int k = g.tid; k < n; k += g.nt) bad |= !isfinite(I.cd[k]);
        bad = g.any(bad);
        if (!bad)
            for (int k = g.tid; k < n; k += g.nt) x[k] += (double)I.cd[k];
        g.sync();   // the next residual reads x's neighbours
        R.applied = !bad;
        if ((st != KC_OK && k_it == 0) || bad) {
            status = bad ? KC_NONFINITE : st;
            break;
        }
    }
    g.sync();
    *iters += total;
    *status_out = status;
}

// ---- stage 6: corrections (the channel branch of k_correct) ----------------------
__device__ __noinline__ void b_correct(const Grp& g, const BInst& I) {
    const kc_phys& P = I.P;
    const Dims D = dims_of(P);
    const Solid S{I.solid, D.NYp};
    const int nx = D.nx, ny = D.ny;
    const double au = P.alpha_u, ap = P.alpha_p, dx = P.dx, dy = P.dy;
    const double* pc = I.pc;
#define BPC_(a, bb) pc[(long long)(a) * D.NYp + (bb)]
    {
        const int NY = D.NYu, n = (nx + 3) * NY;
        for (int k = g.tid; k < n; k += g.nt) {
            const int i = I.du.q(k), j = k - i * NY;
            if (unk_u(P, S, i, j)) {
                I.u[k] = I.u[k] + au * (BPC_(i - 1, j) - BPC_(i, j)) * dy / I.cu[k];
            } else if (i == nx + 1 && j >= 1 && j <= ny && unk_u(P, S, nx, j)) {
                I.u[k] = I.u[k] + au * (BPC_(nx, j) - BPC_(nx + 1, j)) * dy / I.cu[(long long)nx * D.NYu + j];
            }
        }
    }
    {
        const int NY = D.NYv, n = (nx + 2) * NY;
        for (int k = g.tid; k < n; k += g.nt) {
            const int i = I.dv.q(k), j = k - i * NY;
            if (unk_v(P, S, i, j)) I.v[k] = I.v[k] + au * (BPC_(i, j - 1) - BPC_(i, j)) * dx / I.cv[k];
        }
    }
    {
        const int NY = D.NYp, n = (nx + 2) * NY;
        for (int k = g.tid; k < n; k += g.nt) {
            const int i = I.dp.q(k), j = k - i * NY;
            if (i >= 1 && i <= nx && j >= 1 && j <= ny && !S.cell(i, j)) I.p[k] = I.p[k] + ap * pc[k];
        }
    }
#undef BPC_
    g.sync();
}

// ---- one instance's time steps --------------------------------------------------
__device__ __noinline__ void b_run(const Grp& g, const BInst& I, int steps, float* inv, int* inv_bad) {
    const Dims D = dims_of(I.P);
    kc_channel_stats tot{};
    kc_channel_stats S{};
    for (int step = 0; step < steps; ++step) {
        S = kc_channel_stats{};
        double mass = 0.0;
        for (int outer = 0; outer < I.max_outer; ++outer) {
            b_assemble_momentum(g, I);
            int su = KC_OK, sv = KC_OK, sp = KC_OK;
            b_gs_refined(g, I.cu, I.bu, I.cu32, I.um, D.nx + 3, D.NYu, I.du, I.dhu, I, &S.it_u, &S.fallbacks, &su);
            b_gs_refined(g, I.cv, I.bv, I.cv32, I.vm, D.nx + 2, D.NYv, I.dv, I.dhv, I, &S.it_v, &S.fallbacks, &sv);
            b_relax_outlet(g, I);
            mass = b_assemble_pcorr(g, I);
            b_pcorr_solve(g, I, inv, inv_bad, &S.it_p, &sp);
            if (sp != KC_OK && sp != KC_NONFINITE) {
                // the multigrid CG stalled: the refined BiCGSTAB from p' = 0 takes over (the native step
                // falls back to the plain FP64 BiCGSTAB here; on one SM that is too slow to use)
                ++S.fallbacks;
                const int NXp = D.nx + 2, np = NXp * D.NYp;
                for (int k = g.tid; k < np; k += g.nt) I.pc[k] = 0.0;
                g.sync();
                b_bicg_refined(g, I, true, I.cp, I.bp, I.cp32, I.pc, NXp, D.NYp, I.dp, 50ll * np, &S.it_p, &sp);
            }
            b_correct(g, I);
            S.outer += 1;
            const bool nonfinite = su == KC_NONFINITE || sv == KC_NONFINITE || sp == KC_NONFINITE;
            if (nonfinite) S.status = KC_NONFINITE;
            else if ((su != KC_OK || sv != KC_OK || sp != KC_OK) && S.status == KC_OK) S.status = KC_MAXITER;
            S.mass = mass;
            if (nonfinite || !isfinite(mass)) {
                S.status = KC_NONFINITE;
                break;
            }
            if (mass <= I.mass_tol) break;
        }
        {   // time_forward
            const int nu = (D.nx + 3) * D.NYu, nv = (D.nx + 2) * D.NYv;
            for (int k = g.tid; k < nu; k += g.nt) I.u0[k] = I.u[k];
            for (int k = g.tid; k < nv; k += g.nt) I.v0[k] = I.v[k];
            g.sync();
        }
        tot.outer += S.outer;
        tot.fallbacks += S.fallbacks;
        tot.it_u += S.it_u;
        tot.it_v += S.it_v;
        tot.it_p += S.it_p;
        tot.mass = fmax(tot.mass, S.mass);
        if (S.status != KC_OK && tot.status == KC_OK) tot.status = S.status;
        if (S.status == KC_NONFINITE) break;
    }
    if (g.tid == 0) {
        *I.last = S;
        *I.total = tot;
    }
}

// ---- the kernel: block b runs the instances slots[first_b .. first_b + count_b) ------
// (one of 1024 threads, or up to four of 256), each on its own threads and barrier
__global__ void __launch_bounds__(kBBlock, 1)
    k_batch_steps(const BInst* __restrict__ insts, const int* __restrict__ slots, const int2* __restrict__ blocks,
                  int steps) {
    extern __shared__ __align__(16) float b_dyn[];   // the coarsest inverse of each instance of the block
    __shared__ int inv_bad[kBGroups];
    const int2 bl = blocks[blockIdx.x];
    int base = 0;
    for (int q = 0; q < bl.y; ++q) {
        const int id = slots[bl.x + q];
        const int nt = insts[id].nt;
        if ((int)threadIdx.x < base + nt) {
            const Grp g{(int)threadIdx.x - base, nt, q};
            b_run(g, insts[id], steps, b_dyn + q * kBCoarse * kBCoarse, &inv_bad[q]);
            return;
        }
        base += nt;
    }
}

}  // namespace
}  // namespace kc

using namespace kc;

namespace {

struct BSizes {
    long long nu, nv, np;
    int levels;
    int NX[kBLevels], NY[kBLevels];
};
BSizes sizes_of(const kc_channel* c) {
    BSizes z{};
    const int nx = c->phys.nx, ny = c->phys.ny;
    z.nu = (long long)(nx + 3) * (ny + 2);
    z.nv = (long long)(nx + 2) * (ny + 3);
    z.np = (long long)(nx + 2) * (ny + 2);
    z.NX[0] = nx + 2;
    z.NY[0] = ny + 2;
    int L = 0;
    while (L + 1 < kBLevels && (long long)z.NX[L] * z.NY[L] > kBCoarse) {
        z.NX[L + 1] = (z.NX[L] + 1) / 2;
        z.NY[L + 1] = (z.NY[L] + 1) / 2;
        ++L;
    }
    z.levels = L + 1;
    return z;
}
// bytes of one instance's scratch: Gauss-Seidel weights, FP32 residual and correction over the
// larger momentum grid; CG r, z, p, q, d; per level >= 1 five coefficient planes, b, x, w and the
// flags; level 0's w and flags
size_t inst_bytes(const BSizes& z) {
    const long long nm = std::max(z.nu, z.nv);
    size_t o = 8 * align256((size_t)nm * 4) + 5 * align256((size_t)z.np * 4);
    o += align256((size_t)z.np * 4) + align256((size_t)z.np);
    for (int l = 1; l < z.levels; ++l) {
        const size_t n = (size_t)z.NX[l] * z.NY[l];
        o += align256(5 * n * 4) + 3 * align256(n * 4) + align256(n);
    }
    return o;
}
// descriptors, the two statistics arrays, the instance order and the block table
size_t head_bytes(int n) {
    return align256((size_t)n * sizeof(BInst)) + 2 * align256((size_t)n * sizeof(kc_channel_stats)) +
           align256((size_t)n * sizeof(int)) + align256((size_t)n * sizeof(int2));
}
// threads of an instance: a whole block for the large ones, a quarter block for the rest -- a
// function of the instance alone, so an instance computes the same in any batch
int inst_threads(const kc_channel* c) {
    return (long long)(c->phys.nx + 2) * (c->phys.ny + 2) >= kBBigCells ? kBBlock : kBBlock / kBGroups;
}

int check_channel(const kc_channel* c, int k) {
    if (!c) return set_error("kc_channel_batch_fused: instance %d is null", k), KC_ERR_ARG;
    if (c->phys.mode != KC_MODE_CHANNEL)
        return set_error("kc_channel_batch_fused: instance %d: phys.mode must be KC_MODE_CHANNEL", k), KC_ERR_ARG;
    if (c->precision != KC_F32)
        return set_error("kc_channel_batch_fused: instance %d: the batched launch runs the mixed path (KC_F32)", k),
               KC_ERR_ARG;
    if (c->phys.nx < 2 || c->phys.ny < 2 || (long long)(c->phys.nx + 3) * (c->phys.ny + 3) >= (1ll << 22))
        return set_error("kc_channel_batch_fused: instance %d: grid %d x %d outside [2, ...] and 4M cells", k,
                         c->phys.nx, c->phys.ny),
               KC_ERR_ARG;
    // exact row indices by multiply-high need cells x row length < 2^32 on every grid
    if ((long long)(c->phys.nx + 3) * (c->phys.ny + 3) * (c->phys.ny + 3) >= (1ll << 32))
        return set_error("kc_channel_batch_fused: instance %d: grid %d x %d too large", k, c->phys.nx, c->phys.ny),
               KC_ERR_UNSUPPORTED;
    const BSizes z = sizes_of(c);
    if ((long long)z.NX[z.levels - 1] * z.NY[z.levels - 1] > kBCoarse)
        return set_error("kc_channel_batch_fused: instance %d: grid %d x %d does not coarsen to %d cells in %d levels",
                         k, c->phys.nx, c->phys.ny, kBCoarse, kBLevels),
               KC_ERR_UNSUPPORTED;
    const void* need[] = {c->u, c->v, c->p, c->u0, c->v0, c->pcor, c->u_mid, c->v_mid, c->solid, c->coef_u,
                          c->b_u, c->coef_v, c->b_v, c->coef_p, c->b_p, c->coef_u32, c->b_u32, c->coef_v32,
                          c->b_v32, c->coef_p32, c->b_p32};
    for (const void* q : need)
        if (!q) return set_error("kc_channel_batch_fused: instance %d: a field or system buffer is null", k), KC_ERR_ARG;
    return KC_OK;
}

}  // namespace

extern "C" {

size_t kc_channel_batch_fused_ws_bytes(const kc_channel* const* chs, int n) {
    if (!chs || n < 1) return 0;
    size_t total = head_bytes(n);
    for (int k = 0; k < n; ++k) {
        if (!chs[k]) return 0;
        total += inst_bytes(sizes_of(chs[k]));
    }
    return total;
}

int kc_channel_batch_fused(const kc_channel* const* chs, int n, int steps, void* ws, size_t ws_bytes,
                           kc_channel_stats* last, kc_channel_stats* total, void* stream) {
    if (!chs || n < 0 || steps < 0) return set_error("kc_channel_batch_fused: bad arguments"), KC_ERR_ARG;
    if (n == 0 || steps == 0) return KC_OK;
    for (int k = 0; k < n; ++k) {
        const int rc = check_channel(chs[k], k);
        if (rc) return rc;
    }
    const size_t need = kc_channel_batch_fused_ws_bytes(chs, n);
    if (!ws || ws_bytes < need || ((uintptr_t)ws & 255))
        return set_error("kc_channel_batch_fused: workspace %zu bytes (256-aligned) < required %zu", ws_bytes, need),
               KC_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    char* base = (char*)ws;
    BInst* d_inst = (BInst*)base;
    kc_channel_stats* d_last = (kc_channel_stats*)(base + align256((size_t)n * sizeof(BInst)));
    kc_channel_stats* d_total =
        (kc_channel_stats*)((char*)d_last + align256((size_t)n * sizeof(kc_channel_stats)));
    int* d_slots = (int*)((char*)d_total + align256((size_t)n * sizeof(kc_channel_stats)));
    int2* d_blocks = (int2*)((char*)d_slots + align256((size_t)n * sizeof(int)));
    char* o = base + head_bytes(n);
    std::vector<BInst> h(n);
    for (int k = 0; k < n; ++k) {
        const kc_channel* c = chs[k];
        const BSizes z = sizes_of(c);
        BInst& I = h[k];
        memset(&I, 0, sizeof(BInst));
        I.P = c->phys;
        I.K = consts_of(c->phys);
        I.max_outer = c->max_outer;
        I.mass_tol = c->mass_tol;
        I.eps = c->eps;
        I.eps_inner_p = c->eps_inner_p > 0 ? c->eps_inner_p : 1e-4;
        I.u = c->u;
        I.v = c->v;
        I.p = c->p;
        I.u0 = c->u0;
        I.v0 = c->v0;
        I.pc = c->pcor;
        I.um = c->u_mid;
        I.vm = c->v_mid;
        I.solid = c->solid;
        I.cu = c->coef_u;
        I.bu = c->b_u;
        I.cv = c->coef_v;
        I.bv = c->b_v;
        I.cp = c->coef_p;
        I.bp = c->b_p;
        I.cu32 = c->coef_u32;
        I.bu32 = c->b_u32;
        I.cv32 = c->coef_v32;
        I.bv32 = c->b_v32;
        I.cp32 = c->coef_p32;
        I.bp32 = c->b_p32;
        const long long nm = std::max(z.nu, z.nv);
        auto take = [&](size_t bytes) {
            char* q = o;
            o += align256(bytes);
            return q;
        };
        I.gw = (float*)take((size_t)nm * 4);
        I.r32 = (float*)take((size_t)nm * 4);
        I.d32 = (float*)take((size_t)nm * 4);
        for (int q = 0; q < 5; ++q) I.bt[q] = (float*)take((size_t)nm * 4);
        I.eps_inner = c->eps_inner > 0 ? c->eps_inner : 1e-3;
        I.cr = (float*)take((size_t)z.np * 4);
        I.cz = (float*)take((size_t)z.np * 4);
        I.cpv = (float*)take((size_t)z.np * 4);
        I.cq = (float*)take((size_t)z.np * 4);
        I.cd = (float*)take((size_t)z.np * 4);
        I.levels = z.levels;
        const kc_mg_opts& mo = c->mg_opts;
        for (int l = 0; l < z.levels; ++l) {
            BLvl& L = I.lv[l];
            L.NX = z.NX[l];
            L.NY = z.NY[l];
            L.dy = div_of(L.NY);
            L.dh = div_of((L.NY + 1) / 2);
            const size_t nl = (size_t)L.NX * L.NY;
            if (l == 0) {
                L.c = c->coef_p32;
                L.b = I.cr;
                L.x = I.cz;
                L.w = (float*)take(nl * 4);
                L.iso = (unsigned char*)take(nl);
            } else {
                L.c = (float*)take(5 * nl * 4);
                L.b = (float*)take(nl * 4);
                L.x = (float*)take(nl * 4);
                L.w = (float*)take(nl * 4);
                L.iso = (unsigned char*)take(nl);
            }
            const int li = std::min(l, KC_MG_MAX_LEVELS - 1);
            L.omega = mo.omega[li] != 0.f ? mo.omega[li] : (l == 0 ? 1.0f : 1.5f);
            L.alpha = mo.alpha[li] != 0.f ? mo.alpha[li] : (l == 0 ? 1.9f : 2.0f);
            L.nu = l == 0 ? std::max(1, mo.nu_pre) : std::max(1, mo.nu_coarse);
        }
        I.du = div_of(c->phys.ny + 2);
        I.dv = div_of(c->phys.ny + 3);
        I.dp = div_of(c->phys.ny + 2);
        I.dhu = div_of((c->phys.ny + 3) / 2);
        I.dhv = div_of((c->phys.ny + 4) / 2);
        I.nt = inst_threads(c);
        I.last = d_last + k;
        I.total = d_total + k;
    }
    // blocks: each large instance alone, then the others four to a block, largest first
    std::vector<int> order(n);
    for (int k = 0; k < n; ++k) order[k] = k;
    auto cells = [&](int k) { return (long long)(chs[k]->phys.nx + 2) * (chs[k]->phys.ny + 2); };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        if (h[a].nt != h[b].nt) return h[a].nt > h[b].nt;
        return cells(a) > cells(b);
    });
    std::vector<int2> blocks;
    for (int q = 0; q < n;) {
        int used = 0, first = q;
        while (q < n && used + h[order[q]].nt <= kBBlock && q - first < kBGroups) used += h[order[q++]].nt;
        blocks.push_back(make_int2(first, q - first));
    }
    if ((size_t)(o - base) > ws_bytes) return set_error("kc_channel_batch_fused: workspace layout overflow"), KC_ERR_WORKSPACE;
    KC_CUDA(cudaMemcpyAsync(d_inst, h.data(), (size_t)n * sizeof(BInst), cudaMemcpyHostToDevice, s));
    KC_CUDA(cudaMemcpyAsync(d_slots, order.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, s));
    KC_CUDA(cudaMemcpyAsync(d_blocks, blocks.data(), blocks.size() * sizeof(int2), cudaMemcpyHostToDevice, s));
    constexpr size_t dyn = (size_t)kBGroups * kBCoarse * kBCoarse * sizeof(float);
    {   // the dynamic shared memory limit, once per device
        static std::mutex mu;
        static bool set[64] = {false};
        int dev = 0;
        KC_CUDA(cudaGetDevice(&dev));
        if (dev < 0 || dev >= 64) return set_error("kc_channel_batch_fused: device index %d", dev), KC_ERR_ARG;
        std::lock_guard<std::mutex> lk(mu);
        if (!set[dev]) {
            KC_CUDA(cudaFuncSetAttribute(k_batch_steps, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
            set[dev] = true;
        }
    }
    k_batch_steps<<<(unsigned)blocks.size(), kBBlock, dyn, s>>>(d_inst, d_slots, d_blocks, steps);
    KC_LAUNCH_CHECK("k_batch_steps");
    std::vector<kc_channel_stats> hs(2 * (size_t)n);
    KC_CUDA(cudaMemcpyAsync(hs.data(), d_last, (size_t)n * sizeof(kc_channel_stats), cudaMemcpyDeviceToHost, s));
    KC_CUDA(cudaMemcpyAsync(hs.data() + n, d_total, (size_t)n * sizeof(kc_channel_stats), cudaMemcpyDeviceToHost, s));
    KC_CUDA(cudaStreamSynchronize(s));
    if (last) memcpy(last, hs.data(), (size_t)n * sizeof(kc_channel_stats));
    if (total) memcpy(total, hs.data() + n, (size_t)n * sizeof(kc_channel_stats));
    return KC_OK;
}

}  // extern "C"
