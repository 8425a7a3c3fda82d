// Aggregation multigrid V-cycle for 2-D 5-point operators (FP32), used as the
// preconditioner of the mixed-precision pressure-correction solve (CG, or
// right-preconditioned BiCGSTAB).
//
// The reference has no preconditioner beyond Jacobi (karman_taichi.py:398-399,
// 418-419) and names multigrid as its missing next step (README.md:31).  This
// is a GB300 implementation of that step:
//   * coarsening: 2x2 aggregates, Galerkin coarse operator A_c = P^T A P with
//     piecewise-constant P, kept in Laplacian form [row sum, links] so no
//     coarse coefficient is the difference of large numbers (k_mg_coarsen);
//   * rows without off-diagonal links (halo zero rows, identity rows of
//     blocked cells) are "isolated": solved pointwise, never aggregated, and
//     links into them are folded into the row sum -- so a Dirichlet ghost
//     keeps acting as Dirichlet on coarse levels and unit identity rows do not
//     swamp the ~1e-3-scaled pressure rows;
//   * smoother: red-black Gauss-Seidel with a per-level weight omega_l
//     (isolated rows use the exact pointwise solve); coarse corrections are scaled by
//     alpha_l (aggregation multigrid needs over-correction).  The post-smoother
//     visits the colours in the reverse order of the pre-smoother and the
//     coarsest solve is a fixed number of Jacobi sweeps, so for a symmetric
//     operator the V-cycle is a symmetric linear operator (usable by CG);
//   * coarsest level: exact (<= kCoarseDirectMax cells, dense inverse formed at
//     setup, coarsest_sweeps = 0) or Jacobi sweeps in shared memory by one
//     block (<= kCoarsestMax cells, coarsest_sweeps > 0).
// Level 0 is the caller's system (n = NX*NY, far stride NY); levels >= 1 live
// in the multigrid workspace.  The cycle treats every level as a 2-D
// [NX][NY] grid with zero values outside it (a link across the end of a row
// of the flat stencil is a link to a zero cell).  All kernels take an optional "done" word and
// return at once when it is set, so a solver that converged mid-chunk skips
// the remaining preconditioner work of a captured graph.
#include "kc_common.cuh"
#include "kc_mg.h"
#include <algorithm>
#include <mutex>

namespace kc {

constexpr int kCoarsestMax = 1024;      // coarsest level of the Jacobi variant (cells)
constexpr int kCoarseDirectMax = 128;   // coarsest level of the direct variant (cells)
constexpr int kCoarseFallbackSweeps = 64;

__device__ __forceinline__ bool mg_done(const int* done) { return done && __ldcg(done) != 0; }

// ---- setup ---------------------------------------------------------------------
// Level-0 scaled inverse diagonal and isolation flags from the caller's FP32
// coefficients (component stride cs, element stride es; standard or
// Laplacian form: the diagonal is aP, or rs - sum of links).
__global__ void k_mg_diag0(const float* __restrict__ c, long long cs, long long es, int lap, int n, float omega,
                           float* __restrict__ winv, unsigned char* __restrict__ iso) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const long long e = (long long)k * es;
        const float w = c[cs + e], ea = c[2 * cs + e], no = c[3 * cs + e], so = c[4 * cs + e];
        const float d = lap ? c[e] - (w + ea + no + so) : c[e];
        const bool linked = w != 0.f || ea != 0.f || no != 0.f || so != 0.f;
        iso[k] = linked ? 0 : 1;
        winv[k] = d == 0.f ? 0.f : (linked ? omega / d : 1.f / d);
    }
}

// Coarse operator of level l+1 from level l, in Laplacian form
// [rs, aW, aE, aN, aS].  Galerkin with piecewise-constant P: the coarse row
// sum is the sum of the fine row sums, coarse links are the sums of the fine
// links that cross into a neighbouring aggregate, and links inside an
// aggregate cancel exactly.  A link into an isolated cell (or outside the
// grid) sees a zero value there, so it is folded into the row sum.  Nothing
// is subtracted from anything: FP32 storage cannot perturb the row sums.
__global__ void k_mg_coarsen(const float* __restrict__ cf, long long cs, long long es, int lapf,
                             const unsigned char* __restrict__ isof, int NXf, int NYf, float* __restrict__ cc, int NXc,
                             int NYc, float omega, float* __restrict__ winv, unsigned char* __restrict__ isoc) {
    const int J = blockIdx.x * blockDim.x + threadIdx.x;
    const int I = blockIdx.y;
    if (J >= NYc || I >= NXc) return;
    float rs = 0.f, aW = 0.f, aE = 0.f, aN = 0.f, aS = 0.f;
    for (int di = 0; di < 2; ++di) {
        const int i = 2 * I + di;
        if (i >= NXf) continue;
        for (int dj = 0; dj < 2; ++dj) {
            const int j = 2 * J + dj;
            if (j >= NYf) continue;
            const int k = i * NYf + j;
            if (isof[k]) continue;
            const long long e = (long long)k * es;
            const float w = cf[cs + e], ea = cf[2 * cs + e], no = cf[3 * cs + e], so = cf[4 * cs + e];
            float r = lapf ? cf[e] : cf[e] + (w + ea + no + so);
            if (i - 1 < 0 || isof[k - NYf]) r -= w;
            else if (di == 0) aW += w;
            if (i + 1 >= NXf || isof[k + NYf]) r -= ea;
            else if (di == 1) aE += ea;
            if (j + 1 >= NYf || isof[k + 1]) r -= no;
            else if (dj == 1) aN += no;
            if (j - 1 < 0 || isof[k - 1]) r -= so;
            else if (dj == 0) aS += so;
            rs += r;
        }
    }
    const int kc = I * NYc + J;
    const long long nc = (long long)NXc * NYc;
    cc[kc] = rs;
    cc[nc + kc] = aW;
    cc[2 * nc + kc] = aE;
    cc[3 * nc + kc] = aN;
    cc[4 * nc + kc] = aS;
    const bool linked = aW != 0.f || aE != 0.f || aN != 0.f || aS != 0.f;
    const float d = rs - (aW + aE + aN + aS);
    isoc[kc] = linked ? 0 : 1;
    winv[kc] = d == 0.f ? 0.f : (linked ? omega / d : 1.f / d);
}

// ---- cycle kernels -----------------------------------------------------------------
struct Lvl {
    const float* c;     // coefficients
    long long cs, es;
    int NX, NY;
    int lap;            // Laplacian form (component 0 = row sum)
    const float* winv;
    const unsigned char* iso;
};

__device__ __forceinline__ float mg_Ax(const Lvl& L, const float* __restrict__ x, int k) {
    const long long e = (long long)k * L.es;
    const int n = L.NX * L.NY;
    const int j = k % L.NY;
    const float xk = x[k];
    const float xw = k >= L.NY ? x[k - L.NY] : 0.f, xe = k + L.NY < n ? x[k + L.NY] : 0.f;
    const float xn = j + 1 < L.NY ? x[k + 1] : 0.f, xs = j >= 1 ? x[k - 1] : 0.f;
    float y = __ldg(L.c + e) * xk;
    if (L.lap) {
        y = fmaf(__ldg(L.c + L.cs + e), xw - xk, y);
        y = fmaf(__ldg(L.c + 2 * L.cs + e), xe - xk, y);
        y = fmaf(__ldg(L.c + 3 * L.cs + e), xn - xk, y);
        y = fmaf(__ldg(L.c + 4 * L.cs + e), xs - xk, y);
    } else {
        y = fmaf(__ldg(L.c + L.cs + e), xw, y);
        y = fmaf(__ldg(L.c + 2 * L.cs + e), xe, y);
        y = fmaf(__ldg(L.c + 3 * L.cs + e), xn, y);
        y = fmaf(__ldg(L.c + 4 * L.cs + e), xs, y);
    }
    return y;
}

// Red-black Gauss-Seidel half-sweep on cells with (i + j) % 2 == color:
// x += W (b - A x).  In place: a cell of one colour reads only the other.
__global__ void k_mg_rbgs(Lvl L, const float* __restrict__ b, float* __restrict__ x, int color, const int* done) {
    if (mg_done(done)) return;
    const int n = L.NX * L.NY;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = k / L.NY, j = k - i * L.NY;
        if (((i + j) & 1) != color) continue;
        const float r = __ldg(b + k) - mg_Ax(L, x, k);
        x[k] = fmaf(__ldg(L.winv + k), r, x[k]);
    }
}

// first half-sweep from x = 0: red cells x = W b, black cells 0
__global__ void k_mg_first(Lvl L, const float* __restrict__ b, float* __restrict__ x, const int* done) {
    if (mg_done(done)) return;
    const int n = L.NX * L.NY;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = k / L.NY, j = k - i * L.NY;
        x[k] = ((i + j) & 1) == 0 ? __ldg(L.winv + k) * __ldg(b + k) : 0.f;
    }
}

// b_c(I,J) = sum of the fine residual b - A x over the aggregate's coupled cells
__global__ void k_mg_restrict(Lvl F, const float* __restrict__ b, const float* __restrict__ x, float* __restrict__ bc,
                              int NXc, int NYc, const int* done) {
    if (mg_done(done)) return;
    const int J = blockIdx.x * blockDim.x + threadIdx.x;
    const int I = blockIdx.y;
    if (J >= NYc || I >= NXc) return;
    float s = 0.f;
    for (int di = 0; di < 2; ++di) {
        const int i = 2 * I + di;
        if (i >= F.NX) continue;
        for (int dj = 0; dj < 2; ++dj) {
            const int j = 2 * J + dj;
            if (j >= F.NY) continue;
            const int k = i * F.NY + j;
            if (F.iso[k]) continue;
            s += __ldg(b + k) - mg_Ax(F, x, k);
        }
    }
    bc[I * NYc + J] = s;
}

// x_f += alpha * x_c(aggregate) on coupled fine cells
__global__ void k_mg_prolong(Lvl F, float* __restrict__ x, const float* __restrict__ xc, int NYc, float alpha,
                             const int* done) {
    if (mg_done(done)) return;
    const int n = F.NX * F.NY;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        if (F.iso[k]) continue;
        const int i = k / F.NY, j = k - (k / F.NY) * F.NY;
        x[k] = fmaf(alpha, __ldg(xc + (i >> 1) * NYc + (j >> 1)), x[k]);
    }
}

// ---- coarsest level ------------------------------------------------------------------
// Direct variant (coarsest_sweeps == 0): coarsening stops at <= kCoarseDirectMax
// cells, setup inverts the level's dense operator in place by Gauss-Jordan
// elimination without pivoting (the operator is symmetric positive definite:
// Galerkin coarsening of the symmetric p' operator with its Dirichlet outlet
// folded into the row sums; a zero row -- no coupled child -- gets a unit
// diagonal, its right-hand side is zero), and the cycle applies x = A^-1 b.
// A non-positive or non-finite pivot sets the flag and the cycle falls back
// to kCoarseFallbackSweeps Jacobi sweeps.
// The block is 32 x 32 threads; thread (ty, tx) keeps the entries of rows
// ty + 32a and columns tx + 32c in registers (R x R of them, R = ceil(n / 32)
// chosen at launch), so a
// pivot step is one barrier and a few FMAs per entry: the pivot row and
// column go through shared memory, double-buffered so that step p + 1 may
// write while slow readers still read step p's copy.
constexpr int kGjR = kCoarseDirectMax / 32;

template <int R>
__global__ void __launch_bounds__(1024) k_mg_coarse_inverse(Lvl L, float* __restrict__ inv, int* __restrict__ flag) {
    __shared__ float rowp[2][kCoarseDirectMax], colp[2][kCoarseDirectMax];
    const int n = L.NX * L.NY, NY = L.NY;
    const int tx = threadIdx.x, ty = threadIdx.y;
    float a[R][R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int i = ty + 32 * r;
        float d = 0.f, w = 0.f, ea = 0.f, no = 0.f, so = 0.f;
        if (i < n) {
            const long long ce = (long long)i * L.es;
            const float c0 = L.c[ce];
            w = L.c[L.cs + ce];
            ea = L.c[2 * L.cs + ce];
            no = L.c[3 * L.cs + ce];
            so = L.c[4 * L.cs + ce];
            d = L.lap ? c0 - (((w + ea) + no) + so) : c0;   // out-of-grid neighbours hold zero
            if (w == 0.f && ea == 0.f && no == 0.f && so == 0.f && d == 0.f) d = 1.f;   // no coupled child
        }
        const int jr = i % NY;
#pragma unroll
        for (int c = 0; c < R; ++c) {
            const int j = tx + 32 * c;
            float v = 0.f;
            if (i < n && j < n) {
                if (j == i) v = d;
                else if (j == i - NY) v = w;
                else if (j == i + NY) v = ea;
                else if (j == i + 1 && jr + 1 < NY) v = no;
                else if (j == i - 1 && jr >= 1) v = so;
            }
            a[r][c] = v;
        }
    }
    int bad = 0;
    for (int p = 0; p < n; ++p) {
        const int buf = p & 1, pr = p >> 5, pl = p & 31;
        // the owners publish row p and column p as they stand before the step
        if (ty == pl) {
#pragma unroll
            for (int r = 0; r < R; ++r)
                if (r == pr) {
#pragma unroll
                    for (int c = 0; c < R; ++c) rowp[buf][tx + 32 * c] = a[r][c];
                }
        }
        if (tx == pl) {
#pragma unroll
            for (int c = 0; c < R; ++c)
                if (c == pr) {
#pragma unroll
                    for (int r = 0; r < R; ++r) colp[buf][ty + 32 * r] = a[r][c];
                }
        }
        __syncthreads();
        const float piv = rowp[buf][p];
        if (!(piv > 0.f) || !isfinite(piv)) {   // uniform: every thread reads the same pivot
            bad = 1;
            break;
        }
        const float ip = 1.f / piv;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int i = ty + 32 * r;
            const float ci = colp[buf][i];
#pragma unroll
            for (int c = 0; c < R; ++c) {
                const int j = tx + 32 * c;
                const float sp = j == p ? ip : rowp[buf][j] * ip;   // the scaled pivot row
                a[r][c] = i == p ? sp : (j == p ? -ci * ip : fmaf(-ci, sp, a[r][c]));
            }
        }
    }
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int c = 0; c < R; ++c) {
            const int i = ty + 32 * r, j = tx + 32 * c;
            if (i < n && j < n) inv[i * n + j] = a[r][c];
        }
    if (tx == 0 && ty == 0) *flag = bad;
}

// x = A^-1 b (one warp per row), or Jacobi sweeps when sweeps > 0 or the inverse failed
__global__ void __launch_bounds__(kCoarsestMax) k_mg_coarsest(Lvl L, const float* __restrict__ b,
                                                              float* __restrict__ x, int sweeps,
                                                              const float* __restrict__ inv,
                                                              const int* __restrict__ inv_bad, const int* done) {
    pdl_wait();
    pdl_trigger();   // one block: the next grid may queue up at once
    if (mg_done(done)) return;
    const int n = L.NX * L.NY;
    if (sweeps == 0) {
        if (!__ldcg(inv_bad)) {
            const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5, nw = blockDim.x >> 5;
            for (int i = wp; i < n; i += nw) {
                float sacc = 0.f;
                for (int j = lane; j < n; j += 32) sacc = fmaf(inv[i * n + j], b[j], sacc);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) sacc += __shfl_down_sync(kFull, sacc, o);
                if (lane == 0) x[i] = sacc;
            }
            return;
        }
        sweeps = kCoarseFallbackSweeps;
    }
    __shared__ float xs[2][kCoarsestMax];
    const int k = threadIdx.x;
    float bk = 0.f, w = 0.f, c[5] = {0, 0, 0, 0, 0};
    if (k < n) {
        bk = b[k];
        w = L.winv[k];
        const long long e = (long long)k * L.es;
        for (int q = 0; q < 5; ++q) c[q] = L.c[q * L.cs + e];
        xs[0][k] = w * bk;
    }
    __syncthreads();
    int cur = 0;
    for (int s = 0; s < sweeps; ++s) {
        if (k < n) {
            const float* xv = xs[cur];
            const float xk = xv[k];
            const int j = k % L.NY;
            const float xw = k >= L.NY ? xv[k - L.NY] : 0.f, xe = k + L.NY < n ? xv[k + L.NY] : 0.f;
            const float xn = j + 1 < L.NY ? xv[k + 1] : 0.f, xso = j >= 1 ? xv[k - 1] : 0.f;
            float y = c[0] * xk;
            if (L.lap) y += c[1] * (xw - xk) + c[2] * (xe - xk) + c[3] * (xn - xk) + c[4] * (xso - xk);
            else y += c[1] * xw + c[2] * xe + c[3] * xn + c[4] * xso;
            xs[cur ^ 1][k] = xk + w * (bk - y);
        }
        __syncthreads();
        cur ^= 1;
    }
    if (k < n) x[k] = xs[cur][k];
}

// ---- fused cycle kernels (NU pre- and NU post-sweeps per level) ------------------------
// The grid dependency wait, then (small levels: one wave) the early trigger
// that lets the next grid queue up, then the solver's done flag.
template <bool SMALL>
struct MgGate {
    const int* done;
    __device__ __forceinline__ bool operator()() const {
        pdl_wait();
        if (SMALL) pdl_trigger();
        return !mg_done(done);
    }
};

// early != 0 (levels below 0): the launch before this one is a kernel of the
// cycle, which waits for its own predecessor before it lets this grid start,
// so what launches further back wrote (the setup's weights and coefficients,
// the level's pre-smoothed iterate and right-hand side) is final: the tile
// stages it before the wait, behind the previous grid.
template <int TI, int AJ, int RY, bool STAGED, int NU>
__global__ void __launch_bounds__(AJ * RY) k_mg_down(MgLvl L, const float* __restrict__ b, float* __restrict__ xout,
                                                     float* __restrict__ bc, int NXc, int NYc, const int* done,
                                                     int early) {
    mg_down_tile<TI, AJ, RY, false, MgNoMid, MgOwnNone, STAGED, NU>(
        blockIdx.y * TI, blockIdx.x * mg_tj(AJ, NU), L, b, nullptr, 0.f, MgNoMid{}, MgOwnNone{}, xout, bc, NXc, NYc,
        MgGate<(AJ < kMgAJ0)>{done}, early != 0);
    pdl_trigger();
}

template <int TI, int AJ, int RY, bool STAGED, int NU>
__global__ void __launch_bounds__(AJ * RY) k_mg_up(MgLvl L, const float* __restrict__ xpre,
                                                   const float* __restrict__ xc, int NXc, int NYc, float alpha,
                                                   const float* __restrict__ b, float* __restrict__ xout,
                                                   const int* done, int early) {
    mg_up_tile<TI, AJ, RY, MgOwnNone, STAGED, NU>(blockIdx.y * TI, blockIdx.x * mg_tj(AJ, NU), L, xpre, xc, NXc, NYc,
                                                  alpha, b, MgOwnNone{}, xout, MgGate<(AJ < kMgAJ0)>{done},
                                                  early != 0);
    pdl_trigger();
}

// ---- coarse-level tail: the smallest levels of the fused cycle in one block ------------
// A level of a few hundred cells costs two launches of ~3-5 us each for a few
// microseconds of work: each waits for the previous grid to drain and reloads
// its data.  Here one block runs the levels Ls..Lend (from the first level of
// at most kTailMax cells down to the coarsest) with every array in shared
// memory, phases separated by __syncthreads.  Smoother weights, coefficients
// and the coarsest inverse do not depend on the previous launch: they are
// staged before the grid dependency wait, behind the previous kernel's tail.
// The arithmetic per cell is that of mg_down_tile / mg_up_tile /
// k_mg_coarsest, operation for operation, so the cycle's result is bitwise
// the same as with one launch per level.  (Spreading larger levels over a
// thread-block cluster, rows exchanged through distributed shared memory,
// was measured slower than their launches on GB300: 1.2-2.4 us per
// cluster-barrier phase.)
constexpr int kTailThreads = 1024;
constexpr int kTailMax = 1536;    // levels of at most this many cells run in the tail block
constexpr int kTailArrays = 8;    // per cell: x, b, smoother weight, 5 coefficients

struct TailLevel {
    const float* c;      // Laplacian-form coefficients, 5 planes of NX*NY
    const float* winv;   // smoother weights
    int NX, NY;
    float alpha;         // weight of the coarse correction prolonged into this level
    int nu;              // red-black sweeps before and after the coarse correction
    int so;              // shared-memory offset (floats) of the level's arrays
    unsigned mNY, mHalf; // t / NY and t / ((NY + 1) / 2) by tdiv (exact for t, d < 2^16)
};
struct MgTail {
    TailLevel lv[KC_MG_MAX_LEVELS];
    int Ls, Lend, inv_so;
    const float* b_in;   // right-hand side of level Ls (written by the previous launch)
    float* x_out;        // result of level Ls
    const float* inv;    // dense inverse of the coarsest level
    const int* inv_bad;
};

// m = 0 stands for d = 1 (2^32 does not fit)
__device__ __forceinline__ int tdiv(int t, unsigned m) { return m ? (int)__umulhi((unsigned)t, m) : t; }

// one level in shared memory: cell k = i * NY + j
struct TailArr {
    float* x;
    float* b;
    const float* w;
    const float* c;   // component q of cell k at c[q * n + k]
    int n, NX, NY;
    __device__ __forceinline__ float cq(int q, int k) const { return c[q * n + k]; }
    __device__ __forceinline__ bool linked(int k) const {
        return cq(1, k) != 0.f || cq(2, k) != 0.f || cq(3, k) != 0.f || cq(4, k) != 0.f;
    }
    __device__ __forceinline__ float xa(int i, int j) const {
        return (j < 0 || j >= NY || i < 0 || i >= NX) ? 0.f : x[i * NY + j];
    }
    __device__ __forceinline__ float ax(int k, int i, int j, float xv) const {
        return mg_row(cq(0, k), cq(1, k), cq(2, k), cq(3, k), cq(4, k), 1, xv, xa(i - 1, j), xa(i + 1, j),
                      xa(i, j + 1), xa(i, j - 1));
    }
};
__device__ __forceinline__ TailArr tail_arr(float* sm, const TailLevel& L) {
    float* s = sm + L.so;
    const int n = L.NX * L.NY;
    return TailArr{s, s + n, s + 2 * n, s + 3 * n, n, L.NX, L.NY};
}

// half-sweep x += W (b - A x) over the cells of colour col ((i + j) & 1)
__device__ __forceinline__ void tail_sweep(const TailArr& A, const TailLevel& L, int col) {
    const int half = (A.NY + 1) >> 1;
    const int cnt = A.NX * half;
    for (int e = threadIdx.x; e < cnt; e += kTailThreads) {
        const int i = tdiv(e, L.mHalf), m = e - i * half;
        const int j = 2 * m + ((i + col) & 1);
        if (j >= A.NY) continue;
        const int k = i * A.NY + j;
        const float xv = A.x[k];
        A.x[k] = fmaf(A.w[k], A.b[k] - A.ax(k, i, j, xv), xv);
    }
}

__global__ void __launch_bounds__(kTailThreads, 1) k_mg_tail(MgTail T, const int* done) {
    extern __shared__ __align__(16) float sm[];
    const int tid = threadIdx.x;
    // weights, coefficients and the inverse first: they do not depend on the previous launch
    for (int l = T.Ls; l <= T.Lend; ++l) {
        const TailLevel& L = T.lv[l];
        const TailArr A = tail_arr(sm, L);
        float* w = const_cast<float*>(A.w);
        float* c = const_cast<float*>(A.c);
        for (int k = tid; k < A.n; k += kTailThreads) {
            w[k] = __ldg(L.winv + k);
#pragma unroll
            for (int q = 0; q < 5; ++q) c[q * A.n + k] = __ldg(L.c + q * A.n + k);
        }
    }
    const int nc = T.lv[T.Lend].NX * T.lv[T.Lend].NY;
    float* inv = sm + T.inv_so;
    for (int e = tid; e < nc * nc; e += kTailThreads) inv[e] = __ldg(T.inv + e);
    pdl_wait();
    pdl_trigger();
    if (mg_done(done)) return;
    {
        const TailArr A = tail_arr(sm, T.lv[T.Ls]);
        for (int k = tid; k < A.n; k += kTailThreads) A.b[k] = __ldcg(T.b_in + k);
    }
    __syncthreads();
    // downward: red start, 2 nu - 1 half-sweeps (black, red, ...), restriction
    for (int l = T.Ls; l < T.Lend; ++l) {
        const TailLevel& L = T.lv[l];
        const TailLevel& Q = T.lv[l + 1];
        const TailArr A = tail_arr(sm, L);
        for (int k = tid; k < A.n; k += kTailThreads) {
            const int i = tdiv(k, L.mNY), j = k - i * A.NY;
            A.x[k] = ((i + j) & 1) == 0 ? A.w[k] * A.b[k] : 0.f;
        }
        __syncthreads();
        for (int h = 1; h < 2 * L.nu; ++h) {
            tail_sweep(A, L, h & 1);
            __syncthreads();
        }
        const TailArr B = tail_arr(sm, Q);
        for (int t = tid; t < B.n; t += kTailThreads) {
            const int I = tdiv(t, Q.mNY), J = t - I * B.NY;
            float s = 0.f;
#pragma unroll
            for (int di = 0; di < 2; ++di)
#pragma unroll
                for (int dj = 0; dj < 2; ++dj) {
                    const int i = 2 * I + di, j = 2 * J + dj;
                    if (i >= A.NX || j >= A.NY) continue;
                    const int k = i * A.NY + j;
                    if (!A.linked(k)) continue;
                    s += A.b[k] - A.ax(k, i, j, A.x[k]);
                }
            B.b[t] = s;
        }
        __syncthreads();
    }
    {   // coarsest: x = A^-1 b (one warp per row), or Jacobi sweeps when the inverse failed
        const TailArr A = tail_arr(sm, T.lv[T.Lend]);
        const int n = A.n;
        if (!__ldcg(T.inv_bad)) {
            const int lane = tid & 31, wp = tid >> 5, nw = kTailThreads >> 5;
            for (int i = wp; i < n; i += nw) {
                float sacc = 0.f;
                for (int j = lane; j < n; j += 32) sacc = fmaf(inv[i * n + j], A.b[j], sacc);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) sacc += __shfl_down_sync(kFull, sacc, o);
                if (lane == 0) A.x[i] = sacc;
            }
        } else {
            __shared__ float xs[2][kCoarseDirectMax];
            float bk = 0.f, w = 0.f, c[5] = {0, 0, 0, 0, 0};
            if (tid < n) {
                bk = A.b[tid];
                w = A.w[tid];
                for (int q = 0; q < 5; ++q) c[q] = A.cq(q, tid);
                xs[0][tid] = w * bk;
            }
            __syncthreads();
            int cur = 0;
            for (int s = 0; s < kCoarseFallbackSweeps; ++s) {
                if (tid < n) {
                    const float* xv = xs[cur];
                    const float xk = xv[tid];
                    const int j = tid % A.NY;
                    const float xw = tid >= A.NY ? xv[tid - A.NY] : 0.f, xe = tid + A.NY < n ? xv[tid + A.NY] : 0.f;
                    const float xn = j + 1 < A.NY ? xv[tid + 1] : 0.f, xso = j >= 1 ? xv[tid - 1] : 0.f;
                    float y = c[0] * xk;
                    y += c[1] * (xw - xk) + c[2] * (xe - xk) + c[3] * (xn - xk) + c[4] * (xso - xk);
                    xs[cur ^ 1][tid] = xk + w * (bk - y);
                }
                __syncthreads();
                cur ^= 1;
            }
            if (tid < n) A.x[tid] = xs[cur][tid];
        }
        __syncthreads();
    }
    // upward: prolongation, nu sweeps (black then red half-sweep)
    for (int l = T.Lend - 1; l >= T.Ls; --l) {
        const TailLevel& L = T.lv[l];
        const TailLevel& Q = T.lv[l + 1];
        const TailArr A = tail_arr(sm, L);
        const float* xc = sm + Q.so;
        for (int k = tid; k < A.n; k += kTailThreads) {
            if (!A.linked(k)) continue;
            const int i = tdiv(k, L.mNY), j = k - i * A.NY;
            A.x[k] = fmaf(L.alpha, xc[(i >> 1) * Q.NY + (j >> 1)], A.x[k]);
        }
        __syncthreads();
        for (int h = 1; h <= 2 * L.nu; ++h) {
            tail_sweep(A, L, h & 1);
            __syncthreads();
        }
    }
    const TailArr A = tail_arr(sm, T.lv[T.Ls]);
    for (int k = tid; k < A.n; k += kTailThreads) T.x_out[k] = A.x[k];
}

// large levels use the 64-wide tiles (16 x 60 owned cells at one sweep), small ones the 32-wide
// tiles (8 x 28 at one sweep; more blocks in flight)
static inline bool mg_big(int NX, int NY, const kc_mg_opts* o) {
    return (long long)NX * NY >= (o->big_cells > 0 ? o->big_cells : 200000);
}

// ---- host ----------------------------------------------------------------------------
static int mg_levels(int NX, int NY, const kc_mg_opts* o, int* nx, int* ny) {
    int L = 0;
    nx[0] = NX;
    ny[0] = NY;
    const int maxl = std::max(1, std::min(o ? o->max_levels : KC_MG_MAX_LEVELS, (int)KC_MG_MAX_LEVELS));
    const long long target = (o && o->coarsest_sweeps == 0) ? kCoarseDirectMax : kCoarsestMax;
    while (L + 1 < maxl && (long long)nx[L] * ny[L] > target) {
        nx[L + 1] = (nx[L] + 1) / 2;
        ny[L + 1] = (ny[L] + 1) / 2;
        ++L;
    }
    return L + 1;
}

MgLayout mg_layout(int NX, int NY, const kc_mg_opts* o) {
    MgLayout M{};
    M.levels = mg_levels(NX, NY, o, M.nx, M.ny);
    size_t off = 0;
    for (int l = 0; l < M.levels; ++l) {
        const size_t n = (size_t)M.nx[l] * M.ny[l];
        M.off_winv[l] = off;
        off = align256(off + n * 4);
        M.off_iso[l] = off;
        off = align256(off + n);
        if (l >= 1) {
            M.off_coef[l] = off;
            off = align256(off + 5 * n * 4);
            M.off_b[l] = off;
            off = align256(off + n * 4);
        }
        M.off_x[l] = off;
        off = align256(off + n * 4);
        M.off_t[l] = off;
        off = align256(off + n * 4);
    }
    M.off_inv = off;
    off = align256(off + (size_t)kCoarseDirectMax * kCoarseDirectMax * 4);
    M.off_flag = off;
    off = align256(off + 16);
    M.total = off;
    return M;
}

static Lvl level_of(const MgLayout& M, char* base, int l, const float* c0, long long cs0, long long es0,
                    int lap0) {
    Lvl L;
    const long long n = (long long)M.nx[l] * M.ny[l];
    if (l == 0) {
        L.c = c0;
        L.cs = cs0;
        L.es = es0;
        L.lap = lap0;
    } else {
        L.c = (const float*)(base + M.off_coef[l]);
        L.cs = n;
        L.es = 1;
        L.lap = 1;
    }
    L.NX = M.nx[l];
    L.NY = M.ny[l];
    L.winv = (const float*)(base + M.off_winv[l]);
    L.iso = (const unsigned char*)(base + M.off_iso[l]);
    return L;
}

static MgLvl mg_lvl(const Lvl& L) { return MgLvl{L.c, L.cs, L.es, L.NX, L.NY, L.lap, L.winv, L.iso}; }

// red-black sweeps before and after the coarse correction on level l: nu_pre / nu_post on
// level 0, nu_coarse (<= 0 read as 1) below
static inline int mg_nu_coarse(const kc_mg_opts* o) { return std::max(1, o->nu_coarse); }
static inline int mg_nu_pre(const kc_mg_opts* o, int l) { return l == 0 ? o->nu_pre : mg_nu_coarse(o); }
static inline int mg_nu_post(const kc_mg_opts* o, int l) { return l == 0 ? o->nu_post : mg_nu_coarse(o); }

static bool mg_fusable(const MgLayout& M, const kc_mg_opts* o) {
    return o->nu_pre == 1 && o->nu_post == 1 && mg_nu_coarse(o) <= kMgMaxNu && M.levels >= 2;
}

template <int NU>
static cudaError_t launch_down_nu(bool big, const MgLvl& G, const float* b, float* xout, float* bc, int NXc, int NYc,
                                  const int* done, int early, cudaStream_t s) {
    if (big) {
        constexpr int TI = mg_big_ti(NU);
        return launch_chain(k_mg_down<TI, kMgAJ0, kMgRY0, (kMgStagedLarge || NU > 1), NU>,
                            mg_tile_grid(G.NX, G.NY, TI, mg_tj(kMgAJ0, NU)), dim3(kMgNT0), 0, s, G, b, xout, bc, NXc,
                            NYc, done, early);
    }
    return launch_chain(k_mg_down<kMgTI1, kMgAJ1, kMgRY1, true, NU>, mg_tile_grid(G.NX, G.NY, kMgTI1, mg_tj(kMgAJ1, NU)),
                        dim3(kMgNT1), 0, s, G, b, xout, bc, NXc, NYc, done, early);
}

template <int NU>
static cudaError_t launch_up_nu(bool big, const MgLvl& G, const float* xpre, const float* xc, int NXc, int NYc,
                                float alpha, const float* b, float* xout, const int* done, int early, cudaStream_t s) {
    if (big) {
        constexpr int TI = mg_big_ti(NU);
        return launch_chain(k_mg_up<TI, kMgAJ0, kMgRY0, (kMgStagedLarge || NU > 1), NU>,
                            mg_tile_grid(G.NX, G.NY, TI, mg_tj(kMgAJ0, NU)), dim3(kMgNT0), 0, s, G, xpre, xc, NXc,
                            NYc, alpha, b, xout, done, early);
    }
    return launch_chain(k_mg_up<kMgTI1, kMgAJ1, kMgRY1, true, NU>, mg_tile_grid(G.NX, G.NY, kMgTI1, mg_tj(kMgAJ1, NU)),
                        dim3(kMgNT1), 0, s, G, xpre, xc, NXc, NYc, alpha, b, xout, done, early);
}

// level 0 follows launches outside the cycle: its staging waits for the previous grid
static int launch_down(const MgLayout& M, const Lvl& L, int l, const float* b, float* xout, float* bc, const int* done,
                       const kc_mg_opts* o, cudaStream_t s) {
    const MgLvl G = mg_lvl(L);
    const bool big = l == 0 || mg_big(L.NX, L.NY, o);
    const int nu = l == 0 ? 1 : mg_nu_coarse(o);
    const int NXc = M.nx[l + 1], NYc = M.ny[l + 1];
    const int early = l > 0;
    const cudaError_t e = nu == 1   ? launch_down_nu<1>(big, G, b, xout, bc, NXc, NYc, done, early, s)
                          : nu == 2 ? launch_down_nu<2>(big, G, b, xout, bc, NXc, NYc, done, early, s)
                                    : launch_down_nu<3>(big, G, b, xout, bc, NXc, NYc, done, early, s);
    if (e != cudaSuccess) return cuda_status(e, "k_mg_down launch");
    KC_LAUNCH_CHECK_NC("k_mg_down");
    return KC_OK;
}

static int launch_up(const MgLayout& M, const Lvl& L, int l, const float* xpre, const float* xc, float alpha,
                     const float* b, float* xout, const int* done, const kc_mg_opts* o, cudaStream_t s) {
    const MgLvl G = mg_lvl(L);
    const bool big = l == 0 || mg_big(L.NX, L.NY, o);
    const int nu = l == 0 ? 1 : mg_nu_coarse(o);
    const int NXc = M.nx[l + 1], NYc = M.ny[l + 1];
    const int early = l > 0;
    const cudaError_t e = nu == 1   ? launch_up_nu<1>(big, G, xpre, xc, NXc, NYc, alpha, b, xout, done, early, s)
                          : nu == 2 ? launch_up_nu<2>(big, G, xpre, xc, NXc, NYc, alpha, b, xout, done, early, s)
                                    : launch_up_nu<3>(big, G, xpre, xc, NXc, NYc, alpha, b, xout, done, early, s);
    if (e != cudaSuccess) return cuda_status(e, "k_mg_up launch");
    KC_LAUNCH_CHECK_NC("k_mg_up");
    return KC_OK;
}

static inline unsigned pw_grid(long long n) { return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, 4096)); }

int mg_setup(const kc_system* A, void* ws, size_t ws_bytes, const kc_mg_opts* o, cudaStream_t s) {
    if (!A || !A->coef || A->dtype != KC_F32) return set_error("multigrid needs FP32 coefficients"), KC_ERR_ARG;
    const int NY = A->stride;
    if (NY < 1 || A->n % NY != 0) return set_error("multigrid: n = %lld is not a multiple of the stride %d", A->n, NY), KC_ERR_ARG;
    const int NX = (int)(A->n / NY);
    MgLayout M = mg_layout(NX, NY, o);
    if (!ws || ws_bytes < M.total) return set_error("multigrid workspace %zu < %zu", ws_bytes, M.total), KC_ERR_WORKSPACE;
    char* base = (char*)ws;
    const float* c0 = (const float*)A->coef;
    k_mg_diag0<<<pw_grid(A->n), 256, 0, s>>>(c0, A->cs, A->es, A->form == KC_FORM_LAPLACIAN, (int)A->n, o->omega[0],
                                              (float*)(base + M.off_winv[0]), (unsigned char*)(base + M.off_iso[0]));
    KC_LAUNCH_CHECK("k_mg_diag0");
    for (int l = 0; l + 1 < M.levels; ++l) {
        const float* cf = l == 0 ? c0 : (const float*)(base + M.off_coef[l]);
        const long long cs = l == 0 ? A->cs : (long long)M.nx[l] * M.ny[l];
        const long long es = l == 0 ? A->es : 1;
        dim3 g((M.ny[l + 1] + 127) / 128, M.nx[l + 1]);
        const int lapf = l == 0 ? (A->form == KC_FORM_LAPLACIAN) : 1;
        k_mg_coarsen<<<g, 128, 0, s>>>(cf, cs, es, lapf, (const unsigned char*)(base + M.off_iso[l]), M.nx[l], M.ny[l],
                                       (float*)(base + M.off_coef[l + 1]), M.nx[l + 1], M.ny[l + 1],
                                       o->omega[std::min(l + 1, KC_MG_MAX_LEVELS - 1)],
                                       (float*)(base + M.off_winv[l + 1]), (unsigned char*)(base + M.off_iso[l + 1]));
        KC_LAUNCH_CHECK("k_mg_coarsen");
    }
    if (o->coarsest_sweeps == 0) {   // direct coarsest solve: invert the coarsest operator
        const int l = M.levels - 1;
        const int nc = M.nx[l] * M.ny[l];
        const Lvl L = level_of(M, base, l, c0, A->cs, A->es, A->form == KC_FORM_LAPLACIAN);
        if (nc > kCoarseDirectMax) return set_error("kc_mg_setup: coarsest level of %d cells", nc), KC_ERR_ARG;
        float* inv = (float*)(base + M.off_inv);
        int* flag = (int*)(base + M.off_flag);
        static_assert(kGjR == 4, "register tiles of 1..4 rows per thread cover the coarsest level");
        switch ((nc + 31) / 32) {   // the smallest tile that covers the level: a pivot step costs R x R per thread
            case 0:
            case 1: k_mg_coarse_inverse<1><<<1, dim3(32, 32), 0, s>>>(L, inv, flag); break;
            case 2: k_mg_coarse_inverse<2><<<1, dim3(32, 32), 0, s>>>(L, inv, flag); break;
            case 3: k_mg_coarse_inverse<3><<<1, dim3(32, 32), 0, s>>>(L, inv, flag); break;
            default: k_mg_coarse_inverse<4><<<1, dim3(32, 32), 0, s>>>(L, inv, flag); break;
        }
        KC_LAUNCH_CHECK("k_mg_coarse_inverse");
    }
    return KC_OK;
}

// output of level l in the fused cycle (the caller's z for level 0)
static float* mg_final(const MgLayout& M, char* base, int l) { return (float*)(base + M.off_t[l]); }

MgFused mg_fused(const kc_system* A, void* ws, const kc_mg_opts* o) {
    MgFused F{};
    const int NY = A->stride;
    const MgLayout M = mg_layout((int)(A->n / NY), NY, o);
    F.ok = mg_fusable(M, o);
    if (!F.ok) return F;
    char* base = (char*)ws;
    F.L0 = mg_lvl(level_of(M, base, 0, (const float*)A->coef, A->cs, A->es, A->form == KC_FORM_LAPLACIAN));
    F.x0pre = (float*)(base + M.off_x[0]);
    F.b1 = (float*)(base + M.off_b[1]);
    F.final1 = mg_final(M, base, 1);
    F.NX1 = M.nx[1];
    F.NY1 = M.ny[1];
    F.alpha0 = o->alpha[0];
    return F;
}

// ---- coarse-level tail: plan and launch ---------------------------------------------
struct TailPlan {
    bool ok;
    int Ls, Lend;
    size_t smem;
};

static unsigned tail_magic(int d) {
    return d <= 1 ? 0u : (unsigned)((0x100000000ull + (unsigned long long)d - 1) / (unsigned long long)d);
}

// The tail takes the levels from the first one of at most kTailMax cells to
// the coarsest, when that is at least one level above the coarsest (fused
// cycle, exact coarsest solve) and their arrays fit the block's shared memory.
static TailPlan tail_plan(const MgLayout& M, const kc_mg_opts* o) {
    TailPlan P{};
    if (o->tail <= 0 || o->coarsest_sweeps != 0 || !mg_fusable(M, o)) return P;
    const int Lend = M.levels - 1;
    int Ls = 1;
    while (Ls < Lend && (long long)M.nx[Ls] * M.ny[Ls] > o->tail) ++Ls;
    if (Ls >= Lend) return P;
    size_t cells = 0;
    for (int l = Ls; l <= Lend; ++l) cells += (size_t)M.nx[l] * M.ny[l];
    const size_t nc = (size_t)M.nx[Lend] * M.ny[Lend];
    const size_t bytes = (kTailArrays * cells + nc * nc) * sizeof(float);
    if (bytes > 200 * 1024) return P;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return (void)cudaGetLastError(), P;
    static std::mutex mu;
    static bool attr_done[64] = {false};
    {
        std::lock_guard<std::mutex> lk(mu);
        if (dev >= 0 && dev < 64 && !attr_done[dev]) {
            if (cudaFuncSetAttribute(k_mg_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) !=
                cudaSuccess) {
                cudaGetLastError();
                return P;
            }
            attr_done[dev] = true;
        }
    }
    P = TailPlan{true, Ls, Lend, bytes};
    return P;
}

static int launch_tail(const TailPlan& P, const MgLayout& M, char* base, const kc_mg_opts* o, const int* done,
                       cudaStream_t s) {
    MgTail T{};
    int off = 0;
    for (int l = P.Ls; l <= P.Lend; ++l) {
        TailLevel& L = T.lv[l];
        L.c = (const float*)(base + M.off_coef[l]);
        L.winv = (const float*)(base + M.off_winv[l]);
        L.NX = M.nx[l];
        L.NY = M.ny[l];
        L.alpha = o->alpha[std::min(l, KC_MG_MAX_LEVELS - 1)];
        L.nu = std::max(mg_nu_pre(o, l), mg_nu_post(o, l));   // 1 on level 0 (fused cycle), nu_coarse below
        L.so = off;
        L.mNY = tail_magic(L.NY);
        L.mHalf = tail_magic((L.NY + 1) / 2);
        off += kTailArrays * L.NX * L.NY;
    }
    T.inv_so = off;
    const int nc = M.nx[P.Lend] * M.ny[P.Lend];
    off += nc * nc;
    if ((size_t)off * sizeof(float) != P.smem) return set_error("multigrid tail: shared memory plan mismatch"), KC_ERR_ARG;
    T.Ls = P.Ls;
    T.Lend = P.Lend;
    T.b_in = (const float*)(base + M.off_b[P.Ls]);
    T.x_out = mg_final(M, base, P.Ls);
    T.inv = (const float*)(base + M.off_inv);
    T.inv_bad = (const int*)(base + M.off_flag);
    KC_CUDA(launch_chain(k_mg_tail, dim3(1), dim3(kTailThreads), P.smem, s, T, done));
    return KC_OK;
}

int mg_cycle_kernels(const kc_system* A, const kc_mg_opts* o) {
    const int NY = A->stride;
    const MgLayout M = mg_layout((int)(A->n / NY), NY, o);
    if (mg_fusable(M, o)) {
        const TailPlan P = tail_plan(M, o);
        return P.ok ? 2 * P.Ls + 1 : 2 * (M.levels - 1) + 1;
    }
    int n = 1;
    for (int l = 0; l + 1 < M.levels; ++l)
        n += 2 + 2 * std::max(0, mg_nu_pre(o, l) - 1) + 1 + 1 + 2 * std::max(0, mg_nu_post(o, l));
    return n;
}

// levels >= 1 of the fused cycle: b_1 in, final_1 out
int mg_enqueue_coarse(const kc_system* A, void* ws, const kc_mg_opts* o, const int* done, cudaStream_t s,
                      int* kernels) {
    const int NY = A->stride;
    const MgLayout M = mg_layout((int)(A->n / NY), NY, o);
    char* base = (char*)ws;
    const float* c0 = (const float*)A->coef;
    const int lap0 = A->form == KC_FORM_LAPLACIAN;
    int nk = 0, rc;
    const TailPlan P = tail_plan(M, o);
    if (P.ok) {   // levels 1..Ls-1 one launch each, Ls..coarsest in the tail block
        for (int l = 1; l < P.Ls; ++l) {
            const Lvl L = level_of(M, base, l, c0, A->cs, A->es, lap0);
            rc = launch_down(M, L, l, (const float*)(base + M.off_b[l]), (float*)(base + M.off_x[l]),
                             (float*)(base + M.off_b[l + 1]), done, o, s);
            if (rc) return rc;
            ++nk;
        }
        rc = launch_tail(P, M, base, o, done, s);
        if (rc) return rc;
        ++nk;
        for (int l = P.Ls - 1; l >= 1; --l) {
            const Lvl L = level_of(M, base, l, c0, A->cs, A->es, lap0);
            rc = launch_up(M, L, l, (const float*)(base + M.off_x[l]), mg_final(M, base, l + 1),
                           o->alpha[std::min(l, KC_MG_MAX_LEVELS - 1)], (const float*)(base + M.off_b[l]),
                           mg_final(M, base, l), done, o, s);
            if (rc) return rc;
            ++nk;
        }
        if (kernels) *kernels = nk;
        return KC_OK;
    }
    for (int l = 1; l + 1 < M.levels; ++l) {
        const Lvl L = level_of(M, base, l, c0, A->cs, A->es, lap0);
        rc = launch_down(M, L, l, (const float*)(base + M.off_b[l]), (float*)(base + M.off_x[l]),
                         (float*)(base + M.off_b[l + 1]), done, o, s);
        if (rc) return rc;
        ++nk;
    }
    {
        const int l = M.levels - 1;
        const Lvl L = level_of(M, base, l, c0, A->cs, A->es, lap0);
        KC_CUDA(launch_chain(k_mg_coarsest, dim3(1), dim3(kCoarsestMax), 0, s, L, (const float*)(base + M.off_b[l]),
                             mg_final(M, base, l), o->coarsest_sweeps, (const float*)(base + M.off_inv),
                             (const int*)(base + M.off_flag), done));
        KC_LAUNCH_CHECK_NC("k_mg_coarsest");
        ++nk;
    }
    for (int l = M.levels - 2; l >= 1; --l) {
        const Lvl L = level_of(M, base, l, c0, A->cs, A->es, lap0);
        rc = launch_up(M, L, l, (const float*)(base + M.off_x[l]), mg_final(M, base, l + 1),
                       o->alpha[std::min(l, KC_MG_MAX_LEVELS - 1)], (const float*)(base + M.off_b[l]),
                       mg_final(M, base, l), done, o, s);
        if (rc) return rc;
        ++nk;
    }
    if (kernels) *kernels = nk;
    return KC_OK;
}

// Enqueues one V-cycle z = M r (level-0 input r, output z; both n floats).
int mg_enqueue(const kc_system* A, void* ws, const kc_mg_opts* o, const float* r, float* z, const int* done,
               cudaStream_t s, int* kernels) {
    int nk = 0;
    const int NY = A->stride;
    const int NX = (int)(A->n / NY);
    MgLayout M = mg_layout(NX, NY, o);
    char* base = (char*)ws;
    if (mg_fusable(M, o)) {
        const Lvl L0 = level_of(M, base, 0, (const float*)A->coef, A->cs, A->es, A->form == KC_FORM_LAPLACIAN);
        int rc = launch_down(M, L0, 0, r, (float*)(base + M.off_x[0]), (float*)(base + M.off_b[1]), done, o, s);
        if (rc) return rc;
        int kc = 0;
        rc = mg_enqueue_coarse(A, ws, o, done, s, &kc);
        if (rc) return rc;
        rc = launch_up(M, L0, 0, (const float*)(base + M.off_x[0]), mg_final(M, base, 1), o->alpha[0], r, z, done, o, s);
        if (rc) return rc;
        if (kernels) *kernels = kc + 2;
        return KC_OK;
    }
    const float* c0 = (const float*)A->coef;
    const float* bl[KC_MG_MAX_LEVELS];
    float* xl[KC_MG_MAX_LEVELS];
    for (int l = 0; l < M.levels; ++l) {
        bl[l] = l == 0 ? r : (const float*)(base + M.off_b[l]);
        xl[l] = l == 0 ? z : (float*)(base + M.off_x[l]);
    }
    // downward leg: nu_pre (level 0) / nu_coarse red-black sweeps (the first from x = 0), restrict
    for (int l = 0; l < M.levels; ++l) {
        Lvl L = level_of(M, base, l, c0, A->cs, A->es, A->form == KC_FORM_LAPLACIAN);
        const long long n = (long long)M.nx[l] * M.ny[l];
        if (l == M.levels - 1) {
            k_mg_coarsest<<<1, kCoarsestMax, 0, s>>>(L, bl[l], xl[l], o->coarsest_sweeps,
                                                     (const float*)(base + M.off_inv), (const int*)(base + M.off_flag),
                                                     done);
            KC_LAUNCH_CHECK_NC("k_mg_coarsest");
            ++nk;
            break;
        }
        k_mg_first<<<pw_grid(n), 256, 0, s>>>(L, bl[l], xl[l], done);
        KC_LAUNCH_CHECK_NC("k_mg_first");
        ++nk;
        k_mg_rbgs<<<pw_grid(n), 256, 0, s>>>(L, bl[l], xl[l], 1, done);
        KC_LAUNCH_CHECK_NC("k_mg_rbgs");
        ++nk;
        for (int q = 1; q < mg_nu_pre(o, l); ++q) {
            k_mg_rbgs<<<pw_grid(n), 256, 0, s>>>(L, bl[l], xl[l], 0, done);
            k_mg_rbgs<<<pw_grid(n), 256, 0, s>>>(L, bl[l], xl[l], 1, done);
            KC_LAUNCH_CHECK_NC("k_mg_rbgs");
            nk += 2;
        }
        dim3 g((M.ny[l + 1] + 127) / 128, M.nx[l + 1]);
        k_mg_restrict<<<g, 128, 0, s>>>(L, bl[l], xl[l], (float*)bl[l + 1], M.nx[l + 1], M.ny[l + 1], done);
        KC_LAUNCH_CHECK_NC("k_mg_restrict");
        ++nk;
    }
    // upward leg: over-corrected prolongation, nu_post (level 0) / nu_coarse red-black sweeps
    for (int l = M.levels - 2; l >= 0; --l) {
        Lvl L = level_of(M, base, l, c0, A->cs, A->es, A->form == KC_FORM_LAPLACIAN);
        const long long n = (long long)M.nx[l] * M.ny[l];
        k_mg_prolong<<<pw_grid(n), 256, 0, s>>>(L, xl[l], xl[l + 1], M.ny[l + 1],
                                                o->alpha[std::min(l, KC_MG_MAX_LEVELS - 1)], done);
        KC_LAUNCH_CHECK_NC("k_mg_prolong");
        ++nk;
        for (int q = 0; q < mg_nu_post(o, l); ++q) {
            k_mg_rbgs<<<pw_grid(n), 256, 0, s>>>(L, bl[l], xl[l], 1, done);
            k_mg_rbgs<<<pw_grid(n), 256, 0, s>>>(L, bl[l], xl[l], 0, done);
            KC_LAUNCH_CHECK_NC("k_mg_rbgs");
            nk += 2;
        }
    }
    if (kernels) *kernels = nk;
    return KC_OK;
}

}  // namespace kc

using namespace kc;

extern "C" {

void kc_mg_default_opts(kc_mg_opts* o) {
    if (!o) return;
    o->nu_pre = 1;             // the fused two-launch-per-level cycle
    o->nu_post = 1;
    o->nu_coarse = 2;          // two sweeps each way on the latency-bound levels below level 0
    o->coarsest_sweeps = 0;    // exact coarsest solve
    o->max_levels = KC_MG_MAX_LEVELS;
    o->tail = kTailMax;        // the levels of at most 1536 cells in one single-block launch
    o->big_cells = 200000;     // levels of 200k cells and more in the 64-wide tiles
    // Level 0 (one sweep, the expensive level): omega 1.0, alpha 1.9 -- measured on GB300 over
    // five p' systems (three time points of the 2048 x 512 channel, the 320 x 64 channel, a
    // random 1024^2 system): 2-4 CG iterations fewer per solve than the uniform omega 1.1 /
    // alpha 1.8.  Below (two sweeps, over-relaxed): omega 1.5, alpha 2.0 -- with the restated
    // cycle on the 2050 x 514 p' system of the channel 17 CG iterations to 1e-8 against 26
    // with one sweep of omega 1.1.
    for (int l = 0; l < KC_MG_MAX_LEVELS; ++l) {
        o->omega[l] = l == 0 ? 1.0f : 1.5f;
        o->alpha[l] = l == 0 ? 1.9f : 2.0f;
    }
}

size_t kc_mg_ws_bytes(long long n, int stride, const kc_mg_opts* opts) {
    if (n < 1 || stride < 1 || n % stride) return 0;
    kc_mg_opts d;
    if (!opts) {
        kc_mg_default_opts(&d);
        opts = &d;
    }
    return mg_layout((int)(n / stride), stride, opts).total;
}

int kc_mg_setup(const kc_system* A32, void* mg_ws, size_t mg_ws_bytes, const kc_mg_opts* opts, void* stream) {
    kc_mg_opts d;
    if (!opts) {
        kc_mg_default_opts(&d);
        opts = &d;
    }
    return mg_setup(A32, mg_ws, mg_ws_bytes, opts, as_stream(stream));
}

int kc_mg_apply(const kc_system* A32, void* mg_ws, const kc_mg_opts* opts, const float* r, float* z, void* stream) {
    if (!A32 || !mg_ws || !r || !z) return set_error("kc_mg_apply: null argument"), KC_ERR_ARG;
    kc_mg_opts d;
    if (!opts) {
        kc_mg_default_opts(&d);
        opts = &d;
    }
    int nk = 0;
    const int rc = mg_enqueue(A32, mg_ws, opts, r, z, nullptr, as_stream(stream), &nk);
    count_launches(nk);
    return rc;
}

}  // extern "C"
