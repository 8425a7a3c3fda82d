// Tile kernels of the fused multigrid V-cycle (NU pre- and NU post-smoothing
// red-black sweeps per level).  Per level l the cycle is two launches:
//
//   DOWN_l  x  = red half-sweep from 0     (x_red = W b, x_black = 0)
//           x += W (b - A x) on black cells, then red, black, ... (2 NU - 1 half-sweeps)
//           b_{l+1}(I,J) = sum over the aggregate's coupled cells of b - A x
//           writes x (the pre-smoothed iterate) and b_{l+1}
//   UP_l    x  = x_pre + alpha P x_{l+1}   (coupled cells)
//           x += W (b - A x) on black, then on red cells (NU times)
//           writes the level's output
//
// which is the same arithmetic as the unfused kernels (k_mg_first, k_mg_rbgs,
// k_mg_restrict, k_mg_prolong).  A block owns a TI x TJ tile (TI, TJ even, so
// every 2x2 aggregate lies in one tile) and stages an H = 2 NU cell halo in
// shared memory: half-sweep h runs over the staged region less h rings (its
// cells need the previous half-sweep's values one ring further out), so after
// the 2 NU - 1 pre-smoothing half-sweeps the tile and its 1-ring are exact --
// what the residual needs -- and the 2 NU post-smoothing half-sweeps end
// exactly on the tile.  Halo values are recomputed by every block that needs
// them, never exchanged, so a launch has no inter-block dependence.  The
// operator is the 2-D 5-point stencil with zero values outside [0,NX) x [0,NY).
//
// Staging is asynchronous (cp.async, zero-filled outside the grid): every
// thread issues all of its copies before waiting, so a block has its whole
// tile in flight at once -- the kernels are bound by memory latency
// otherwise.  (A tensor-map TMA box needs 16-byte row pitches, which the
// padded [nx+2][ny+2] fields do not have in general.)
//
// The level-0 launches of the preconditioned CG fold CG's pointwise passes in:
// DOWN_0 forms b = r - alpha q from two staged arrays and hands every owned
// cell to an Own policy; a Mid policy runs between issuing and awaiting the
// copies (CG's x update, whose loads then overlap the staging).
#pragma once
#include "kc_common.cuh"

namespace kc {

struct MgLvl {
    const float* c;        // 5 coefficient components
    long long cs, es;      // component stride, element stride
    int NX, NY;
    int lap;               // Laplacian form: component 0 is the row sum
    const float* winv;     // smoother weights (1/d for isolated rows)
    const unsigned char* iso;
};

// ---- asynchronous global -> shared copies (zero fill when !valid) -------------
__device__ __forceinline__ void cp_async4(float* smem, const float* gmem, bool valid) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(valid ? 4 : 0)
                 : "memory");
}
// two consecutive floats at once (both addresses 8-byte aligned), zero-filled when !valid
__device__ __forceinline__ void cp_async8f(float* smem, const float* gmem, bool valid) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(valid ? 8 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
// wait until at most N of this thread's most recent commit groups are pending
template <int N>
__device__ __forceinline__ void cp_async_wait_group() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

__device__ __forceinline__ float mg_row(float c0, float cw, float ce, float cn, float cs_, int lap, float x,
                                        float xw, float xe, float xn, float xs) {
    float y = c0 * x;
    if (lap) {
        y = fmaf(cw, xw - x, y);
        y = fmaf(ce, xe - x, y);
        y = fmaf(cn, xn - x, y);
        y = fmaf(cs_, xs - x, y);
    } else {
        y = fmaf(cw, xw, y);
        y = fmaf(ce, xe, y);
        y = fmaf(cn, xn, y);
        y = fmaf(cs_, xs, y);
    }
    return y;
}

struct MgNoMid {
    __device__ __forceinline__ void operator()() const {}
};
// Own policies see every owned cell once and may accumulate into a per-thread
// value of type Own::Sum, which the tile function returns.
struct MgOwnNone {
    struct Sum {};
    __device__ __forceinline__ void operator()(int, float, Sum&) const {}
    __device__ __forceinline__ void operator()(int, float, float, Sum&) const {}
};

// Tile geometry: rows of AJ = 32 or 64 staged cells (TJ = AJ - 2H owned
// columns plus the H-cell halo on each side), so a row is one or two warps
// and every index is a shift; RY thread rows walk the AI = TI + 2H staged rows.
// All staged arrays share the [AI][AJ] layout.  i0 - H and j0 - H are even
// (TI, TJ and H are), so a cell's colour (i + j) & 1 is (a + b) & 1 in tile
// coordinates and its aggregate's staged coarse index is (a >> 1, b >> 1).
template <int TI, int AJ_, int RY_, int H_ = 2>
struct MgTile {
    static constexpr int AJ = AJ_, RY = RY_, NT = AJ * RY, H = H_;
    static constexpr int TJ = AJ - 2 * H, AI = TI + 2 * H, A = AI * AJ;
    static_assert(H % 2 == 0 && H >= 2, "the halo is two cells per sweep");
    static_assert(TI % 2 == 0 && TJ % 2 == 0 && TJ > 0, "aggregates must not straddle tiles");
    static_assert((AJ & (AJ - 1)) == 0, "row width must be a power of two");
    __device__ static __forceinline__ int tx() { return threadIdx.x & (AJ - 1); }
    __device__ static __forceinline__ int ty() { return threadIdx.x / AJ; }
};

// Visits the cells of colour col ((a + b) & 1) in rows [a0, a1) and columns
// [b0, b1) of a tile staged as [AI][AJ], handing f their staged index.  AJ / 2
// threads share a row, thread m taking column 2 m or 2 m + 1 (whichever has the
// colour), so every lane of a warp has a cell: with one thread per column,
// every other lane would sit out each half-sweep.  Which thread updates a cell
// does not change what it computes.
template <class T, class F>
__device__ __forceinline__ void mg_colour_cells(int col, int a0, int a1, int b0, int b1, const F& f) {
    constexpr int HJ = T::AJ / 2, RP = T::NT / HJ;   // threads per row, rows per pass
    static_assert(T::NT % HJ == 0, "whole rows per pass");
    const int m = threadIdx.x & (HJ - 1);
    for (int a = a0 + (int)threadIdx.x / HJ; a < a1; a += RP) {
        const int b = 2 * m + ((a + col) & 1);
        if (b >= b0 && b < b1) f(a * T::AJ + b);
    }
}

// stage the 5 coefficient components over the whole staged region of the tile at (i0, j0)
// (H: halo width, the region starts at (i0 - H, j0 - H))
template <int TI, class T, int H = T::H>
__device__ __forceinline__ void mg_stage_coef(const MgLvl& L, int i0, int j0, float* sc) {
    const int b = T::tx(), j = j0 + b - H;
    const bool jin = j >= 0 && j < L.NY;
    for (int a = T::ty(); a < T::AI; a += T::RY) {
        const int i = i0 + a - H;
        const bool in = jin && i >= 0 && i < L.NX;
        const float* g = in ? L.c + (long long)(i * L.NY + j) * L.es : L.c;
        const int u = a * T::AJ + b;
#pragma unroll
        for (int q = 0; q < 5; ++q) cp_async4(sc + q * T::A + u, g + q * L.cs, in);
    }
}

// As mg_stage_coef, two columns per copy.  Needs an even row length NY and
// an even region origin j0 - H: then a pair (j, j + 1) with j even starts on
// an 8-byte boundary and lies wholly inside or outside the grid.
template <int TI, class T>
__device__ __forceinline__ void mg_stage_coef_pairs(const MgLvl& L, int i0, int j0, float* sc) {
    constexpr int PJ = T::AJ / 2;
    for (int e = threadIdx.x; e < T::AI * PJ; e += T::NT) {
        const int a = e / PJ, b = 2 * (e - a * PJ);
        const int i = i0 + a - T::H, j = j0 + b - T::H;
        const bool in = i >= 0 && i < L.NX && j >= 0 && j < L.NY;
        const float* g = in ? L.c + (long long)(i * L.NY + j) * L.es : L.c;
        const int u = a * T::AJ + b;
#pragma unroll
        for (int q = 0; q < 5; ++q) cp_async8f(sc + q * T::A + u, g + q * L.cs, in);
    }
}

// Coefficients of a tile: staged in shared memory (STAGED) or read through
// the read-only cache at the point of use (fewer staged arrays -> more
// resident blocks).  Indexed by staged position u = a * AJ + b.
template <class T, bool STAGED>
struct MgCoef {
    const float* sc;
    MgLvl L;
    int i0, j0;
    __device__ __forceinline__ float get(int q, int u) const {
        if (STAGED) return sc[q * T::A + u];
        const int a = u / T::AJ, b = u - a * T::AJ;
        const int i = i0 + a - T::H, j = j0 + b - T::H;
        if (i < 0 || i >= L.NX || j < 0 || j >= L.NY) return 0.f;
        return __ldg(L.c + q * L.cs + (long long)(i * L.NY + j) * L.es);
    }
    __device__ __forceinline__ float ax(const float* sx, int u) const {
        return mg_row(get(0, u), get(1, u), get(2, u), get(3, u), get(4, u), L.lap, sx[u], sx[u - T::AJ],
                      sx[u + T::AJ], sx[u + 1], sx[u - 1]);
    }
    __device__ __forceinline__ bool linked(int u) const {
        return get(1, u) != 0.f || get(2, u) != 0.f || get(3, u) != 0.f || get(4, u) != 0.f;
    }
};

// Shared-memory arrays of one tile, all [AI][AJ] except sxc (coarse cells
// under the tile, [TI/2 + 2][AJ/2]).  DOWN stages sb, sq (HasQ), sw, sc and
// uses sx as scratch; UP stages sx (the pre-smoothed iterate), sb, sw, sxc, sc.
struct MgStage {
    float* sb;
    float* sq;
    float* sw;
    float* sc;    // 5 coefficient components
    float* sx;
    float* sxc;
    float* ss;    // a further staged array of the caller's (the single-reduction CG's previous s)
};

// DOWN, asynchronous part, in two halves by what they depend on: the smoother
// weights and coefficients (written by the hierarchy's setup, several launches
// back) and the right-hand side b_in (and q), which the previous launch of the
// cycle writes.  Halo H cells.
template <int TI, int AJ, int RY, int H = 2>
__device__ __forceinline__ void mg_down_issue_fixed(int i0, int j0, const MgLvl& L, MgStage S) {
    using T = MgTile<TI, AJ, RY, H>;
    const int b = T::tx(), j = j0 + b - H;
    const bool jin = j >= 0 && j < L.NY;
    for (int a = T::ty(); a < T::AI; a += T::RY) {
        const int i = i0 + a - H;
        const bool in = jin && i >= 0 && i < L.NX;
        cp_async4(S.sw + a * T::AJ + b, L.winv + (in ? i * L.NY + j : 0), in);
    }
    mg_stage_coef<TI, T>(L, i0, j0, S.sc);
}
template <int TI, int AJ, int RY, bool HasQ, int H = 2>
__device__ __forceinline__ void mg_down_issue_rhs(int i0, int j0, const MgLvl& L, const float* __restrict__ b_in,
                                                  const float* __restrict__ q, MgStage S) {
    using T = MgTile<TI, AJ, RY, H>;
    const int b = T::tx(), j = j0 + b - H;
    const bool jin = j >= 0 && j < L.NY;
    for (int a = T::ty(); a < T::AI; a += T::RY) {
        const int i = i0 + a - H;
        const bool in = jin && i >= 0 && i < L.NX;
        const int k = in ? i * L.NY + j : 0;
        const int u = a * T::AJ + b;
        cp_async4(S.sb + u, b_in + k, in);
        if (HasQ) cp_async4(S.sq + u, q + k, in);
    }
}

// DOWN, after the tile's copies have landed: b = b_in - alpha q, red start,
// 2 NU - 1 half-sweeps (black, red, ...) over shrinking rings, x and the
// restricted residual out
// right-hand side of the DOWN pass at staged position u: b_in (MgPreB) or
// b_in - alpha q (MgPreQ); k is the cell index of an owned cell, else -1
struct MgPreB {
    __device__ __forceinline__ float operator()(const MgStage& S, int u, int) const { return S.sb[u]; }
};
struct MgPreQ {
    float alpha;
    __device__ __forceinline__ float operator()(const MgStage& S, int u, int) const {
        return fmaf(-alpha, S.sq[u], S.sb[u]);
    }
};

template <int TI, int AJ, int RY, class Pre, class Own, int NU = 1>
__device__ __forceinline__ void mg_down_compute_pre(int i0, int j0, const MgLvl& L, const Pre& pre, const Own& own,
                                                    MgStage S, float* __restrict__ xout, float* __restrict__ bc,
                                                    int NXc, int NYc, typename Own::Sum& sum) {
    using T = MgTile<TI, AJ, RY, 2 * NU>;
    constexpr int H = T::H;
    float* sb = S.sb;
    const float* sw = S.sw;
    float* sx = S.sx;
    const MgCoef<T, true> C{S.sc, L, i0, j0};
    const int b = T::tx(), j = j0 + b - H;
    const bool jown = b >= H && b < T::TJ + H && j < L.NY;
    // b, owned cells, red start (x = W b on red, 0 on black)
    for (int a = T::ty(); a < T::AI; a += T::RY) {
        const int u = a * T::AJ + b;
        const int i = i0 + a - H;
        const int k = (jown && a >= H && a < TI + H && i < L.NX) ? i * L.NY + j : -1;
        const float bv = pre(S, u, k);
        sb[u] = bv;
        if (k >= 0) own(k, bv, sum);
        sx[u] = ((a + b) & 1) == 0 ? sw[u] * bv : 0.f;
    }
    __syncthreads();
    // half-sweep h = 1 .. 2 NU - 1 (odd: black, even: red) over the region less h rings
#pragma unroll
    for (int h = 1; h < 2 * NU; ++h) {
        mg_colour_cells<T>(h & 1, h, T::AI - h, h, AJ - h,
                           [&](int u) { sx[u] = fmaf(sw[u], sb[u] - C.ax(sx, u), sx[u]); });
        __syncthreads();
    }
    // owned cells: write x
    if (jown)
        for (int a = H + T::ty(); a < TI + H; a += T::RY) {
            const int i = i0 + a - H;
            if (i < L.NX) xout[i * L.NY + j] = sx[a * T::AJ + b];
        }
    // aggregates: restricted residual over coupled cells
    for (int t = threadIdx.x; t < (TI / 2) * (T::TJ / 2); t += T::NT) {
        const int ag = t / (T::TJ / 2), bg = t - ag * (T::TJ / 2);
        const int I = (i0 >> 1) + ag, J = (j0 >> 1) + bg;
        if (I >= NXc || J >= NYc) continue;
        float s = 0.f;
#pragma unroll
        for (int di = 0; di < 2; ++di)
#pragma unroll
            for (int dj = 0; dj < 2; ++dj) {
                const int a = 2 * ag + di + H, bb = 2 * bg + dj + H;
                if (i0 + a - H >= L.NX || j0 + bb - H >= L.NY) continue;
                const int u = a * T::AJ + bb;
                if (!C.linked(u)) continue;
                s += sb[u] - C.ax(sx, u);
            }
        bc[I * NYc + J] = s;
    }
}

template <int TI, int AJ, int RY, bool HasQ, class Own, int NU = 1>
__device__ __forceinline__ void mg_down_compute(int i0, int j0, const MgLvl& L, float alpha, const Own& own,
                                                MgStage S, float* __restrict__ xout, float* __restrict__ bc,
                                                int NXc, int NYc, typename Own::Sum& sum) {
    if (HasQ)
        mg_down_compute_pre<TI, AJ, RY, MgPreQ, Own, NU>(i0, j0, L, MgPreQ{alpha}, own, S, xout, bc, NXc, NYc, sum);
    else
        mg_down_compute_pre<TI, AJ, RY, MgPreB, Own, NU>(i0, j0, L, MgPreB{}, own, S, xout, bc, NXc, NYc, sum);
}

// DOWN tile at (i0, j0) (multiples of TI, TJ).  b = HasQ ? b_in - alpha q : b_in over the staged region.
// NU sweeps need the staged coefficients (STAGED); the unstaged variant is the one-sweep cycle.
// gate() runs the grid dependency wait and returns false when the solve is
// over; with early, the weights and coefficients are staged before it (the
// caller guarantees that the launch before this one waited for its own
// predecessor first, so the setup that wrote them has finished).
template <int TI, int AJ, int RY, bool HasQ, class Mid, class Own, bool STAGED = true, int NU = 1, class Gate>
__device__ __forceinline__ typename Own::Sum mg_down_tile(int i0, int j0, const MgLvl& L, const float* __restrict__ b_in,
                                                          const float* __restrict__ q, float alpha, const Mid& mid,
                                                          const Own& own, float* __restrict__ xout,
                                                          float* __restrict__ bc, int NXc, int NYc, const Gate& gate,
                                                          bool early) {
    static_assert(STAGED || NU == 1, "several sweeps per level read the staged coefficients");
    if (STAGED) {
        using TS = MgTile<TI, AJ, RY, 2 * NU>;
        __shared__ __align__(16) float sb[TS::A], sw[TS::A], sx[TS::A];
        __shared__ __align__(16) float sq[HasQ ? TS::A : 1];
        __shared__ __align__(16) float sc[5 * TS::A];
        const MgStage S{sb, sq, sw, sc, sx, nullptr, nullptr};
        if (early) mg_down_issue_fixed<TI, AJ, RY, 2 * NU>(i0, j0, L, S);
        if (!gate()) {
            cp_async_wait_all();
            return typename Own::Sum{};
        }
        if (!early) mg_down_issue_fixed<TI, AJ, RY, 2 * NU>(i0, j0, L, S);
        mg_down_issue_rhs<TI, AJ, RY, HasQ, 2 * NU>(i0, j0, L, b_in, q, S);
        cp_async_commit();
        mid();
        cp_async_wait_all();
        __syncthreads();
        typename Own::Sum sum{};
        mg_down_compute<TI, AJ, RY, HasQ, Own, NU>(i0, j0, L, alpha, own, S, xout, bc, NXc, NYc, sum);
        return sum;
    }
    using T = MgTile<TI, AJ, RY>;
    __shared__ __align__(16) float sb[T::A], sw[T::A], sx[T::A];
    __shared__ __align__(16) float sq[HasQ ? T::A : 1];
    const MgCoef<T, false> C{nullptr, L, i0, j0};
    const int b = T::tx(), j = j0 + b - 2;
    const bool jin = j >= 0 && j < L.NY;
    const bool jown = b >= 2 && b < T::TJ + 2 && j < L.NY;
    typename Own::Sum sum{};
    if (!gate()) return sum;
    for (int a = T::ty(); a < T::AI; a += T::RY) {
        const int i = i0 + a - 2;
        const bool in = jin && i >= 0 && i < L.NX;
        const int k = in ? i * L.NY + j : 0;
        const int u = a * T::AJ + b;
        cp_async4(sb + u, b_in + k, in);
        if (HasQ) cp_async4(sq + u, q + k, in);
        cp_async4(sw + u, L.winv + k, in);
    }
    cp_async_commit();
    mid();
    cp_async_wait_all();
    __syncthreads();
    for (int a = T::ty(); a < T::AI; a += T::RY) {
        const int u = a * T::AJ + b;
        const int i = i0 + a - 2;
        float bv = sb[u];
        if (HasQ) {
            bv = fmaf(-alpha, sq[u], bv);
            sb[u] = bv;
        }
        if (jown && a >= 2 && a < TI + 2 && i < L.NX) own(i * L.NY + j, bv, sum);
        sx[u] = ((a + b) & 1) == 0 ? sw[u] * bv : 0.f;
    }
    __syncthreads();
    if (b >= 1 && b < AJ - 1)
        for (int a = 1 + T::ty(); a < T::AI - 1; a += T::RY) {
            if (((a + b) & 1) == 0) continue;
            const int u = a * T::AJ + b;
            sx[u] = fmaf(sw[u], sb[u] - C.ax(sx, u), sx[u]);
        }
    __syncthreads();
    if (jown)
        for (int a = 2 + T::ty(); a < TI + 2; a += T::RY) {
            const int i = i0 + a - 2;
            if (i < L.NX) xout[i * L.NY + j] = sx[a * T::AJ + b];
        }
    for (int t = threadIdx.x; t < (TI / 2) * (T::TJ / 2); t += T::NT) {
        const int ag = t / (T::TJ / 2), bg = t - ag * (T::TJ / 2);
        const int I = (i0 >> 1) + ag, J = (j0 >> 1) + bg;
        if (I >= NXc || J >= NYc) continue;
        float s = 0.f;
#pragma unroll
        for (int di = 0; di < 2; ++di)
#pragma unroll
            for (int dj = 0; dj < 2; ++dj) {
                const int a = 2 * ag + di + 2, bb = 2 * bg + dj + 2;
                if (i0 + a - 2 >= L.NX || j0 + bb - 2 >= L.NY) continue;
                const int u = a * T::AJ + bb;
                if (!C.linked(u)) continue;
                s += sb[u] - C.ax(sx, u);
            }
        bc[I * NYc + J] = s;
    }
    return sum;
}

// UP, asynchronous part, in two halves by what they depend on: x_pre, b_in, W
// and the coefficients (written launches back), and the coarse cells under
// the tile (the previous launch's result; they start at (i0 - H) / 2, (j0 - H) / 2).
template <int TI, int AJ, int RY, int H = 2>
__device__ __forceinline__ void mg_up_issue_fixed(int i0, int j0, const MgLvl& L, const float* __restrict__ xpre,
                                                  const float* __restrict__ b_in, MgStage S) {
    using T = MgTile<TI, AJ, RY, H>;
    const int b = T::tx(), j = j0 + b - H;
    const bool jin = j >= 0 && j < L.NY;
    for (int a = T::ty(); a < T::AI; a += T::RY) {
        const int i = i0 + a - H;
        const bool in = jin && i >= 0 && i < L.NX;
        const int k = in ? i * L.NY + j : 0;
        const int u = a * T::AJ + b;
        cp_async4(S.sx + u, xpre + k, in);
        cp_async4(S.sb + u, b_in + k, in);
        cp_async4(S.sw + u, L.winv + k, in);
    }
    mg_stage_coef<TI, T>(L, i0, j0, S.sc);
}
template <int TI, int AJ, int RY, int H = 2>
__device__ __forceinline__ void mg_up_issue_coarse(int i0, int j0, const float* __restrict__ xc, int NXc, int NYc,
                                                   MgStage S) {
    using T = MgTile<TI, AJ, RY, H>;
    constexpr int XI = TI / 2 + H, XJ = AJ / 2;
    for (int t = threadIdx.x; t < XI * XJ; t += T::NT) {
        const int ca = t / XJ, cb = t - ca * XJ;
        const int I = (i0 >> 1) - H / 2 + ca, J = (j0 >> 1) - H / 2 + cb;
        const bool in = I >= 0 && I < NXc && J >= 0 && J < NYc;
        cp_async4(S.sxc + t, xc + (in ? I * NYc + J : 0), in);
    }
}

// UP, after the copies have landed: prolong (coupled cells, told apart by
// their links), half-sweeps black, red, ... over shrinking rings (2 NU in
// all, the last -- red -- on the owned cells), write
template <int TI, int AJ, int RY, class Own, int NU = 1>
__device__ __forceinline__ void mg_up_compute(int i0, int j0, const MgLvl& L, float alpha, const Own& own,
                                              MgStage S, float* __restrict__ xout, typename Own::Sum& sum) {
    using T = MgTile<TI, AJ, RY, 2 * NU>;
    constexpr int H = T::H, XJ = AJ / 2;
    float* sx = S.sx;
    const float* sb = S.sb;
    const float* sw = S.sw;
    const float* sxc = S.sxc;
    const MgCoef<T, true> C{S.sc, L, i0, j0};
    const int b = T::tx(), j = j0 + b - H;
    // prolongation over the staged region (coupled cells only; a, b >= 0 <=> i, j >= i0-H, j0-H)
    for (int a = T::ty(); a < T::AI; a += T::RY) {
        const int u = a * T::AJ + b;
        if (!C.linked(u)) continue;
        sx[u] = fmaf(alpha, sxc[(a >> 1) * XJ + (b >> 1)], sx[u]);
    }
    __syncthreads();
    // half-sweep h = 1 .. 2 NU - 1 (odd: black, even: red) over the region less h rings
#pragma unroll
    for (int h = 1; h < 2 * NU; ++h) {
        mg_colour_cells<T>(h & 1, h, T::AI - h, h, AJ - h,
                           [&](int u) { sx[u] = fmaf(sw[u], sb[u] - C.ax(sx, u), sx[u]); });
        __syncthreads();
    }
    // the last (red) half-sweep on the owned cells, then write
    if (b >= H && b < T::TJ + H && j < L.NY)
        for (int a = H + T::ty(); a < TI + H; a += T::RY) {
            const int i = i0 + a - H;
            if (i >= L.NX) continue;
            const int u = a * T::AJ + b;
            float xv = sx[u];
            if (((a + b) & 1) == 0) xv = fmaf(sw[u], sb[u] - C.ax(sx, u), xv);
            const int k = i * L.NY + j;
            xout[k] = xv;
            own(k, xv, sb[u], sum);
        }
}

// UP tile at (i0, j0): prolong (coupled cells, told apart by their links),
// then the NU post-smoothing sweeps (black, red), the last red half-sweep on the owned cells.
// gate and early as for mg_down_tile (early: x_pre, b_in, W and the coefficients before the wait)
template <int TI, int AJ, int RY, class Own, bool STAGED = true, int NU = 1, class Gate>
__device__ __forceinline__ typename Own::Sum mg_up_tile(int i0, int j0, const MgLvl& L, const float* __restrict__ xpre,
                                                        const float* __restrict__ xc, int NXc, int NYc, float alpha,
                                                        const float* __restrict__ b_in, const Own& own,
                                                        float* __restrict__ xout, const Gate& gate, bool early) {
    static_assert(STAGED || NU == 1, "several sweeps per level read the staged coefficients");
    if (STAGED) {
        using TS = MgTile<TI, AJ, RY, 2 * NU>;
        constexpr int XIS = TI / 2 + TS::H, XJS = AJ / 2;   // coarse cells under the staged region
        __shared__ __align__(16) float sx[TS::A], sb[TS::A], sw[TS::A], sxc[XIS * XJS];
        __shared__ __align__(16) float sc[5 * TS::A];
        const MgStage S{sb, nullptr, sw, sc, sx, sxc, nullptr};
        if (early) mg_up_issue_fixed<TI, AJ, RY, 2 * NU>(i0, j0, L, xpre, b_in, S);
        if (!gate()) {
            cp_async_wait_all();
            return typename Own::Sum{};
        }
        if (!early) mg_up_issue_fixed<TI, AJ, RY, 2 * NU>(i0, j0, L, xpre, b_in, S);
        mg_up_issue_coarse<TI, AJ, RY, 2 * NU>(i0, j0, xc, NXc, NYc, S);
        cp_async_commit();
        cp_async_wait_all();
        __syncthreads();
        typename Own::Sum sum{};
        mg_up_compute<TI, AJ, RY, Own, NU>(i0, j0, L, alpha, own, S, xout, sum);
        return sum;
    }
    using T = MgTile<TI, AJ, RY>;
    constexpr int XI = TI / 2 + 2, XJ = AJ / 2;   // coarse cells under the staged region
    __shared__ __align__(16) float sx[T::A], sb[T::A], sw[T::A], sxc[XI * XJ];
    const MgCoef<T, false> C{nullptr, L, i0, j0};
    const int b = T::tx(), j = j0 + b - 2;
    const bool jin = j >= 0 && j < L.NY;
    typename Own::Sum sum{};
    if (!gate()) return sum;
    for (int a = T::ty(); a < T::AI; a += T::RY) {
        const int i = i0 + a - 2;
        const bool in = jin && i >= 0 && i < L.NX;
        const int k = in ? i * L.NY + j : 0;
        const int u = a * T::AJ + b;
        cp_async4(sx + u, xpre + k, in);
        cp_async4(sb + u, b_in + k, in);
        cp_async4(sw + u, L.winv + k, in);
    }
    for (int t = threadIdx.x; t < XI * XJ; t += T::NT) {
        const int ca = t / XJ, cb = t - ca * XJ;
        const int I = (i0 >> 1) - 1 + ca, J = (j0 >> 1) - 1 + cb;
        const bool in = I >= 0 && I < NXc && J >= 0 && J < NYc;
        cp_async4(sxc + t, xc + (in ? I * NYc + J : 0), in);
    }
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    for (int a = T::ty(); a < T::AI; a += T::RY) {
        const int u = a * T::AJ + b;
        if (!C.linked(u)) continue;
        sx[u] = fmaf(alpha, sxc[(a >> 1) * XJ + (b >> 1)], sx[u]);
    }
    __syncthreads();
    if (b >= 1 && b < AJ - 1)
        for (int a = 1 + T::ty(); a < T::AI - 1; a += T::RY) {
            if (((a + b) & 1) == 0) continue;
            const int u = a * T::AJ + b;
            sx[u] = fmaf(sw[u], sb[u] - C.ax(sx, u), sx[u]);
        }
    __syncthreads();
    if (b >= 2 && b < T::TJ + 2 && j < L.NY)
        for (int a = 2 + T::ty(); a < TI + 2; a += T::RY) {
            const int i = i0 + a - 2;
            if (i >= L.NX) continue;
            const int u = a * T::AJ + b;
            float xv = sx[u];
            if (((a + b) & 1) == 0) xv = fmaf(sw[u], sb[u] - C.ax(sx, u), xv);
            const int k = i * L.NY + j;
            xout[k] = xv;
            own(k, xv, sb[u], sum);
        }
    return sum;
}

// ---- UP with a 3-cell halo: z final on the owned cells and their 1-ring ----
// The single-reduction CG needs w = A z next to z, so the UP pass also
// finishes the red cells of the 1-ring (the black half-sweep then covers the
// 2-ring): the staged region is the tile plus 3 cells, TJ = AJ - 6 owned
// columns.  z on the owned cells is the same, operation for operation, as
// with the 2-cell halo.
template <int TI, int AJ_, int RY_>
struct MgTile3 {
    static constexpr int AJ = AJ_, RY = RY_, NT = AJ * RY, H = 3;
    static constexpr int TJ = AJ - 6, AI = TI + 6, A = AI * AJ;
    static constexpr int XI = TI / 2 + 4, XJ = AJ / 2 + 1, XC = XI * XJ;   // coarse cells under the region
    static_assert(TI % 2 == 0 && TJ % 2 == 0, "aggregates must not straddle tiles");
    static_assert((AJ & (AJ - 1)) == 0, "row width must be a power of two");
    __device__ static __forceinline__ int tx() { return threadIdx.x & (AJ - 1); }
    __device__ static __forceinline__ int ty() { return threadIdx.x / AJ; }
};

// stage x_pre, W and the coefficients of the tile at (i0, j0) (region from i0 - 3, j0 - 3): data
// written launches back
template <int TI, int AJ, int RY>
__device__ __forceinline__ void mg_up3_issue_fixed(int i0, int j0, const MgLvl& L, const float* __restrict__ xpre,
                                                   MgStage S) {
    using T = MgTile3<TI, AJ, RY>;
    const int b = T::tx(), j = j0 + b - 3;
    const bool jin = j >= 0 && j < L.NY;
    for (int a = T::ty(); a < T::AI; a += T::RY) {
        const int i = i0 + a - 3;
        const bool in = jin && i >= 0 && i < L.NX;
        const int k = in ? i * L.NY + j : 0;
        const int u = a * T::AJ + b;
        cp_async4(S.sx + u, xpre + k, in);
        cp_async4(S.sw + u, L.winv + k, in);
    }
    mg_stage_coef<TI, T, 3>(L, i0, j0, S.sc);
}
// stage b and the coarse cells under the tile (the coarse result: the previous launch's)
template <int TI, int AJ, int RY>
__device__ __forceinline__ void mg_up3_issue_rest(int i0, int j0, const MgLvl& L, const float* __restrict__ xc,
                                                  int NXc, int NYc, const float* __restrict__ b_in, MgStage S) {
    using T = MgTile3<TI, AJ, RY>;
    const int b = T::tx(), j = j0 + b - 3;
    const bool jin = j >= 0 && j < L.NY;
    for (int a = T::ty(); a < T::AI; a += T::RY) {
        const int i = i0 + a - 3;
        const bool in = jin && i >= 0 && i < L.NX;
        cp_async4(S.sb + a * T::AJ + b, b_in + (in ? i * L.NY + j : 0), in);
    }
    for (int t = threadIdx.x; t < T::XC; t += T::NT) {
        const int ca = t / T::XJ, cb = t - ca * T::XJ;
        const int I = (i0 >> 1) - 2 + ca, J = (j0 >> 1) - 2 + cb;
        const bool in = I >= 0 && I < NXc && J >= 0 && J < NYc;
        cp_async4(S.sxc + t, xc + (in ? I * NYc + J : 0), in);
    }
}
template <int TI, int AJ, int RY>
__device__ __forceinline__ void mg_up3_issue(int i0, int j0, const MgLvl& L, const float* __restrict__ xpre,
                                             const float* __restrict__ xc, int NXc, int NYc,
                                             const float* __restrict__ b_in, MgStage S) {
    mg_up3_issue_fixed<TI, AJ, RY>(i0, j0, L, xpre, S);
    mg_up3_issue_rest<TI, AJ, RY>(i0, j0, L, xc, NXc, NYc, b_in, S);
}

// prolong, black half-sweep over the 2-ring, red half-sweep over the 1-ring;
// then on the owned cells z, w = A z and the sums (r, z), (w, z)
template <int TI, int AJ, int RY, class Acc2>
__device__ __forceinline__ void mg_up3_compute(int i0, int j0, const MgLvl& L, float alpha, MgStage S,
                                               float* __restrict__ z_out, float* __restrict__ w_out, Acc2& rz,
                                               Acc2& wz) {
    using T = MgTile3<TI, AJ, RY>;
    float* sx = S.sx;
    const float* sb = S.sb;
    const float* sw = S.sw;
    const float* sxc = S.sxc;
    const MgCoef<T, true> C{S.sc, L, i0, j0};
    const int b = T::tx(), j = j0 + b - 3;
    // prolongation over the staged region (coupled cells only); the coarse cell of staged (a, b) is ((a+1)/2, (b+1)/2)
    for (int a = T::ty(); a < T::AI; a += T::RY) {
        const int u = a * T::AJ + b;
        if (!C.linked(u)) continue;
        sx[u] = fmaf(alpha, sxc[((a + 1) >> 1) * T::XJ + ((b + 1) >> 1)], sx[u]);
    }
    __syncthreads();
    // black half-sweep over the 2-ring and inside ((a + b) odd <=> (i + j) odd: the offset 3 + 3 is even)
    const auto relax = [&](int u) { sx[u] = fmaf(sw[u], sb[u] - C.ax(sx, u), sx[u]); };
    mg_colour_cells<T>(1, 1, T::AI - 1, 1, AJ - 1, relax);
    __syncthreads();
    // red half-sweep over the 1-ring and inside
    mg_colour_cells<T>(0, 2, T::AI - 2, 2, AJ - 2, relax);
    __syncthreads();
    // owned cells: z, w = A z, (r, z), (w, z)
    if (b >= 3 && b < T::TJ + 3 && j < L.NY)
        for (int a = 3 + T::ty(); a < TI + 3; a += T::RY) {
            const int i = i0 + a - 3;
            if (i >= L.NX) continue;
            const int u = a * T::AJ + b;
            const float zv = sx[u];
            const float wv = C.ax(sx, u);
            const int k = i * L.NY + j;
            z_out[k] = zv;
            w_out[k] = wv;
            rz.add(sb[u], zv);
            wz.add(wv, zv);
        }
}

}  // namespace kc
