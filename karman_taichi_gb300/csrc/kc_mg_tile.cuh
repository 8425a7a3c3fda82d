// Tile kernels of the fused multigrid V-cycle (one pre- and one post-smoothing
// red-black sweep per level).  Per level l the cycle is two launches:
//
//   DOWN_l  x  = red half-sweep from 0     (x_red = W b, x_black = 0)
//           x += W (b - A x) on black cells
//           b_{l+1}(I,J) = sum over the aggregate's coupled cells of b - A x
//           writes x (the pre-smoothed iterate) and b_{l+1}
//   UP_l    x  = x_pre + alpha P x_{l+1}   (coupled cells)
//           x += W (b - A x) on black, then on red cells
//           writes the level's output
//
// which is the same arithmetic as the unfused kernels (k_mg_first, k_mg_rbgs,
// k_mg_restrict, k_mg_prolong).  A block owns a TI x TJ tile (TI, TJ even, so
// every 2x2 aggregate lies in one tile) and stages a 2-cell halo in shared
// memory: the black cells of the 1-cell ring need the red cells of the 2-cell
// ring.  Halo values are recomputed by every block that needs them, never
// exchanged, so a launch has no inter-block dependence.  The operator is the
// 2-D 5-point stencil with zero values outside [0,NX) x [0,NY).
//
// The level-0 launches of the preconditioned CG fold CG's pointwise passes in
// through the BSrc (where b comes from) and Own (what happens to each owned
// cell) policies.
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

// b from a plain array
struct MgBLoad {
    const float* __restrict__ b;
    __device__ __forceinline__ float operator()(int k) const { return __ldg(b + k); }
};
struct MgOwnNone {
    __device__ __forceinline__ void operator()(int, float) const {}
    __device__ __forceinline__ void operator()(int, float, float) const {}
};

template <int TI, int TJ>
struct MgTileDims {
    static constexpr int AI = TI + 4, AJ = TJ + 4;   // 2-cell halo
    static constexpr int CI = TI + 2, CJ = TJ + 2;   // 1-cell halo
};

// stage the 5 coefficient components over the 1-cell halo ring (0 outside)
template <int TI, int TJ, int NT>
__device__ __forceinline__ void mg_stage_coef(const MgLvl& L, int i0, int j0, float (*sc)[(TI + 2) * (TJ + 2)]) {
    using D = MgTileDims<TI, TJ>;
    for (int t = threadIdx.x; t < D::CI * D::CJ; t += NT) {
        const int ii = t / D::CJ, jj = t - ii * D::CJ;
        const int i = i0 + ii - 1, j = j0 + jj - 1;
        const bool in = i >= 0 && i < L.NX && j >= 0 && j < L.NY;
        const long long e = in ? (long long)(i * L.NY + j) * L.es : 0;
#pragma unroll
        for (int q = 0; q < 5; ++q) sc[q][t] = in ? __ldg(L.c + q * L.cs + e) : 0.f;
    }
}

// (A x)(cell at 2-halo coords (a, b)); x staged over the 2-cell halo, coefficients over the 1-cell halo
template <int TI, int TJ>
__device__ __forceinline__ float mg_ax_smem(const float* sx, const float (*sc)[(TI + 2) * (TJ + 2)], int lap, int a,
                                            int b) {
    using D = MgTileDims<TI, TJ>;
    const int t = (a - 1) * D::CJ + (b - 1);
    const int u = a * D::AJ + b;
    return mg_row(sc[0][t], sc[1][t], sc[2][t], sc[3][t], sc[4][t], lap, sx[u], sx[u - D::AJ], sx[u + D::AJ],
                  sx[u + 1], sx[u - 1]);
}

template <int TI, int TJ, int NT, class BSrc, class Own>
__device__ __forceinline__ void mg_down_tile(const MgLvl& L, const BSrc& bsrc, const Own& own,
                                             float* __restrict__ xout, float* __restrict__ bc, int NXc, int NYc) {
    using D = MgTileDims<TI, TJ>;
    __shared__ float sb[D::AI * D::AJ], sw[D::AI * D::AJ], sx[D::AI * D::AJ];
    __shared__ float sc[5][D::CI * D::CJ];
    const int i0 = blockIdx.y * TI, j0 = blockIdx.x * TJ;
    // b and W over the 2-cell halo; red cells start at W b, black at 0
    for (int t = threadIdx.x; t < D::AI * D::AJ; t += NT) {
        const int a = t / D::AJ, b = t - a * D::AJ;
        const int i = i0 + a - 2, j = j0 + b - 2;
        float bv = 0.f, wv = 0.f;
        if (i >= 0 && i < L.NX && j >= 0 && j < L.NY) {
            const int k = i * L.NY + j;
            bv = bsrc(k);
            wv = __ldg(L.winv + k);
            if (a >= 2 && a < TI + 2 && b >= 2 && b < TJ + 2) own(k, bv);
        }
        sb[t] = bv;
        sw[t] = wv;
        sx[t] = ((i + j) & 1) == 0 ? wv * bv : 0.f;
    }
    mg_stage_coef<TI, TJ, NT>(L, i0, j0, sc);
    __syncthreads();
    // black half-sweep over the 1-cell halo (reads red neighbours only)
    for (int t = threadIdx.x; t < D::CI * D::CJ; t += NT) {
        const int a = t / D::CJ + 1, b = t - (t / D::CJ) * D::CJ + 1;
        const int i = i0 + a - 2, j = j0 + b - 2;
        if (((i + j) & 1) == 0) continue;
        const int u = a * D::AJ + b;
        sx[u] = fmaf(sw[u], sb[u] - mg_ax_smem<TI, TJ>(sx, sc, L.lap, a, b), sx[u]);
    }
    __syncthreads();
    // owned cells: write x; aggregates: restricted residual
    for (int t = threadIdx.x; t < TI * TJ; t += NT) {
        const int a = t / TJ, b = t - a * TJ;
        const int i = i0 + a, j = j0 + b;
        if (i < L.NX && j < L.NY) xout[i * L.NY + j] = sx[(a + 2) * D::AJ + b + 2];
    }
    for (int t = threadIdx.x; t < (TI / 2) * (TJ / 2); t += NT) {
        const int ag = t / (TJ / 2), bg = t - ag * (TJ / 2);
        const int I = (i0 >> 1) + ag, J = (j0 >> 1) + bg;
        if (I >= NXc || J >= NYc) continue;
        float s = 0.f;
#pragma unroll
        for (int di = 0; di < 2; ++di)
#pragma unroll
            for (int dj = 0; dj < 2; ++dj) {
                const int a = 2 * ag + di + 2, b = 2 * bg + dj + 2;
                const int i = i0 + a - 2, j = j0 + b - 2;
                if (i >= L.NX || j >= L.NY) continue;
                const int tc = (a - 1) * D::CJ + (b - 1);
                const bool linked = sc[1][tc] != 0.f || sc[2][tc] != 0.f || sc[3][tc] != 0.f || sc[4][tc] != 0.f;
                if (!linked) continue;
                s += sb[a * D::AJ + b] - mg_ax_smem<TI, TJ>(sx, sc, L.lap, a, b);
            }
        bc[I * NYc + J] = s;
    }
}

template <int TI, int TJ, int NT, class BSrc, class Own>
__device__ __forceinline__ void mg_up_tile(const MgLvl& L, const float* __restrict__ xpre,
                                           const float* __restrict__ xc, int NYc, float alpha, const BSrc& bsrc,
                                           const Own& own, float* __restrict__ xout) {
    using D = MgTileDims<TI, TJ>;
    __shared__ float sx[D::AI * D::AJ];
    __shared__ float sb[D::CI * D::CJ], sw[D::CI * D::CJ];
    __shared__ float sc[5][D::CI * D::CJ];
    const int i0 = blockIdx.y * TI, j0 = blockIdx.x * TJ;
    // prolongation over the 2-cell halo
    for (int t = threadIdx.x; t < D::AI * D::AJ; t += NT) {
        const int a = t / D::AJ, b = t - a * D::AJ;
        const int i = i0 + a - 2, j = j0 + b - 2;
        float xv = 0.f;
        if (i >= 0 && i < L.NX && j >= 0 && j < L.NY) {
            const int k = i * L.NY + j;
            xv = __ldg(xpre + k);
            if (!__ldg(L.iso + k)) xv = fmaf(alpha, __ldg(xc + (i >> 1) * NYc + (j >> 1)), xv);
        }
        sx[t] = xv;
    }
    for (int t = threadIdx.x; t < D::CI * D::CJ; t += NT) {
        const int a = t / D::CJ, b = t - a * D::CJ;
        const int i = i0 + a - 1, j = j0 + b - 1;
        float bv = 0.f, wv = 0.f;
        if (i >= 0 && i < L.NX && j >= 0 && j < L.NY) {
            const int k = i * L.NY + j;
            bv = bsrc(k);
            wv = __ldg(L.winv + k);
        }
        sb[t] = bv;
        sw[t] = wv;
    }
    mg_stage_coef<TI, TJ, NT>(L, i0, j0, sc);
    __syncthreads();
    // black half-sweep over the 1-cell halo
    for (int t = threadIdx.x; t < D::CI * D::CJ; t += NT) {
        const int a = t / D::CJ + 1, b = t - (t / D::CJ) * D::CJ + 1;
        const int i = i0 + a - 2, j = j0 + b - 2;
        if (((i + j) & 1) == 0) continue;
        const int u = a * D::AJ + b;
        sx[u] = fmaf(sw[t], sb[t] - mg_ax_smem<TI, TJ>(sx, sc, L.lap, a, b), sx[u]);
    }
    __syncthreads();
    // red half-sweep on the owned cells, then write
    for (int t = threadIdx.x; t < TI * TJ; t += NT) {
        const int a = t / TJ + 2, b = t - (t / TJ) * TJ + 2;
        const int i = i0 + a - 2, j = j0 + b - 2;
        if (i >= L.NX || j >= L.NY) continue;
        const int u = a * D::AJ + b;
        const int tc = (a - 1) * D::CJ + (b - 1);
        float xv = sx[u];
        if (((i + j) & 1) == 0) xv = fmaf(sw[tc], sb[tc] - mg_ax_smem<TI, TJ>(sx, sc, L.lap, a, b), xv);
        const int k = i * L.NY + j;
        xout[k] = xv;
        own(k, xv, sb[tc]);
    }
}

}  // namespace kc
