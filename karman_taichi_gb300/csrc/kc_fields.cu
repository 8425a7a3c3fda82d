// Post-processing of the SIMPLE fields for output (karman_taichi.py:545-583):
// velocities interpolated to cell centres, the cell divergence, and the
// display canvases (3x nearest upsampling, each field scaled to [0, 1] by
// its own minimum and maximum).  The reference draws the canvases with
// ti.GUI; here they are plain device arrays that the host writes as CSV or
// image files (no graphics stack).
#include "kc_common.cuh"
#include <algorithm>

namespace kc {

constexpr int kPostThreads = 256;
constexpr int kPostMaxBlocks = 1024;
constexpr int kPostFields = 5;   // u_post, v_post, p, pcor, udiv (the order of the canvases)

struct PostWs {
    unsigned ticket;
    unsigned pad[3];
    double part[2 * kPostFields][kPostMaxBlocks];   // [min fields..., max fields...][block]
};

// block-wide minimum and maximum of one value per thread (result in thread 0)
__device__ __forceinline__ void block_min_max(double& lo, double& hi) {
    __shared__ double sl[32], sh[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = fmin(lo, __shfl_down_sync(kFull, lo, o));
        hi = fmax(hi, __shfl_down_sync(kFull, hi, o));
    }
    if (lane == 0) {
        sl[w] = lo;
        sh[w] = hi;
    }
    __syncthreads();
    if (w == 0) {
        lo = lane < nw ? sl[lane] : INFINITY;
        hi = lane < nw ? sh[lane] : -INFINITY;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo = fmin(lo, __shfl_down_sync(kFull, lo, o));
            hi = fmax(hi, __shfl_down_sync(kFull, hi, o));
        }
    }
    __syncthreads();
}

// u_post[i][j] = (u[i][j] + u[i+1][j]) / 2, v_post[i][j] = (v[i][j] + v[i][j+1]) / 2 over [nx+2][ny+2];
// udiv[i][j] = (u[i][j] - u[i+1][j]) dy + (v[i][j+1] - v[i][j]) dx on i in [1,nx], j in [1,ny]
// (other entries untouched, as in the reference); min / max of the five fields over [nx+2][ny+2]
// with the reference's starting values max = 0, min = 1e9 (scale_field, karman_taichi.py:573-583).
__global__ void __launch_bounds__(kPostThreads)
    k_post_cells(int nx, int ny, double dx, double dy, const double* __restrict__ u, const double* __restrict__ v,
                 const double* __restrict__ p, const double* __restrict__ pc, double* __restrict__ up,
                 double* __restrict__ vp, double* __restrict__ ud, PostWs* ws, double* __restrict__ minmax) {
    const int NX = nx + 2, NY = ny + 2;
    const long long n = (long long)NX * NY;
    double mn[kPostFields], mx[kPostFields];
#pragma unroll
    for (int f = 0; f < kPostFields; ++f) {
        mn[f] = 1.0e9;
        mx[f] = 0.0;
    }
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / NY), j = (int)(k % NY);
        const double uc = 0.5 * (u[(long long)i * NY + j] + u[(long long)(i + 1) * NY + j]);
        const double vc = 0.5 * (v[(long long)i * (NY + 1) + j] + v[(long long)i * (NY + 1) + j + 1]);
        up[k] = uc;
        vp[k] = vc;
        if (i >= 1 && i <= nx && j >= 1 && j <= ny) {
            const double d = (u[(long long)i * NY + j] - u[(long long)(i + 1) * NY + j]) * dy +
                             (v[(long long)i * (NY + 1) + j + 1] - v[(long long)i * (NY + 1) + j]) * dx;
            ud[k] = d;
        }
        const double f[kPostFields] = {uc, vc, p[k], pc[k], ud[k]};
#pragma unroll
        for (int q = 0; q < kPostFields; ++q) {
            mn[q] = fmin(mn[q], f[q]);
            mx[q] = fmax(mx[q], f[q]);
        }
    }
    // (each cell's udiv is written and read by the same thread, so the extremes see final values)
#pragma unroll
    for (int q = 0; q < kPostFields; ++q) {
        double lo = mn[q], hi = mx[q];
        block_min_max(lo, hi);
        if (threadIdx.x == 0) {
            ws->part[q][blockIdx.x] = lo;
            ws->part[kPostFields + q][blockIdx.x] = hi;
        }
    }
    if (!arrive_last(&ws->ticket, gridDim.x)) return;
    // last block: every thread folds a stride of the block partials (min / max are exact in any order)
    for (int q = 0; q < kPostFields; ++q) {
        double lo = 1.0e9, hi = 0.0;
        for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
            lo = fmin(lo, __ldcg(&ws->part[q][b]));
            hi = fmax(hi, __ldcg(&ws->part[kPostFields + q][b]));
        }
        block_min_max(lo, hi);
        if (threadIdx.x == 0) {
            minmax[2 * q] = lo;
            minmax[2 * q + 1] = hi;
        }
    }
    if (threadIdx.x == 0) ws->ticket = 0;
}

// disp[f][I][J] = (field_f[I/3][J/3] - min_f) / (max_f - min_f + 1e-9), f = u_post, v_post, p, pcor, udiv:
// one thread per cell writes its 3x3 pixels of all five canvases
__global__ void k_post_disp(int nx, int ny, const double* __restrict__ up, const double* __restrict__ vp,
                            const double* __restrict__ p, const double* __restrict__ pc, const double* __restrict__ ud,
                            const double* __restrict__ minmax, float* __restrict__ disp) {
    const int NX = nx + 2, NY = ny + 2, DY = 3 * NY;
    const long long n = (long long)NX * NY, nd = 9 * n;
    double lo[kPostFields], sc[kPostFields];
#pragma unroll
    for (int f = 0; f < kPostFields; ++f) {
        lo[f] = minmax[2 * f];
        sc[f] = 1.0 / (minmax[2 * f + 1] - lo[f] + 1.0e-9);
    }
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / NY), j = (int)(k - (long long)i * NY);
        const double val[kPostFields] = {up[k], vp[k], p[k], pc[k], ud[k]};
#pragma unroll
        for (int f = 0; f < kPostFields; ++f) {
            const float d = (float)((val[f] - lo[f]) * sc[f]);
            float* o = disp + f * nd + (long long)(3 * i) * DY + 3 * j;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                o[(long long)a * DY] = d;
                o[(long long)a * DY + 1] = d;
                o[(long long)a * DY + 2] = d;
            }
        }
    }
}

}  // namespace kc

using namespace kc;

extern "C" {

size_t kc_post_process_ws_bytes(void) { return sizeof(PostWs); }

int kc_post_process(int nx, int ny, double dx, double dy, const double* u, const double* v, const double* p,
                    const double* pcor, double* u_post, double* v_post, double* udiv, double* minmax, float* disp,
                    void* ws, size_t ws_bytes, void* stream) {
    if (nx < 1 || ny < 1 || !u || !v || !p || !pcor || !u_post || !v_post || !udiv || !minmax)
        return set_error("kc_post_process: bad arguments"), KC_ERR_ARG;
    if (!ws || ws_bytes < sizeof(PostWs))
        return set_error("kc_post_process: workspace %zu < %zu", ws_bytes, sizeof(PostWs)), KC_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    const long long n = (long long)(nx + 2) * (ny + 2);
    const int nb = (int)std::max<long long>(1, std::min<long long>((n + kPostThreads - 1) / kPostThreads, kPostMaxBlocks));
    k_post_cells<<<nb, kPostThreads, 0, s>>>(nx, ny, dx, dy, u, v, p, pcor, u_post, v_post, udiv, (PostWs*)ws, minmax);
    KC_LAUNCH_CHECK("k_post_cells");
    if (disp) {
        k_post_disp<<<(unsigned)std::min<long long>((n + 255) / 256, 8192), 256, 0, s>>>(nx, ny, u_post, v_post, p,
                                                                                        pcor, udiv, minmax, disp);
        KC_LAUNCH_CHECK("k_post_disp");
    }
    return KC_OK;
}

}  // extern "C"
