// Kernels of the learned initial guess: a small U-Net on the pressure grid,
// trained and evaluated on the GPU.
//
// Activations are NHWC bfloat16 with the channel count padded to a multiple
// of 16 (the K step of the tensor-core MMA); weights of a 3x3 convolution are
// stored [tap = 3*ky + kx][Cout][Cin_pad] (the reduction index contiguous).
//
//   kc_unet_conv3x3      y = act(conv(x, W) + bias), implicit GEMM on the
//                        tensor cores: M = 64 pixels of one row per block,
//                        N = Cout, K = 9 taps x Cin_pad, BF16 operands, FP32
//                        accumulation (mma.sync.m16n8k16).  Used for the
//                        forward pass and, with flipped/transposed weights,
//                        for the data gradient of the backward pass.
//   kc_unet_conv3x3_wgrad dW[tap][co][ci] += sum_px dy[px][co] x[px+tap][ci],
//                        db[co] += sum_px dy[px][co] (FP32, tensor cores with
//                        M = Cout, N = 16 input channels, K = pixels).
//   pooling, upsampling + concatenation, 1x1 head, features, loss, Adam:
//                        pointwise kernels.
//
// The reference has no learned component; this is the "learned" row of the
// accelerated path (an initial guess for the p' solve).
#include "kc_common.cuh"
#include <cuda_bf16.h>

namespace kc {

typedef __nv_bfloat16 bf16;

// ---- tensor-core MMA (m16n8k16, bf16 x bf16 -> f32) ----------------------------
// Fragment layout (PTX ISA, mma.m16n8k16 .bf16): with g = lane / 4, t = lane % 4
//   A (16x16, row major): a0 = A[g][2t..2t+1], a1 = A[g+8][2t..], a2 = A[g][2t+8..], a3 = A[g+8][2t+8..]
//   B (16x8, K x N):      b0 = B[2t..2t+1][g],  b1 = B[2t+8..2t+9][g]
//   C (16x8, f32):        c0,c1 = C[g][2t..2t+1], c2,c3 = C[g+8][2t..2t+1]
__device__ __forceinline__ void mma_bf16(float (&c)[4], const unsigned (&a)[4], const unsigned (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ unsigned ld_u32(const bf16* p) { return *reinterpret_cast<const unsigned*>(p); }
__device__ __forceinline__ unsigned pack_bf16(bf16 lo, bf16 hi) {
    return (unsigned)__bfloat16_as_ushort(lo) | ((unsigned)__bfloat16_as_ushort(hi) << 16);
}

// ---- 3x3 convolution (forward / data gradient) ------------------------------------
constexpr int kConvPx = 64;        // pixels of one row per block (4 warps x 16)
constexpr int kConvThreads = 128;

// x [H][W][Cin] (Cin % 16 == 0); weight of (tap, co, ci) at w[tap * wtap + co * Cin + ci];
// y[px * ldy + co] for co < COUT (a channel group of a wider tensor when ldy > COUT).
// act: 0 none, 1 ReLU.  mask (nullable, same indexing as y): y *= (mask > 0) -- the
// ReLU derivative of the layer below when the kernel computes a data gradient.
template <int COUT>
__global__ void __launch_bounds__(kConvThreads)
    k_conv3x3(const bf16* __restrict__ x, int H, int W, int Cin, const bf16* __restrict__ w, long long wtap,
              const float* __restrict__ bias, int act, const bf16* __restrict__ mask, bf16* __restrict__ y,
              int ldy) {
    __shared__ __align__(16) bf16 sx[3][kConvPx + 2][16];
    __shared__ __align__(16) bf16 sw[9][COUT][16];
    const int i = blockIdx.y, j0 = blockIdx.x * kConvPx;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float acc[COUT / 8][4];
#pragma unroll
    for (int n = 0; n < COUT / 8; ++n) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;
    for (int c0 = 0; c0 < Cin; c0 += 16) {
        // stage 3 rows x 66 pixels x 16 channels (16-byte vectors: 2 per pixel), zero outside
        for (int e = threadIdx.x; e < 3 * (kConvPx + 2) * 2; e += kConvThreads) {
            const int half = e & 1, p = (e >> 1) % (kConvPx + 2), r = (e >> 1) / (kConvPx + 2);
            const int ii = i + r - 1, jj = j0 + p - 1;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (ii >= 0 && ii < H && jj >= 0 && jj < W)
                v = *reinterpret_cast<const uint4*>(x + ((size_t)ii * W + jj) * Cin + c0 + half * 8);
            *reinterpret_cast<uint4*>(&sx[r][p][half * 8]) = v;
        }
        for (int e = threadIdx.x; e < 9 * COUT * 2; e += kConvThreads) {
            const int half = e & 1, co = (e >> 1) % COUT, tap = (e >> 1) / COUT;
            *reinterpret_cast<uint4*>(&sw[tap][co][half * 8]) =
                *reinterpret_cast<const uint4*>(w + (size_t)tap * wtap + (size_t)co * Cin + c0 + half * 8);
        }
        __syncthreads();
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
            const int ky = tap / 3, kx = tap % 3;
            const int p = warp * 16 + g + kx;   // staged column of output pixel (warp*16 + g) shifted by kx-1
            unsigned a[4];
            a[0] = ld_u32(&sx[ky][p][2 * t]);
            a[1] = ld_u32(&sx[ky][p + 8][2 * t]);
            a[2] = ld_u32(&sx[ky][p][2 * t + 8]);
            a[3] = ld_u32(&sx[ky][p + 8][2 * t + 8]);
#pragma unroll
            for (int n = 0; n < COUT / 8; ++n) {
                unsigned b[2];
                b[0] = ld_u32(&sw[tap][n * 8 + g][2 * t]);
                b[1] = ld_u32(&sw[tap][n * 8 + g][2 * t + 8]);
                mma_bf16(acc[n], a, b);
            }
        }
        __syncthreads();
    }
    // epilogue: bias, activation, mask, bf16 store (two channels per 32-bit store)
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        const int jj = j0 + warp * 16 + g + half * 8;
        if (jj >= W) continue;
        const size_t o = ((size_t)i * W + jj) * ldy;
#pragma unroll
        for (int n = 0; n < COUT / 8; ++n) {
            const int co = n * 8 + 2 * t;
            float v0 = acc[n][2 * half], v1 = acc[n][2 * half + 1];
            if (bias) {
                v0 += bias[co];
                v1 += bias[co + 1];
            }
            if (act == 1) {
                v0 = fmaxf(v0, 0.f);
                v1 = fmaxf(v1, 0.f);
            }
            if (mask) {
                const unsigned m = ld_u32(mask + o + co);
                if (__bfloat162float(__ushort_as_bfloat16((unsigned short)(m & 0xffff))) <= 0.f) v0 = 0.f;
                if (__bfloat162float(__ushort_as_bfloat16((unsigned short)(m >> 16))) <= 0.f) v1 = 0.f;
            }
            *reinterpret_cast<unsigned*>(y + o + co) = pack_bf16(__float2bfloat16(v0), __float2bfloat16(v1));
        }
    }
}

// ---- weight gradient ---------------------------------------------------------------
// One block: a strip of kWgRows rows x 64 pixels, 16 input channels, all Cout.
// Warp w owns output channels [16w, 16w+16) (COUT/16 warps) and all 9 taps:
//   dW^T[tap][co][ci] = sum_px dy[px][co] * x[px + tap][ci]   (M = co, N = ci, K = px)
constexpr int kWgRows = 8;

template <int COUT>
__global__ void __launch_bounds__(COUT * 2)
    k_conv3x3_wgrad(const bf16* __restrict__ x, const bf16* __restrict__ dy, int H, int W, int Cin,
                    float* __restrict__ dw, float* __restrict__ db) {
    constexpr int NT = COUT * 2;   // COUT/16 warps
    __shared__ __align__(16) bf16 sdy[COUT][kConvPx + 8];        // transposed: [co][px]
    __shared__ __align__(16) bf16 sxt[3][16][kConvPx + 8];       // transposed: [row][ci][staged px], px 0 = j0-1
    const int c0 = blockIdx.z * 16, j0 = blockIdx.x * kConvPx, i0 = blockIdx.y * kWgRows;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float acc[9][2][4];
#pragma unroll
    for (int tp = 0; tp < 9; ++tp)
#pragma unroll
        for (int n = 0; n < 2; ++n) acc[tp][n][0] = acc[tp][n][1] = acc[tp][n][2] = acc[tp][n][3] = 0.f;
    float bacc = 0.f;   // bias gradient of channel threadIdx.x (threads < COUT), channel block 0 only
    for (int i = i0; i < min(i0 + kWgRows, H); ++i) {
        for (int e = threadIdx.x; e < kConvPx * COUT; e += NT) {
            const int co = e % COUT, p = e / COUT;
            const int jj = j0 + p;
            sdy[co][p] = jj < W ? dy[((size_t)i * W + jj) * COUT + co] : __float2bfloat16(0.f);
        }
        for (int e = threadIdx.x; e < 3 * 16 * (kConvPx + 2); e += NT) {
            const int ci = e % 16, p = (e / 16) % (kConvPx + 2), r = e / (16 * (kConvPx + 2));
            const int ii = i + r - 1, jj = j0 + p - 1;
            sxt[r][ci][p] = (ii >= 0 && ii < H && jj >= 0 && jj < W) ? x[((size_t)ii * W + jj) * Cin + c0 + ci]
                                                                     : __float2bfloat16(0.f);
        }
        __syncthreads();
        if (blockIdx.z == 0 && threadIdx.x < COUT)
            for (int p = 0; p < kConvPx; ++p) bacc += __bfloat162float(sdy[threadIdx.x][p]);
#pragma unroll
        for (int k0 = 0; k0 < kConvPx; k0 += 16) {
            unsigned a[4];
            const int co = warp * 16 + g;
            a[0] = ld_u32(&sdy[co][k0 + 2 * t]);
            a[1] = ld_u32(&sdy[co + 8][k0 + 2 * t]);
            a[2] = ld_u32(&sdy[co][k0 + 2 * t + 8]);
            a[3] = ld_u32(&sdy[co + 8][k0 + 2 * t + 8]);
#pragma unroll
            for (int tp = 0; tp < 9; ++tp) {
                const int ky = tp / 3, kx = tp % 3;
#pragma unroll
                for (int n = 0; n < 2; ++n) {
                    // B[k = px][n = ci]: staged column of px is px + kx (odd offsets: pack two halves)
                    const bf16* col = &sxt[ky][n * 8 + g][k0 + kx];
                    unsigned b[2];
                    b[0] = pack_bf16(col[2 * t], col[2 * t + 1]);
                    b[1] = pack_bf16(col[2 * t + 8], col[2 * t + 9]);
                    mma_bf16(acc[tp][n], a, b);
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int tp = 0; tp < 9; ++tp)
#pragma unroll
        for (int n = 0; n < 2; ++n) {
            const int co = warp * 16 + g, ci = c0 + n * 8 + 2 * t;
            float* d = dw + ((size_t)tp * COUT + co) * Cin + ci;
            atomicAdd(d, acc[tp][n][0]);
            atomicAdd(d + 1, acc[tp][n][1]);
            atomicAdd(d + 8 * (size_t)Cin, acc[tp][n][2]);
            atomicAdd(d + 8 * (size_t)Cin + 1, acc[tp][n][3]);
        }
    if (blockIdx.z == 0 && threadIdx.x < COUT && db) atomicAdd(db + threadIdx.x, bacc);
}

// W'[tap'][ci][co] = W[8 - tap'][co][ci]: the weights of the data-gradient convolution
__global__ void k_flip_weights(const bf16* __restrict__ w, int Cout, int Cin, int cin_real, bf16* __restrict__ wt) {
    const int n = 9 * Cout * Cin;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const int ci = e % Cin, co = (e / Cin) % Cout, tap = e / (Cin * Cout);
        // wt layout [tap][Cin (as output)][Cout (as input)]
        wt[((size_t)(8 - tap) * Cin + ci) * Cout + co] = ci < cin_real ? w[e] : __float2bfloat16(0.f);
    }
}

// ---- pooling / upsampling / concatenation ------------------------------------------
// 2x2 average pool: x [H][W][C] -> y [H/2][W/2][C] (H, W even)
__global__ void k_pool2(const bf16* __restrict__ x, int H, int W, int C, bf16* __restrict__ y) {
    const int Ho = H / 2, Wo = W / 2;
    const long long n = (long long)Ho * Wo * C;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % C);
        const long long px = e / C;
        const int jo = (int)(px % Wo), io = (int)(px / Wo);
        const size_t b = ((size_t)(2 * io) * W + 2 * jo) * C + c;
        const float s = __bfloat162float(x[b]) + __bfloat162float(x[b + C]) + __bfloat162float(x[b + (size_t)W * C]) +
                        __bfloat162float(x[b + (size_t)W * C + C]);
        y[e] = __float2bfloat16(0.25f * s);
    }
}
// gradient: dx[2io+di][2jo+dj][c] = dy[io][jo][c] / 4  (+= when accumulate)
__global__ void k_pool2_bwd(const bf16* __restrict__ dy, int H, int W, int C, bf16* __restrict__ dx, int accumulate) {
    const long long n = (long long)H * W * C;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % C);
        const long long px = e / C;
        const int j = (int)(px % W), i = (int)(px / W);
        float v = 0.25f * __bfloat162float(dy[((size_t)(i / 2) * (W / 2) + j / 2) * C + c]);
        if (accumulate) v += __bfloat162float(dx[e]);
        dx[e] = __float2bfloat16(v);
    }
}
// y [H][W][Cu + Cs] = concat(nearest-upsample(u [H/2][W/2][Cu]), s [H][W][Cs])
__global__ void k_up2_concat(const bf16* __restrict__ u, int Cu, const bf16* __restrict__ s, int Cs, int H, int W,
                             bf16* __restrict__ y) {
    const int C = Cu + Cs;
    const long long n = (long long)H * W * C;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % C);
        const long long px = e / C;
        const int j = (int)(px % W), i = (int)(px / W);
        y[e] = c < Cu ? u[((size_t)(i / 2) * (W / 2) + j / 2) * Cu + c] : s[px * Cs + (c - Cu)];
    }
}
// gradient of k_up2_concat: du = sum over the 2x2 children, ds (+)= dy[.., Cu:]
__global__ void k_up2_concat_bwd(const bf16* __restrict__ dy, int Cu, int Cs, int H, int W, bf16* __restrict__ du,
                                 bf16* __restrict__ ds, int accumulate_s) {
    const int C = Cu + Cs, Ho = H / 2, Wo = W / 2;
    const long long nu = (long long)Ho * Wo * Cu;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nu; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % Cu);
        const long long px = e / Cu;
        const int jo = (int)(px % Wo), io = (int)(px / Wo);
        const size_t b = ((size_t)(2 * io) * W + 2 * jo) * C + c;
        const float v = __bfloat162float(dy[b]) + __bfloat162float(dy[b + C]) + __bfloat162float(dy[b + (size_t)W * C]) +
                        __bfloat162float(dy[b + (size_t)W * C + C]);
        du[e] = __float2bfloat16(v);
    }
    const long long ns = (long long)H * W * Cs;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ns; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % Cs);
        const long long px = e / Cs;
        float v = __bfloat162float(dy[px * C + Cu + c]);
        if (accumulate_s) v += __bfloat162float(ds[e]);
        ds[e] = __float2bfloat16(v);
    }
}
// dy *= (y > 0): ReLU derivative in place
__global__ void k_relu_bwd(bf16* __restrict__ dy, const bf16* __restrict__ y, long long n) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        if (!(__bfloat162float(y[e]) > 0.f)) dy[e] = __float2bfloat16(0.f);
}

// ---- head (1x1, C -> 1, FP32 out), loss, features -------------------------------------
__global__ void k_head(const bf16* __restrict__ x, int C, long long npx, const float* __restrict__ w,
                       const float* __restrict__ b, float* __restrict__ out) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npx; p += (long long)gridDim.x * blockDim.x) {
        float s = b[0];
        for (int c = 0; c < C; ++c) s = fmaf(__bfloat162float(x[p * C + c]), w[c], s);
        out[p] = s;
    }
}
// given dout (FP32), dx = dout * w (bf16) and partials for dw, db (atomics)
__global__ void k_head_bwd(const bf16* __restrict__ x, int C, long long npx, const float* __restrict__ w,
                           const float* __restrict__ dout, bf16* __restrict__ dx, float* __restrict__ dw,
                           float* __restrict__ db) {
    float lw[64], lb = 0.f;
    for (int c = 0; c < C; ++c) lw[c] = 0.f;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npx; p += (long long)gridDim.x * blockDim.x) {
        const float d = dout[p];
        lb += d;
        for (int c = 0; c < C; ++c) {
            lw[c] = fmaf(d, __bfloat162float(x[p * C + c]), lw[c]);
            dx[p * C + c] = __float2bfloat16(d * w[c]);
        }
    }
    for (int c = 0; c < C; ++c) {
        float v = lw[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(dw + c, v);
    }
    for (int o = 16; o > 0; o >>= 1) lb += __shfl_down_sync(kFull, lb, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(db, lb);
}
// loss = sum_fluid (out - target)^2 / count; dout = 2 (out - target) / count on fluid cells, 0 elsewhere
__global__ void k_mse(const float* __restrict__ out, const float* __restrict__ target, const float* __restrict__ wgt,
                      long long npx, float inv_count, float* __restrict__ dout, float* __restrict__ loss) {
    float s = 0.f;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npx; p += (long long)gridDim.x * blockDim.x) {
        const float d = (out[p] - target[p]) * wgt[p];
        s = fmaf(d, d, s);
        dout[p] = 2.f * d * wgt[p] * inv_count;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(kFull, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s * inv_count);
}

// ---- Adam --------------------------------------------------------------------------
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       long long n, float lr, float b1, float b2, float eps, float c1, float c2,
                       bf16* __restrict__ p16) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float gi = g[e];
        const float mi = b1 * m[e] + (1.f - b1) * gi;
        const float vi = b2 * v[e] + (1.f - b2) * gi * gi;
        m[e] = mi;
        v[e] = vi;
        const float pi = p[e] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
        p[e] = pi;
        if (p16) p16[e] = __float2bfloat16(pi);
    }
}

__global__ void k_f32_to_bf16(const float* __restrict__ a, bf16* __restrict__ b, long long n) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        b[e] = __float2bfloat16(a[e]);
}

static inline unsigned pw(long long n) { return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, 8192)); }

}  // namespace kc

using namespace kc;

extern "C" {

int kc_unet_conv3x3(const void* x, int H, int W, int cin, const void* w, long long wtap, const float* bias,
                    int cout, int act, const void* mask, void* y, int ldy, void* stream) {
    if (!x || !w || !y || H < 1 || W < 1 || cin < 16 || cin % 16 || (cout != 16 && cout != 32 && cout != 48 && cout != 64))
        return set_error("kc_unet_conv3x3: bad arguments (H=%d W=%d cin=%d cout=%d; cin %% 16 == 0, cout in "
                         "{16,32,48,64})", H, W, cin, cout),
               KC_ERR_ARG;
    if (wtap == 0) wtap = (long long)cout * cin;
    if (ldy == 0) ldy = cout;
    if (ldy < cout || ldy % 2 || wtap % 8 || wtap < (long long)cout * cin)
        return set_error("kc_unet_conv3x3: ldy=%d, wtap=%lld", ldy, wtap), KC_ERR_ARG;
    if (((uintptr_t)x | (uintptr_t)w) & 15) return set_error("kc_unet_conv3x3: x and w must be 16-byte aligned"), KC_ERR_ARG;
    if (((uintptr_t)y | (uintptr_t)mask) & 3) return set_error("kc_unet_conv3x3: y and mask must be 4-byte aligned"), KC_ERR_ARG;
    const dim3 grid((W + kConvPx - 1) / kConvPx, H);
    cudaStream_t s = as_stream(stream);
    const bf16 *xb = (const bf16*)x, *wb = (const bf16*)w, *mb = (const bf16*)mask;
    bf16* yb = (bf16*)y;
    switch (cout) {
        case 16: k_conv3x3<16><<<grid, kConvThreads, 0, s>>>(xb, H, W, cin, wb, wtap, bias, act, mb, yb, ldy); break;
        case 32: k_conv3x3<32><<<grid, kConvThreads, 0, s>>>(xb, H, W, cin, wb, wtap, bias, act, mb, yb, ldy); break;
        case 48: k_conv3x3<48><<<grid, kConvThreads, 0, s>>>(xb, H, W, cin, wb, wtap, bias, act, mb, yb, ldy); break;
        default: k_conv3x3<64><<<grid, kConvThreads, 0, s>>>(xb, H, W, cin, wb, wtap, bias, act, mb, yb, ldy); break;
    }
    KC_LAUNCH_CHECK("k_conv3x3");
    return KC_OK;
}

int kc_unet_conv3x3_wgrad(const void* x, const void* dy, int H, int W, int cin, int cout, float* dw, float* db,
                          void* stream) {
    if (!x || !dy || !dw || H < 1 || W < 1 || cin < 16 || cin % 16 || (cout != 16 && cout != 32 && cout != 48 && cout != 64))
        return set_error("kc_unet_conv3x3_wgrad: bad arguments"), KC_ERR_ARG;
    const dim3 grid((W + kConvPx - 1) / kConvPx, (H + kWgRows - 1) / kWgRows, cin / 16);
    cudaStream_t s = as_stream(stream);
    const bf16 *xb = (const bf16*)x, *db16 = (const bf16*)dy;
    switch (cout) {
        case 16: k_conv3x3_wgrad<16><<<grid, 32, 0, s>>>(xb, db16, H, W, cin, dw, db); break;
        case 32: k_conv3x3_wgrad<32><<<grid, 64, 0, s>>>(xb, db16, H, W, cin, dw, db); break;
        case 48: k_conv3x3_wgrad<48><<<grid, 96, 0, s>>>(xb, db16, H, W, cin, dw, db); break;
        default: k_conv3x3_wgrad<64><<<grid, 128, 0, s>>>(xb, db16, H, W, cin, dw, db); break;
    }
    KC_LAUNCH_CHECK("k_conv3x3_wgrad");
    return KC_OK;
}

int kc_unet_flip_weights(const void* w, int cout, int cin, int cin_real, void* wt, void* stream) {
    if (!w || !wt || cout < 1 || cin < 1) return set_error("kc_unet_flip_weights: bad arguments"), KC_ERR_ARG;
    k_flip_weights<<<pw(9ll * cout * cin), 256, 0, as_stream(stream)>>>((const bf16*)w, cout, cin, cin_real, (bf16*)wt);
    KC_LAUNCH_CHECK("k_flip_weights");
    return KC_OK;
}

int kc_unet_pool2(const void* x, int H, int W, int C, void* y, void* stream) {
    if (!x || !y || H % 2 || W % 2) return set_error("kc_unet_pool2: H, W must be even"), KC_ERR_ARG;
    k_pool2<<<pw((long long)H * W * C / 4), 256, 0, as_stream(stream)>>>((const bf16*)x, H, W, C, (bf16*)y);
    KC_LAUNCH_CHECK("k_pool2");
    return KC_OK;
}

int kc_unet_pool2_bwd(const void* dy, int H, int W, int C, void* dx, int accumulate, void* stream) {
    if (!dy || !dx || H % 2 || W % 2) return set_error("kc_unet_pool2_bwd: H, W must be even"), KC_ERR_ARG;
    k_pool2_bwd<<<pw((long long)H * W * C), 256, 0, as_stream(stream)>>>((const bf16*)dy, H, W, C, (bf16*)dx,
                                                                           accumulate);
    KC_LAUNCH_CHECK("k_pool2_bwd");
    return KC_OK;
}

int kc_unet_up2_concat(const void* u, int cu, const void* s, int cs, int H, int W, void* y, void* stream) {
    if (!u || !s || !y || H % 2 || W % 2) return set_error("kc_unet_up2_concat: H, W must be even"), KC_ERR_ARG;
    k_up2_concat<<<pw((long long)H * W * (cu + cs)), 256, 0, as_stream(stream)>>>((const bf16*)u, cu, (const bf16*)s,
                                                                                   cs, H, W, (bf16*)y);
    KC_LAUNCH_CHECK("k_up2_concat");
    return KC_OK;
}

int kc_unet_up2_concat_bwd(const void* dy, int cu, int cs, int H, int W, void* du, void* ds, int accumulate_s,
                           void* stream) {
    if (!dy || !du || !ds || H % 2 || W % 2) return set_error("kc_unet_up2_concat_bwd: H, W must be even"), KC_ERR_ARG;
    k_up2_concat_bwd<<<pw((long long)H * W * (cu + cs)), 256, 0, as_stream(stream)>>>(
        (const bf16*)dy, cu, cs, H, W, (bf16*)du, (bf16*)ds, accumulate_s);
    KC_LAUNCH_CHECK("k_up2_concat_bwd");
    return KC_OK;
}

int kc_unet_relu_bwd(void* dy, const void* y, long long n, void* stream) {
    if (!dy || !y || n < 0) return set_error("kc_unet_relu_bwd: bad arguments"), KC_ERR_ARG;
    k_relu_bwd<<<pw(n), 256, 0, as_stream(stream)>>>((bf16*)dy, (const bf16*)y, n);
    KC_LAUNCH_CHECK("k_relu_bwd");
    return KC_OK;
}

int kc_unet_head(const void* x, int C, long long npx, const float* w, const float* b, float* out, void* stream) {
    if (!x || !w || !b || !out || C < 1 || C > 64) return set_error("kc_unet_head: bad arguments"), KC_ERR_ARG;
    k_head<<<pw(npx), 256, 0, as_stream(stream)>>>((const bf16*)x, C, npx, w, b, out);
    KC_LAUNCH_CHECK("k_head");
    return KC_OK;
}

int kc_unet_head_bwd(const void* x, int C, long long npx, const float* w, const float* dout, void* dx, float* dw,
                     float* db, void* stream) {
    if (!x || !w || !dout || !dx || !dw || !db || C < 1 || C > 64)
        return set_error("kc_unet_head_bwd: bad arguments"), KC_ERR_ARG;
    k_head_bwd<<<pw(npx), 256, 0, as_stream(stream)>>>((const bf16*)x, C, npx, w, dout, (bf16*)dx, dw, db);
    KC_LAUNCH_CHECK("k_head_bwd");
    return KC_OK;
}

int kc_unet_mse(const float* out, const float* target, const float* weight, long long npx, float inv_count,
                float* dout, float* loss, void* stream) {
    if (!out || !target || !weight || !dout || !loss) return set_error("kc_unet_mse: bad arguments"), KC_ERR_ARG;
    k_mse<<<pw(npx), 256, 0, as_stream(stream)>>>(out, target, weight, npx, inv_count, dout, loss);
    KC_LAUNCH_CHECK("k_mse");
    return KC_OK;
}

int kc_unet_adam(float* p, const float* g, float* m, float* v, long long n, float lr, float b1, float b2, float eps,
                 int step, void* p_bf16, void* stream) {
    if (!p || !g || !m || !v || n < 0 || step < 1) return set_error("kc_unet_adam: bad arguments"), KC_ERR_ARG;
    const float c1 = 1.f / (1.f - powf(b1, (float)step)), c2 = 1.f / (1.f - powf(b2, (float)step));
    k_adam<<<pw(n), 256, 0, as_stream(stream)>>>(p, g, m, v, n, lr, b1, b2, eps, c1, c2, (bf16*)p_bf16);
    KC_LAUNCH_CHECK("k_adam");
    return KC_OK;
}

int kc_unet_to_bf16(const float* a, void* b, long long n, void* stream) {
    if (!a || !b || n < 0) return set_error("kc_unet_to_bf16: bad arguments"), KC_ERR_ARG;
    k_f32_to_bf16<<<pw(n), 256, 0, as_stream(stream)>>>(a, (bf16*)b, n);
    KC_LAUNCH_CHECK("k_f32_to_bf16");
    return KC_OK;
}

}  // extern "C"

// =====================================================================================
// Features of the p' system and the prediction -> initial guess map
// =====================================================================================
namespace kc {

// Per row i of the [NX][NY] p' grid: rowv[0][i] = sum_j b (fluid), rowv[1][i] = sum_j |aE| (fluid),
// rowv[2][i] = sum_j b^2, rowv[3][i] = sum_j d (d = -sum of links), rowv[4][i] = fluid count.
__global__ void k_feat_rows(const double* __restrict__ b, const float* __restrict__ c, long long cs, int NX, int NY,
                            double* __restrict__ rowv) {
    const int i = blockIdx.x;
    double v[5] = {0, 0, 0, 0, 0};
    for (int j = threadIdx.x; j < NY; j += blockDim.x) {
        const long long k = (long long)i * NY + j;
        const float w = c[cs + k], e = c[2 * cs + k], nn = c[3 * cs + k], s = c[4 * cs + k];
        if (w == 0.f && e == 0.f && nn == 0.f && s == 0.f) continue;
        const double bk = b[k];
        v[0] += bk;
        v[1] += -(double)e;
        v[2] += bk * bk;
        v[3] += -((double)w + e + nn + s);
        v[4] += 1.0;
    }
    block_sum<5>(v);
    if (threadIdx.x == 0)
        for (int q = 0; q < 5; ++q) rowv[(size_t)q * NX + i] = v[q];
}

// Inclusive prefix sum of v[0..n) over one block of kScanThreads threads (each
// thread a contiguous chunk, then a Hillis-Steele scan of the chunk totals);
// reverse = true sums from the end.  Fixed order: bitwise reproducible.
constexpr int kScanThreads = 1024;
__device__ void block_scan(double* v, int n, bool reverse) {
    __shared__ double tot[kScanThreads];
    const int per = (n + kScanThreads - 1) / kScanThreads, t = threadIdx.x;
    const int lo = t * per, hi = min(n, lo + per);
    auto at = [&](int q) -> double& { return v[reverse ? n - 1 - q : q]; };
    double s = 0;
    for (int q = lo; q < hi; ++q) s += at(q);
    tot[t] = s;
    __syncthreads();
    for (int o = 1; o < kScanThreads; o <<= 1) {
        const double add = t >= o ? tot[t - o] : 0.0;
        __syncthreads();
        tot[t] += add;
        __syncthreads();
    }
    double run = t > 0 ? tot[t - 1] : 0.0;
    for (int q = lo; q < hi; ++q) {
        run += at(q);
        at(q) = run;
    }
    __syncthreads();
}

// One block: sc[0] = s_b, sc[1] = mean d, sc[2] = s_p, sc[3] = fluid count; p1[i] = P1(i)
// (the 1-D solution: F(i) = sum_{i'<=i} B(i'), P1(i) = sum_{i'>=i} F(i') / A(i')).
// scratch: NX doubles
__global__ void __launch_bounds__(kScanThreads)
    k_feat_scan(const double* __restrict__ rowv, int NX, double* __restrict__ p1, double* __restrict__ scratch,
                double* __restrict__ sc) {
    double g[3] = {0, 0, 0};
    for (int i = threadIdx.x; i < NX; i += blockDim.x) {
        g[0] += rowv[2 * (size_t)NX + i];
        g[1] += rowv[3 * (size_t)NX + i];
        g[2] += rowv[4 * (size_t)NX + i];
        scratch[i] = rowv[i];
    }
    block_sum<3>(g);
    __shared__ double G[3];
    if (threadIdx.x == 0)
        for (int q = 0; q < 3; ++q) G[q] = g[q];
    __syncthreads();
    block_scan(scratch, NX, false);                       // F(i)
    for (int i = threadIdx.x; i < NX; i += blockDim.x) {
        const double A = rowv[(size_t)NX + i];
        p1[i] = A > 0 ? scratch[i] / A : 0.0;
    }
    __syncthreads();
    block_scan(p1, NX, true);                             // P1(i)
    double pp[1] = {0};
    for (int i = threadIdx.x; i < NX; i += blockDim.x) pp[0] += p1[i] * p1[i] * rowv[4 * (size_t)NX + i];
    block_sum<1>(pp);
    if (threadIdx.x == 0) {
        const double n = G[2] > 0 ? G[2] : 1.0;
        sc[0] = G[0] > 0 ? sqrt(G[0] / n) : 1e-300;
        sc[1] = G[1] > 0 ? G[1] / n : 1e-300;
        sc[2] = pp[0] > 0 ? sqrt(pp[0] / n) : 1e-300;
        sc[3] = G[2];
    }
}

// feat[H][W][16] (bf16): channels 0..3 = b/s_b, fluid, d/mean d, P1/s_p on fluid cells, 0 elsewhere
// (padding included); fluid[NX][NY] (nullable, FP32 0/1).
__global__ void k_feat_fill(const double* __restrict__ b, const float* __restrict__ c, long long cs, int NX, int NY,
                            const double* __restrict__ p1, const double* __restrict__ sc, int H, int W,
                            bf16* __restrict__ feat, float* __restrict__ fluid) {
    const double isb = 1.0 / sc[0], idm = 1.0 / sc[1], isp = 1.0 / sc[2];
    const long long n = (long long)H * W;
    for (long long px = blockIdx.x * (long long)blockDim.x + threadIdx.x; px < n; px += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(px / W), j = (int)(px % W);
        float f[4] = {0.f, 0.f, 0.f, 0.f};
        if (i < NX && j < NY) {
            const long long k = (long long)i * NY + j;
            const float w = c[cs + k], e = c[2 * cs + k], nn = c[3 * cs + k], s = c[4 * cs + k];
            const bool fl = !(w == 0.f && e == 0.f && nn == 0.f && s == 0.f);
            if (fl) {
                f[0] = (float)(b[k] * isb);
                f[1] = 1.f;
                f[2] = (float)(-((double)w + e + nn + s) * idm);
                f[3] = (float)(p1[i] * isp);
            }
            if (fluid) fluid[k] = fl ? 1.f : 0.f;
        }
        uint4 lo, hi = make_uint4(0, 0, 0, 0);
        lo.x = pack_bf16(__float2bfloat16(f[0]), __float2bfloat16(f[1]));
        lo.y = pack_bf16(__float2bfloat16(f[2]), __float2bfloat16(f[3]));
        lo.z = lo.w = 0;
        uint4* o = reinterpret_cast<uint4*>(feat + px * 16);
        o[0] = lo;
        o[1] = hi;
    }
}

// x0[i][j] = s_p * bilinear 2x upsampling of out[H/2][W/2] at (i, j), fluid cells only (0 elsewhere).
// The coarse value of cell (I, J) sits at fine position (2I + 1/2, 2J + 1/2).
__global__ void k_guess_up2(const float* __restrict__ out, int Hh, int Wh, const float* __restrict__ c, long long cs,
                            int NX, int NY, const double* __restrict__ sc, double* __restrict__ x0) {
    const double sp = sc[2];
    const long long n = (long long)NX * NY;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / NY), j = (int)(k % NY);
        const bool fl = !(c[cs + k] == 0.f && c[2 * cs + k] == 0.f && c[3 * cs + k] == 0.f && c[4 * cs + k] == 0.f);
        if (!fl) {
            x0[k] = 0.0;
            continue;
        }
        const float fi = 0.5f * i - 0.25f, fj = 0.5f * j - 0.25f;
        int i0 = (int)floorf(fi), j0 = (int)floorf(fj);
        const float ti = fi - i0, tj = fj - j0;
        const int i1 = min(max(i0 + 1, 0), Hh - 1), j1 = min(max(j0 + 1, 0), Wh - 1);
        i0 = min(max(i0, 0), Hh - 1);
        j0 = min(max(j0, 0), Wh - 1);
        const float v = (1 - ti) * ((1 - tj) * out[(size_t)i0 * Wh + j0] + tj * out[(size_t)i0 * Wh + j1]) +
                        ti * ((1 - tj) * out[(size_t)i1 * Wh + j0] + tj * out[(size_t)i1 * Wh + j1]);
        x0[k] = sp * (double)v;
    }
}

// target[H/2][W/2] = 2x2 average of p'/s_p over the fluid cells of each block, weight = fluid share
__global__ void k_target_down2(const double* __restrict__ p, const float* __restrict__ c, long long cs, int NX, int NY,
                               const double* __restrict__ sc, int Hh, int Wh, float* __restrict__ tgt,
                               float* __restrict__ wgt) {
    const double isp = 1.0 / sc[2];
    const long long n = (long long)Hh * Wh;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int I = (int)(e / Wh), J = (int)(e % Wh);
        double s = 0;
        int m = 0;
        for (int di = 0; di < 2; ++di)
            for (int dj = 0; dj < 2; ++dj) {
                const int i = 2 * I + di, j = 2 * J + dj;
                if (i >= NX || j >= NY) continue;
                const long long k = (long long)i * NY + j;
                if (c[cs + k] == 0.f && c[2 * cs + k] == 0.f && c[3 * cs + k] == 0.f && c[4 * cs + k] == 0.f) continue;
                s += p[k];
                ++m;
            }
        tgt[e] = m ? (float)(s / m * isp) : 0.f;
        wgt[e] = 0.25f * m;
    }
}

}  // namespace kc

extern "C" {

size_t kc_unet_features_ws_bytes(int NX) { return (size_t)(7 * (size_t)NX + 8) * sizeof(double); }

int kc_unet_features(const double* b, const float* coef32, int NX, int NY, int H, int W, void* feat, float* fluid,
                     double* scales, void* ws, size_t ws_bytes, void* stream) {
    if (!b || !coef32 || !feat || !scales || NX < 1 || NY < 1 || H < NX || W < NY)
        return set_error("kc_unet_features: bad arguments"), KC_ERR_ARG;
    if (!ws || ws_bytes < kc_unet_features_ws_bytes(NX))
        return set_error("kc_unet_features: workspace %zu < %zu", ws_bytes, kc_unet_features_ws_bytes(NX)),
               KC_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    double* rowv = (double*)ws;
    double* p1 = rowv + 5 * (size_t)NX;
    double* scratch = p1 + NX;
    const long long cs = (long long)NX * NY;
    k_feat_rows<<<NX, 256, 0, s>>>(b, coef32, cs, NX, NY, rowv);
    k_feat_scan<<<1, kScanThreads, 0, s>>>(rowv, NX, p1, scratch, scales);
    k_feat_fill<<<pw((long long)H * W), 256, 0, s>>>(b, coef32, cs, NX, NY, p1, scales, H, W, (bf16*)feat, fluid);
    KC_LAUNCH_CHECK("features");
    count_launches(2);
    return KC_OK;
}

int kc_unet_guess_up2(const float* out, int Hh, int Wh, const float* coef32, int NX, int NY, const double* scales,
                      double* x0, void* stream) {
    if (!out || !coef32 || !scales || !x0 || 2 * Hh < NX || 2 * Wh < NY)
        return set_error("kc_unet_guess_up2: bad arguments"), KC_ERR_ARG;
    k_guess_up2<<<pw((long long)NX * NY), 256, 0, as_stream(stream)>>>(out, Hh, Wh, coef32, (long long)NX * NY, NX, NY,
                                                                        scales, x0);
    KC_LAUNCH_CHECK("k_guess_up2");
    return KC_OK;
}

int kc_unet_target_down2(const double* p, const float* coef32, int NX, int NY, const double* scales, int Hh, int Wh,
                         float* target, float* weight, void* stream) {
    if (!p || !coef32 || !scales || !target || !weight || 2 * Hh < NX || 2 * Wh < NY)
        return set_error("kc_unet_target_down2: bad arguments"), KC_ERR_ARG;
    k_target_down2<<<pw((long long)Hh * Wh), 256, 0, as_stream(stream)>>>(p, coef32, (long long)NX * NY, NX, NY, scales,
                                                                           Hh, Wh, target, weight);
    KC_LAUNCH_CHECK("k_target_down2");
    return KC_OK;
}

}  // extern "C"

// ---- native prediction: features -> U-Net forward -> upsampled guess ------------------------
// The fixed architecture (4 levels, 16/32/48/64 channels, two 3x3 convolutions
// with ReLU per level, 2x2 average pooling, nearest upsampling with skip
// concatenation, 1x1 head) run from C++, so that a caller without Python (the
// native SIMPLE step) can apply the network.  Parameters are one flat buffer,
// layer by layer: w [9][cout][cin] then b [cout], then the head's w [16] and
// b [1]; `params` is the FP32 copy (biases, head), `params16` the BF16 copy
// (convolution weights) at the same element offsets.
namespace {
struct UnetLayer {
    int cin, cout;
};
constexpr int kUnetLayers = 14;
constexpr UnetLayer kUnet[kUnetLayers] = {{16, 16}, {16, 16}, {16, 32}, {32, 32}, {32, 48}, {48, 48}, {48, 64},
                                          {64, 64}, {112, 48}, {48, 48}, {80, 32}, {32, 32}, {48, 16}, {16, 16}};

struct UnetPlan {
    int Hf, Wf, Hh, Wh;          // full-resolution feature grid, network grid
    size_t off[32];              // byte offsets in the workspace
    size_t total;
};
// workspace slots
enum { kSlotFull, kFluid, kScales, kFeatWs, kIn, kE0a, kS0, kX1, kE1a, kS1, kX2, kE2a, kS2, kX3, kB3a, kY3, kC2, kD2a,
       kY2, kC1, kD1a, kY1, kC0, kD0a, kY0, kOut, kSlots };

UnetPlan unet_plan(int NX, int NY) {
    UnetPlan P{};
    P.Hf = (NX + 15) / 16 * 16;
    P.Wf = (NY + 15) / 16 * 16;
    P.Hh = P.Hf / 2;
    P.Wh = P.Wf / 2;
    const size_t h0 = (size_t)P.Hh * P.Wh, h1 = h0 / 4, h2 = h0 / 16, h3 = h0 / 64, b2 = 2;
    const size_t bytes[kSlots] = {(size_t)P.Hf * P.Wf * 16 * b2, (size_t)NX * NY * 4, 4 * 8,
                                  kc_unet_features_ws_bytes(NX), h0 * 16 * b2, h0 * 16 * b2, h0 * 16 * b2,
                                  h1 * 16 * b2, h1 * 32 * b2, h1 * 32 * b2, h2 * 32 * b2, h2 * 48 * b2,
                                  h2 * 48 * b2, h3 * 48 * b2, h3 * 64 * b2, h3 * 64 * b2, h2 * 112 * b2,
                                  h2 * 48 * b2, h2 * 48 * b2, h1 * 80 * b2, h1 * 32 * b2, h1 * 32 * b2,
                                  h0 * 48 * b2, h0 * 16 * b2, h0 * 16 * b2, h0 * 4};
    size_t o = 0;
    for (int q = 0; q < kSlots; ++q) {
        P.off[q] = o;
        o = align256(o + bytes[q]);
    }
    P.total = o;
    return P;
}
}  // namespace

extern "C" {

long long kc_unet_param_count(void) {
    long long n = 0;
    for (const auto& l : kUnet) n += 9ll * l.cout * l.cin + l.cout;
    return n + 16 + 1;
}

size_t kc_unet_predict_ws_bytes(int NX, int NY) {
    if (NX < 1 || NY < 1) return 0;
    return unet_plan(NX, NY).total;
}

int kc_unet_predict(const kc_unet_net* net, const double* b, const float* coef32, double* x0, void* stream) {
    if (!net || !net->params || !net->params16 || !b || !coef32 || !x0)
        return set_error("kc_unet_predict: null argument"), KC_ERR_ARG;
    const int NX = net->NX, NY = net->NY;
    if (NX < 2 || NY < 2) return set_error("kc_unet_predict: grid %d x %d too small", NX, NY), KC_ERR_ARG;
    const UnetPlan P = unet_plan(NX, NY);
    if (!net->ws || net->ws_bytes < P.total || ((uintptr_t)net->ws & 255))
        return set_error("kc_unet_predict: workspace %zu bytes (256-aligned) < required %zu", net->ws_bytes, P.total),
               KC_ERR_WORKSPACE;
    char* w = (char*)net->ws;
    auto at = [&](int slot) { return (void*)(w + P.off[slot]); };
    int rc = kc_unet_features(b, coef32, NX, NY, P.Hf, P.Wf, at(kSlotFull), (float*)at(kFluid), (double*)at(kScales),
                              at(kFeatWs), kc_unet_features_ws_bytes(NX), stream);
    if (rc) return rc;
    rc = kc_unet_pool2(at(kSlotFull), P.Hf, P.Wf, 16, at(kIn), stream);
    if (rc) return rc;
    // parameter offsets, in elements, layer by layer
    long long wo[kUnetLayers], bo[kUnetLayers], o = 0;
    for (int l = 0; l < kUnetLayers; ++l) {
        wo[l] = o;
        o += 9ll * kUnet[l].cout * kUnet[l].cin;
        bo[l] = o;
        o += kUnet[l].cout;
    }
    const long long head_w = o, head_b = o + 16;
    const float* pf = (const float*)net->params;
    const unsigned short* p16 = (const unsigned short*)net->params16;
    int dims[4][2] = {{P.Hh, P.Wh}, {P.Hh / 2, P.Wh / 2}, {P.Hh / 4, P.Wh / 4}, {P.Hh / 8, P.Wh / 8}};
    auto conv = [&](int l, int lvl, int sx, int sy) {
        return kc_unet_conv3x3(at(sx), dims[lvl][0], dims[lvl][1], kUnet[l].cin, p16 + wo[l], 0, pf + bo[l],
                               kUnet[l].cout, 1, nullptr, at(sy), 0, stream);
    };
    // encoder
    if ((rc = conv(0, 0, kIn, kE0a)) || (rc = conv(1, 0, kE0a, kS0))) return rc;
    if ((rc = kc_unet_pool2(at(kS0), dims[0][0], dims[0][1], 16, at(kX1), stream))) return rc;
    if ((rc = conv(2, 1, kX1, kE1a)) || (rc = conv(3, 1, kE1a, kS1))) return rc;
    if ((rc = kc_unet_pool2(at(kS1), dims[1][0], dims[1][1], 32, at(kX2), stream))) return rc;
    if ((rc = conv(4, 2, kX2, kE2a)) || (rc = conv(5, 2, kE2a, kS2))) return rc;
    if ((rc = kc_unet_pool2(at(kS2), dims[2][0], dims[2][1], 48, at(kX3), stream))) return rc;
    // bottleneck
    if ((rc = conv(6, 3, kX3, kB3a)) || (rc = conv(7, 3, kB3a, kY3))) return rc;
    // decoder
    if ((rc = kc_unet_up2_concat(at(kY3), 64, at(kS2), 48, dims[2][0], dims[2][1], at(kC2), stream))) return rc;
    if ((rc = conv(8, 2, kC2, kD2a)) || (rc = conv(9, 2, kD2a, kY2))) return rc;
    if ((rc = kc_unet_up2_concat(at(kY2), 48, at(kS1), 32, dims[1][0], dims[1][1], at(kC1), stream))) return rc;
    if ((rc = conv(10, 1, kC1, kD1a)) || (rc = conv(11, 1, kD1a, kY1))) return rc;
    if ((rc = kc_unet_up2_concat(at(kY1), 32, at(kS0), 16, dims[0][0], dims[0][1], at(kC0), stream))) return rc;
    if ((rc = conv(12, 0, kC0, kD0a)) || (rc = conv(13, 0, kD0a, kY0))) return rc;
    if ((rc = kc_unet_head(at(kY0), 16, (long long)P.Hh * P.Wh, pf + head_w, pf + head_b, (float*)at(kOut), stream)))
        return rc;
    return kc_unet_guess_up2((const float*)at(kOut), P.Hh, P.Wh, coef32, NX, NY, (const double*)at(kScales), x0,
                             stream);
}

}  // extern "C"
