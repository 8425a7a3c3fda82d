// Shared device helpers for libkarman_gb300: error reporting, deterministic
// block reductions and the "last block finalises" ticket.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>
#include <utility>
#include "karman_gb300.h"

namespace kc {

constexpr int kWarp = 32;
constexpr unsigned kFull = 0xffffffffu;

// ---- host-side error bookkeeping (thread local message) -------------------
void set_error(const char* fmt, ...);
int cuda_status(cudaError_t e, const char* what);
#define KC_CUDA(call)                                              \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return ::kc::cuda_status(e_, #call); \
    } while (0)
// Process-wide count of kernels this library has launched (kc_launch_count).
void count_launches(long long n);
#define KC_LAUNCH_CHECK_NC(what)                                   \
    do {                                                           \
        cudaError_t e_ = cudaGetLastError();                       \
        if (e_ != cudaSuccess) return ::kc::cuda_status(e_, what); \
    } while (0)
#define KC_LAUNCH_CHECK(what)          \
    do {                               \
        ::kc::count_launches(1);       \
        KC_LAUNCH_CHECK_NC(what);      \
    } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// ---- programmatic dependent launch ---------------------------------------------
// Kernels of a dependent chain (the CG iteration and its V-cycle) start with
// pdl_wait(): it returns once the preceding grid has completed and its writes
// are visible (at once when the kernel was launched without the attribute),
// so it must come before any read of a predecessor's output.  pdl_trigger()
// lets the next grid's blocks be scheduled while this grid finishes.
// Invariant of the chain: every kernel in it calls pdl_wait() before
// pdl_trigger().  A grid therefore starts only once the grid two launches
// back has completed, and the multigrid tiles (k_mg_down / k_mg_up below
// level 0, k_pcc_down0 inside the iterations, k_pcc_up0) stage what launches
// further back wrote -- the hierarchy's weights and coefficients, a level's
// pre-smoothed iterate -- before their own wait.  A kernel added to the
// chain must keep that order.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

constexpr bool kUsePDL = true;

template <typename... KArgs, typename... Args>
inline cudaError_t launch_chain(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                                Args&&... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = kUsePDL ? at : nullptr;
    cfg.numAttrs = kUsePDL ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Small device -> host readbacks (solver state, residual norms) go through a
// per-thread pinned buffer: a copy into pageable memory is staged by the
// driver and serialises host threads that each drive their own stream.
// Copies `bytes` (<= 4096) from device src on stream s, waits, returns a
// pointer to the host copy (valid until this thread's next call), or null on
// a CUDA error (reported through set_error).
const void* readback(const void* src, size_t bytes, cudaStream_t s);
// While an object of this type lives, readbacks of the constructing thread
// copy into a static per-thread pageable buffer instead of the pinned one, so
// that no host memory is allocated for them (the allocation-free entry points
// use it; a pageable copy is slower but allocates nothing).
struct PageableReadbacks {
    PageableReadbacks();
    ~PageableReadbacks();
    PageableReadbacks(const PageableReadbacks&) = delete;
    PageableReadbacks& operator=(const PageableReadbacks&) = delete;
};
inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// binary64 -> binary32 with IEEE 754 round to nearest, ties to even, in
// integer arithmetic: on GB300 the FP64 pipe issues a few operations per SM
// per clock and the conversion instruction occupies it, while the integer
// pipes are idle in the FP64 stage kernels.  Results in the normal binary32
// range (biased binary64 exponent 897..1150) keep the top 23 fraction bits
// and round on the 29 dropped ones; a carry out of the fraction steps the
// exponent (up to infinity above the largest finite value, as RN does).
// Zeros, subnormal results, overflow, infinities and NaN take the hardware
// conversion.  Bit-identical to (float)x for every input.
__device__ __forceinline__ float f64_to_f32(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32);
    const unsigned e = (hi >> 20) & 0x7FFu;
    if (e - 897u > 1150u - 897u) return (float)x;
    const unsigned long long m = b & 0x000FFFFFFFFFFFFFull;
    unsigned r = ((e - 896u) << 23) | (unsigned)(m >> 29);
    const unsigned rem = (unsigned)(m & 0x1FFFFFFFull), half = 0x10000000u;
    r += (rem > half || (rem == half && (r & 1u))) ? 1u : 0u;
    return __uint_as_float(r | (hi & 0x80000000u));
}

// ---- warp / block reductions (fixed order => bitwise reproducible) --------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(kFull, v, o));
    return v;
}

// Sums NV values over the block; the result is valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV]) {
    __shared__ double sh[NV][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double s = warp_sum(v[q]);
        if (lane == 0) sh[q][w] = s;
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double s = lane < nw ? sh[q][lane] : 0.0;
            v[q] = warp_sum(s);
        }
    }
    __syncthreads();
}

template <int NV>
__device__ __forceinline__ void block_max(double (&v)[NV]) {
    __shared__ double sh[NV][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double s = warp_max(v[q]);
        if (lane == 0) sh[q][w] = s;
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double s = lane < nw ? sh[q][lane] : 0.0;
            v[q] = warp_max(s);
        }
    }
    __syncthreads();
}

// Every block calls this after writing its partials; returns true in exactly
// one block (the last to arrive), which then owns the final reduction and
// resets the ticket.  No block ever waits on another.
__device__ __forceinline__ bool arrive_last(unsigned* ticket, unsigned nblocks) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = atomicAdd(ticket, 1u);
        last = (t == nblocks - 1);
    }
    __syncthreads();
    if (last) __threadfence();
    return last;
}

// Fixed-order sum of partials[0..count) (stride between vectors: ld) for NV
// vectors, executed by one whole block; result valid in thread 0.
template <int NV>
__device__ __forceinline__ void reduce_partials(const double* partials, int ld, int count,
                                                double (&out)[NV]) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double s = 0.0;
        for (int i = threadIdx.x; i < count; i += blockDim.x)
            s += __ldcg(partials + q * ld + i);
        out[q] = s;
    }
    block_sum<NV>(out);
}

template <int NV>
__device__ __forceinline__ void reduce_partials_max(const double* partials, int ld, int count,
                                                    double (&out)[NV]) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double s = 0.0;
        for (int i = threadIdx.x; i < count; i += blockDim.x)
            s = fmax(s, __ldcg(partials + q * ld + i));
        out[q] = s;
    }
    block_max<NV>(out);
}

// Small reduction workspace used by assembly / correction kernels.
struct ReduceWs {
    unsigned ticket[8];
    double pad[4];
    double partials[4][4096];
};
constexpr int kReduceMaxBlocks = 4096;

// ---- inner-product accumulators -------------------------------------------------
// FP64 accumulation, and for FP32 vectors a double-float one: every product
// split exactly into a float pair (fmaf) and summed in float-pair arithmetic
// (about 48 bits), all on the FP32 pipe -- GB300 issues FP64 at a small
// fraction of the FP32 rate.
template <typename T>
struct Acc;
template <>
struct Acc<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double a, double b) { s = fma(a, b, s); }
};
struct DF {
    float hi, lo;
};
__device__ __forceinline__ DF df_add(DF a, DF b) {
    const float s = a.hi + b.hi;
    const float bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b.hi - bb);
    e += a.lo + b.lo;
    const float h = s + e;
    return {h, e - (h - s)};
}
template <>
struct Acc<float> {
    DF s{0.f, 0.f};
    __device__ __forceinline__ void add(float a, float b) {
        const float p = a * b;
        const float e = fmaf(a, b, -p);   // a*b == p + e exactly
        s = df_add(s, DF{p, e});
    }
};

// ---- bounded grid barrier for cooperative (persistent) kernels ---------------
// Blocks meet here between phases.  A wait gives up after kSpinLimit polls,
// raises err and every block leaves: no wait can run forever.
struct GridBar {
    unsigned count;
    unsigned gen;
    int err;
    int pad;
};
constexpr unsigned kSpinLimit = 1u << 22;   // ~0.5 s at 40 ns per poll: far beyond any healthy wait

// Every block of a cooperative launch calls this; returns false (and every
// later call returns false at once) if any wait gave up after `limit` polls.
__device__ __forceinline__ bool grid_sync(GridBar* bar, unsigned nb, unsigned limit = kSpinLimit) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* gen = &bar->gen;
        volatile int* err = &bar->err;
        const unsigned g = *gen;
        __threadfence();
        if (atomicAdd(&bar->count, 1u) == nb - 1) {
            atomicExch(&bar->count, 0u);
            __threadfence();
            atomicAdd(&bar->gen, 1u);
        } else {
            unsigned spins = 0;
            while (*gen == g) {
                if (*err) break;
                if (++spins > limit) {
                    atomicExch(&bar->err, 1);
                    break;
                }
                __nanosleep(40);
            }
        }
        __threadfence();
        ok = *err == 0;
    }
    __syncthreads();
    return ok;
}

}  // namespace kc
