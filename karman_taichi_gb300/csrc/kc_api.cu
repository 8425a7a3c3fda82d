// Library-level entry points of libkarman_gb300: version, status strings,
// thread-local error text, device-to-device copies and FP64 -> FP32 copies.
#include "kc_common.cuh"
#include <algorithm>
#include <string>
#include <stdarg.h>
#include <stdio.h>
#include <atomic>

namespace kc {

static thread_local char g_err[512] = "";
static std::atomic<long long> g_launches{0};

void count_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int cuda_status(cudaError_t e, const char* what) {
    set_error("%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
    return KC_ERR_CUDA;
}

}  // namespace kc

namespace kc {

static thread_local int g_pageable_depth = 0;
PageableReadbacks::PageableReadbacks() { ++g_pageable_depth; }
PageableReadbacks::~PageableReadbacks() { --g_pageable_depth; }

const void* readback(const void* src, size_t bytes, cudaStream_t s) {
    struct Pinned {
        void* p = nullptr;
        ~Pinned() {
            if (p) cudaFreeHost(p);
        }
    };
    static thread_local Pinned buf;
    alignas(64) static thread_local unsigned char pageable[4096];
    if (bytes > 4096) {
        set_error("readback of %zu bytes exceeds the 4096-byte readback buffer", bytes);
        return nullptr;
    }
    if (g_pageable_depth > 0) {
        cudaError_t e = cudaMemcpyAsync(pageable, src, bytes, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            cuda_status(e, "readback");
            return nullptr;
        }
        return pageable;
    }
    if (!buf.p) {
        cudaError_t e = cudaMallocHost(&buf.p, 4096);
        if (e != cudaSuccess) {
            buf.p = nullptr;
            cuda_status(e, "cudaMallocHost (readback buffer)");
            return nullptr;
        }
    }
    cudaError_t e = cudaMemcpyAsync(buf.p, src, bytes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cuda_status(e, "readback");
        return nullptr;
    }
    return buf.p;
}

}  // namespace kc

extern "C" {

int kc_version(void) { return 10000; }

const char* kc_status_str(int status) {
    switch (status) {
        case KC_OK: return "converged";
        case KC_MAXITER: return "iteration cap reached";
        case KC_BREAKDOWN_RHO: return "breakdown: rho == 0";
        case KC_BREAKDOWN_OMEGA: return "breakdown: omega == 0";
        case KC_NONFINITE: return "non-finite value in the recurrence";
        case KC_STALL: return "residual stalled";
        case KC_ERR_ARG: return "invalid argument";
        case KC_ERR_CUDA: return "CUDA error";
        case KC_ERR_WORKSPACE: return "workspace missing, misaligned or too small";
        case KC_ERR_UNSUPPORTED: return "unsupported configuration";
        default: return "unknown status";
    }
}

const char* kc_last_error(void) { return kc::g_err; }

long long kc_launch_count(void) { return kc::g_launches.load(std::memory_order_relaxed); }

int kc_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int kc_copy(void* dst, const void* src, size_t bytes, void* stream) {
    if (!dst || !src) return kc::set_error("kc_copy: null pointer"), KC_ERR_ARG;
    if (bytes == 0) return KC_OK;
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, kc::as_stream(stream));
    if (e != cudaSuccess) return kc::cuda_status(e, "kc_copy");
    return KC_OK;
}

}  // extern "C"

namespace kc {
__global__ void __launch_bounds__(256) k_to_f32(const double* __restrict__ src, float* __restrict__ dst, long long n) {
    for (long long k = blockIdx.x * 256ll + threadIdx.x; k < n; k += (long long)gridDim.x * 256)
        dst[k] = f64_to_f32(src[k]);
}
}  // namespace kc

extern "C" {

int kc_to_f32(const double* src, float* dst, long long n, void* stream) {
    if (n < 0 || (n > 0 && (!src || !dst))) return kc::set_error("kc_to_f32: bad arguments"), KC_ERR_ARG;
    if (n == 0) return KC_OK;
    const long long blocks = std::min<long long>((n + 255) / 256, 152ll * 8);
    kc::k_to_f32<<<(unsigned)blocks, 256, 0, kc::as_stream(stream)>>>(src, dst, n);
    KC_LAUNCH_CHECK("k_to_f32");
    return KC_OK;
}

// sizeof of the ABI structs, for bindings that mirror them (ctypes, cgo, ...)
size_t kc_struct_size(const char* name) {
    if (!name) return 0;
    const std::string n(name);
    if (n == "kc_system") return sizeof(kc_system);
    if (n == "kc_solve_opts") return sizeof(kc_solve_opts);
    if (n == "kc_solve_info") return sizeof(kc_solve_info);
    if (n == "kc_mg_opts") return sizeof(kc_mg_opts);
    if (n == "kc_phys") return sizeof(kc_phys);
    if (n == "kc_karman") return sizeof(kc_karman);
    if (n == "kc_channel") return sizeof(kc_channel);
    if (n == "kc_channel_stats") return sizeof(kc_channel_stats);
    if (n == "kc_unet_net") return sizeof(kc_unet_net);
    if (n == "kc_flex_info") return sizeof(kc_flex_info);
    if (n == "kc_recycle_state") return sizeof(kc_recycle_state);
    return 0;
}
}  // extern "C"
