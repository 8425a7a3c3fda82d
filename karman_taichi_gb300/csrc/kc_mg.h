// Internal interface of the multigrid preconditioner (kc_mg.cu) used by the
// preconditioned solver driver (kc_solver.cu).
#pragma once
#include <cuda_runtime.h>
#include "karman_gb300.h"

namespace kc {

struct MgLayout {
    int levels;
    int nx[KC_MG_MAX_LEVELS], ny[KC_MG_MAX_LEVELS];
    size_t off_winv[KC_MG_MAX_LEVELS], off_iso[KC_MG_MAX_LEVELS], off_coef[KC_MG_MAX_LEVELS];
    size_t off_b[KC_MG_MAX_LEVELS], off_x[KC_MG_MAX_LEVELS], off_t[KC_MG_MAX_LEVELS];
    size_t total;
};

MgLayout mg_layout(int NX, int NY, const kc_mg_opts* o);
int mg_setup(const kc_system* A, void* ws, size_t ws_bytes, const kc_mg_opts* o, cudaStream_t s);
// Enqueues z = M r; kernels return at once when *done != 0 (done may be
// null).  Launches are not counted: *kernels (if not null) receives their number.
int mg_enqueue(const kc_system* A, void* ws, const kc_mg_opts* o, const float* r, float* z, const int* done,
               cudaStream_t s, int* kernels = nullptr);

}  // namespace kc
