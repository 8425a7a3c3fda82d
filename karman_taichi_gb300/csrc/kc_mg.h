// Internal interface of the multigrid preconditioner (kc_mg.cu) used by the
// preconditioned solver driver (kc_solver.cu).
#pragma once
#include <cuda_runtime.h>
#include "karman_gb300.h"
#include "kc_mg_tile.cuh"

namespace kc {

// level-0 tile of the fused cycle (also used by the preconditioned CG's fused
// level-0 kernels): 16 x 60 owned cells, 64-wide staged rows, 4 thread rows
constexpr int kMgTI0 = 16, kMgAJ0 = 64, kMgRY0 = 4, kMgTJ0 = kMgAJ0 - 4, kMgNT0 = kMgAJ0 * kMgRY0;
// coefficients of level 0 and the large levels staged in shared memory (true)
// or read through the read-only cache (false: 4 instead of 9 staged arrays,
// more resident blocks); staging measured faster on GB300 at 2050 x 514
// (p' solve 5.30 vs 5.53 ms per outer iteration)
constexpr bool kMgStagedLarge = true;
// tiles of the small levels: 8 rows, 32-wide staged rows (8 x 28 owned cells at one sweep)
constexpr int kMgTI1 = 8, kMgAJ1 = 32, kMgRY1 = 4, kMgNT1 = kMgAJ1 * kMgRY1;
// Levels >= 1 may take NU = 1..3 red-black sweeps before and after their
// coarse correction (kc_mg_opts.nu_coarse): the staged halo is 2 NU cells, so
// the large tiles keep 64-wide rows and lose rows as NU grows -- their nine
// staged [TI + 4 NU][64] arrays stay within 48 KB of static shared memory --
// and the small tiles keep 8 rows (24 x 32 at NU = 3: 24 KB).
constexpr int kMgMaxNu = 3;
__host__ __device__ constexpr int mg_big_ti(int nu) { return nu <= 1 ? kMgTI0 : (nu == 2 ? 12 : 8); }
__host__ __device__ constexpr int mg_tj(int AJ, int nu) { return AJ - 4 * nu; }
inline dim3 mg_tile_grid(int NX, int NY, int TI, int TJ) { return dim3((NY + TJ - 1) / TJ, (NX + TI - 1) / TI); }
inline int mg_fused_blocks0(long long n, int S) {
    const dim3 g = mg_tile_grid((int)(n / S), S, kMgTI0, kMgTJ0);
    return (int)(g.x * g.y);
}

struct MgLayout {
    int levels;
    int nx[KC_MG_MAX_LEVELS], ny[KC_MG_MAX_LEVELS];
    size_t off_winv[KC_MG_MAX_LEVELS], off_iso[KC_MG_MAX_LEVELS], off_coef[KC_MG_MAX_LEVELS];
    size_t off_b[KC_MG_MAX_LEVELS], off_x[KC_MG_MAX_LEVELS], off_t[KC_MG_MAX_LEVELS];
    size_t off_inv, off_flag;   // direct coarsest solve: dense inverse, failure flag
    size_t total;
};

MgLayout mg_layout(int NX, int NY, const kc_mg_opts* o);
// number of kernels one mg_enqueue launches for A
int mg_cycle_kernels(const kc_system* A, const kc_mg_opts* o);

// The fused cycle (one pre- and one post-sweep on level 0, nu_coarse on the
// levels below, at least two levels) split at level 0, for solvers that fuse their own pointwise work
// into the level-0 launches: the caller's level-0 DOWN writes x0pre and b1,
// mg_enqueue_coarse runs levels >= 1 and leaves their result in final1, the
// caller's level-0 UP prolongs final1 with alpha0.
struct MgFused {
    bool ok;
    MgLvl L0;
    float* x0pre;
    float* b1;
    const float* final1;
    int NX1, NY1;
    float alpha0;
};
MgFused mg_fused(const kc_system* A, void* ws, const kc_mg_opts* o);
int mg_enqueue_coarse(const kc_system* A, void* ws, const kc_mg_opts* o, const int* done, cudaStream_t s,
                      int* kernels);
int mg_setup(const kc_system* A, void* ws, size_t ws_bytes, const kc_mg_opts* o, cudaStream_t s);
// Enqueues z = M r; kernels return at once when *done != 0 (done may be
// null).  Launches are not counted: *kernels (if not null) receives their number.
int mg_enqueue(const kc_system* A, void* ws, const kc_mg_opts* o, const float* r, float* z, const int* done,
               cudaStream_t s, int* kernels = nullptr);

}  // namespace kc
