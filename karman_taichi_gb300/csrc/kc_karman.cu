// karman_taichi.py assembled-matrix path, re-expressed as flat 5-point
// stencil planes (one thread per matrix row).
//
// The reference writes its matrices into persistent pointer-SNode fields with
// two sequential loops per fill (karman_taichi.py:162-248, 251-294, 297-339).
// Because the cell-type field ct never changes, the set of entries each row
// writes is the same on every call, so the final value of every stencil entry
// is a closed-form function of the current fields: start from 0 (never
// written), apply the first loop's branch, then the second loop's branch.
// Entries the second loop does not touch keep the first loop's value -- this
// reproduces the stale a_N link of the obstacle-wall rows (:231-239) and the
// un-cleared links of the outlet pin rows (:334-336) exactly.
//
// Plane slots by flat offset: 0 diagonal, 1 k-S, 2 k+S, 3 k+1, 4 k-1, where
// S = ny for u and p rows and S = ny+1 for v rows.  (The reference names the
// k+1 entry "as" and k-1 "an" because its j axis points south.)
//
// Compiled with -fmad=false so the coefficient arithmetic keeps the
// reference's operation order.
#include "kc_common.cuh"
#include <algorithm>

namespace kc {

struct KGeo {
    int nx, ny, NYu, NYv, NYp;
};
__host__ __device__ inline KGeo kgeo(const kc_karman& K) { return {K.nx, K.ny, K.ny + 2, K.ny + 3, K.ny + 2}; }

#define CT(a, b) ct[(long long)(a) * G.NYp + (b)]
#define U_(a, b) u[(long long)(a) * G.NYu + (b)]
#define V_(a, b) v[(long long)(a) * G.NYv + (b)]
#define P_(a, b) p[(long long)(a) * G.NYp + (b)]

// fill_Au (karman_taichi.py:162-248)
__global__ void k_karman_fill_u(kc_karman K, const int* ct, const double* u, const double* v, const double* p,
                                const double* u0, double* coef, double* bvec, double* Mvec) {
    const KGeo G = kgeo(K);
    const int nx = G.nx, ny = G.ny;
    const long long n = (long long)(nx + 1) * ny;
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = (int)(k / ny) + 1, j = (int)(k % ny) + 1;
    const double mu = K.mu, rho = K.rho, dx = K.dx, dy = K.dy, dt = K.dt;
    double c[5] = {0, 0, 0, 0, 0};
    double b = 0.0;
    // expressions shared by the branches
    auto as_ = [&]() { return -mu * dx / dy - rho * 0.5 * (V_(i - 1, j + 1) + V_(i, j + 1)) * dx; };
    auto aw_ = [&]() { return -mu * dy / dx - rho * 0.5 * (U_(i, j) + U_(i - 1, j)) * dy; };
    auto ae_ = [&]() { return -mu * dy / dx - (-rho * 0.5 * (U_(i, j) + U_(i + 1, j)) * dy); };
    auto an_ = [&]() { return -mu * dx / dy - (-rho * 0.5 * (V_(i - 1, j) + V_(i, j)) * dx); };
    auto bsrc = [&]() { return (P_(i - 1, j) - P_(i, j)) * dy + rho * dx * dy / dt * u0[(long long)i * G.NYu + j]; };
    // first loop
    if (CT(i - 1, j) == 1) {
        c[0] = 1.0;
        c[2] = -1.0;
        b = 0.0;
    } else if (CT(i, j) == 1) {
        c[0] = 1.0;
        c[1] = -1.0;
        b = 0.0;
    } else if ((CT(i, j) + CT(i, j - 1)) == 0) {
        c[3] = as_();
        c[1] = aw_();
        c[2] = ae_();
        c[0] = -c[3] - c[1] - c[2] + rho * dx * dy / dt + 2 * mu * dx / dy;
        b = bsrc();
    } else if ((CT(i, j) + CT(i, j + 1)) == 0) {
        c[4] = an_();
        c[1] = aw_();
        c[2] = ae_();
        c[0] = -c[4] - c[1] - c[2] + rho * dx * dy / dt + 2 * mu * dx / dy;
        b = bsrc();
    } else {
        c[4] = an_();
        c[3] = as_();
        c[1] = aw_();
        c[2] = ae_();
        c[0] = -c[4] - c[3] - c[1] - c[2] + rho * dx * dy / dt;
        b = bsrc();
    }
    const double M = c[0];
    // second loop: internal obstacle (i in [2, nx], j in [2, ny-1])
    if (i >= 2 && i <= nx && j >= 2 && j <= ny - 1) {
        const int s1 = CT(i - 1, j) + CT(i, j);
        if (s1 == 0 || s1 == 2) {
            c[1] = c[2] = c[3] = c[4] = 0.0;
            c[0] = 1.0;
            b = 0.0;
        } else if ((CT(i, j) + CT(i, j - 1)) == 0 || (CT(i - 1, j) + CT(i - 1, j - 1)) == 0) {
            c[3] = as_();
            c[1] = aw_();
            c[2] = ae_();
            c[0] = -c[3] - c[1] - c[2] + rho * dx * dy / dt + 2 * mu * dx / dy;
            b = bsrc();
        }
    }
#pragma unroll
    for (int q = 0; q < 5; ++q) coef[q * n + k] = c[q];
    bvec[k] = b;
    Mvec[k] = M;
}

// fill_Av (karman_taichi.py:251-294)
__global__ void k_karman_fill_v(kc_karman K, const int* ct, const double* u, const double* v, const double* p,
                                const double* v0, double* coef, double* bvec, double* Mvec) {
    const KGeo G = kgeo(K);
    const int nx = G.nx, ny = G.ny;
    const long long n = (long long)nx * (ny + 1);
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = (int)(k / (ny + 1)) + 1, j = (int)(k % (ny + 1)) + 1;
    const double mu = K.mu, rho = K.rho, dx = K.dx, dy = K.dy, dt = K.dt;
    double c[5] = {0, 0, 0, 0, 0};
    double b = 0.0;
    auto an_ = [&]() { return -mu * dx / dy - (-rho * 0.5 * (V_(i, j - 1) + V_(i, j)) * dx); };
    auto as_ = [&]() { return -mu * dx / dy - (rho * 0.5 * (V_(i, j + 1) + V_(i, j)) * dx); };
    auto ae_ = [&]() { return -mu * dy / dx - (-rho * 0.5 * (U_(i + 1, j - 1) + U_(i + 1, j)) * dy); };
    auto aw_ = [&]() { return -mu * dy / dx - (rho * 0.5 * (U_(i, j) + U_(i, j - 1)) * dy); };
    auto bsrc = [&]() { return (P_(i, j) - P_(i, j - 1)) * dx + rho * dx * dy / dt * v0[(long long)i * G.NYv + j]; };
    const int s = CT(i, j) + CT(i, j - 1);
    if (s == 0 || s == 2) {
        c[0] = 1.0;
        b = V_(i, j);
    } else if ((CT(i, j) + CT(i - 1, j)) == 0) {
        c[4] = an_();
        c[3] = as_();
        c[2] = ae_();
        c[0] = -c[4] - c[3] - c[2] + rho * dx * dy / dt + 2 * mu * dy / dx;
        b = bsrc();
    } else if ((CT(i, j) + CT(i + 1, j)) == 0) {
        c[4] = an_();
        c[3] = as_();
        c[1] = aw_();
        c[0] = -c[4] - c[3] - c[1] + rho * dx * dy / dt + 2 * mu * dy / dx;
        b = bsrc();
    } else {
        c[4] = an_();
        c[3] = as_();
        c[1] = aw_();
        c[2] = ae_();
        c[0] = -c[4] - c[3] - c[1] - c[2] + rho * dx * dy / dt;
        b = bsrc();
    }
#pragma unroll
    for (int q = 0; q < 5; ++q) coef[q * n + k] = c[q];
    bvec[k] = b;
    Mvec[k] = c[0];
}

// fill_Ap (karman_taichi.py:297-339)
__global__ void k_karman_fill_p(kc_karman K, const int* ct, const double* u, const double* v, const double* cu,
                                const double* cv, double* coef, double* bvec, double* Mvec) {
    const KGeo G = kgeo(K);
    const int nx = G.nx, ny = G.ny;
    const long long n = (long long)nx * ny;
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = (int)(k / ny) + 1, j = (int)(k % ny) + 1;
    const double rho = K.rho, dx = K.dx, dy = K.dy;
    double c[5];
    double b = rho * (U_(i, j) - U_(i + 1, j)) * dy + rho * (V_(i, j + 1) - V_(i, j)) * dx;
    const long long vk = (long long)(i - 1) * (ny + 1) + (j - 1);
    c[4] = -rho * dx * dx / cv[vk];       // Av[vk, vk]      (plane 0 of the v system)
    c[3] = -rho * dx * dx / cv[vk + 1];   // Av[vk+1, vk+1]
    c[1] = -rho * dy * dy / cu[k];        // Au[k, k]
    c[2] = -rho * dy * dy / cu[k + ny];   // Au[k+ny, k+ny]
    if ((CT(i, j) + CT(i, j - 1)) == 0) c[4] = 0.0;
    if ((CT(i, j) + CT(i, j + 1)) == 0) c[3] = 0.0;
    if ((CT(i, j) + CT(i - 1, j)) == 0) c[1] = 0.0;
    if ((CT(i, j) + CT(i + 1, j)) == 0) c[2] = 0.0;
    c[0] = -c[4] - c[3] - c[1] - c[2];
    double M = c[0];
    // second loop: inlet rows 0..ny-1 pinned with off-diagonals cleared;
    // outlet rows n-ny+1 .. n-1 pinned, links kept (row n is out of range)
    if (k < ny) {
        c[1] = c[2] = c[3] = c[4] = 0.0;
        c[0] = 1.0;
        M = 1.0;
        b = 0.0;
    }
    if (k >= n - ny + 1) {
        c[0] = 1.0;
        M = 1.0;
        b = 0.0;
    }
#pragma unroll
    for (int q = 0; q < 5; ++q) coef[q * n + k] = c[q];
    bvec[k] = b;
    Mvec[k] = M;
}

// xu_back / xv_back / xp_back (karman_taichi.py:459-478)
__global__ void k_karman_back(kc_karman K, int which, const double* x, double* f) {
    const KGeo G = kgeo(K);
    const int nx = G.nx, ny = G.ny;
    const int rows = which == 0 ? nx + 1 : nx;
    const int cols = which == 1 ? ny + 1 : ny;
    const long long n = (long long)rows * cols;
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = (int)(k / cols), j = (int)(k % cols);
    const double a = K.velo_rel;
    if (which == 0) {
        double* o = f + (long long)(i + 1) * G.NYu + (j + 1);
        *o = *o + a * (x[k] - *o);
    } else if (which == 1) {
        double* o = f + (long long)(i + 1) * G.NYv + (j + 1);
        *o = *o + a * (x[k] - *o);
    } else {
        f[(long long)(i + 1) * G.NYp + (j + 1)] = x[k];
    }
}

// puv_correction (karman_taichi.py:507-542): z = 0 u faces, 1 v faces, 2 p cells
__global__ void __launch_bounds__(256)
    k_karman_puv(kc_karman K, const int* ct, const double* pc, const double* cu, const double* cv, double* u,
                 double* v, double* p, ReduceWs* ws, double* pmax_out) {
    const KGeo G = kgeo(K);
    const int nx = G.nx, ny = G.ny;
    const int z = blockIdx.z;
    double mx = 0.0;
    const long long n = z == 0 ? (long long)(nx + 1) * ny : (z == 1 ? (long long)nx * (ny + 1)
                                                                     : (long long)(nx + 2) * (ny + 2));
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        if (z == 0) {
            const int i = (int)(t / ny) + 1, j = (int)(t % ny) + 1;
            const int s = CT(i - 1, j) + CT(i, j);
            if (s != 0 && s != 2) {
                double* o = u + (long long)i * G.NYu + j;
                *o = *o + (pc[(long long)(i - 1) * G.NYp + j] - pc[(long long)i * G.NYp + j]) * K.dy / cu[t];
            }
        } else if (z == 1) {
            const int i = (int)(t / (ny + 1)) + 1, j = (int)(t % (ny + 1)) + 1;
            const int s = CT(i, j) + CT(i, j - 1);
            if (s != 0 && s != 2) {
                double* o = v + (long long)i * G.NYv + j;
                *o = *o + (pc[(long long)i * G.NYp + j] - pc[(long long)i * G.NYp + j - 1]) * K.dx / cv[t];
            }
        } else {
            const double q = pc[t];
            if (ct[t] != 1) p[t] = p[t] + K.p_rel * q;
            mx = fmax(mx, fabs(q));
        }
    }
    double a[1] = {mx};
    block_max<1>(a);
    if (threadIdx.x == 0) ws->partials[z][blockIdx.x] = a[0];
    const unsigned nb = gridDim.x * gridDim.z;
    if (arrive_last(&ws->ticket[0], nb)) {
        double m[1];
        reduce_partials_max<1>(ws->partials[2], 0, gridDim.x, m);
        if (threadIdx.x == 0) {
            if (pmax_out) *pmax_out = m[0];
            ws->ticket[0] = 0;
        }
    }
}

// correct_conserv (karman_taichi.py:586-601): one block
__global__ void __launch_bounds__(256) k_karman_conserv(kc_karman K, double* u) {
    const KGeo G = kgeo(K);
    double acc[2] = {0.0, 0.0};
    for (int j = 1 + threadIdx.x; j <= G.ny; j += blockDim.x) {
        acc[0] += u[(long long)1 * G.NYu + j];
        acc[1] += u[(long long)(G.nx + 1) * G.NYu + j];
    }
    block_sum<2>(acc);
    __shared__ double coef;
    if (threadIdx.x == 0) coef = acc[0] / acc[1];
    __syncthreads();
    for (int j = 1 + threadIdx.x; j <= G.ny; j += blockDim.x) {
        double* o = u + (long long)(G.nx + 1) * G.NYu + j;
        *o = coef * *o;
    }
}

// udiv of correct_conserv (karman_taichi.py:610-613)
__global__ void k_karman_udiv(kc_karman K, const double* u, const double* v, double* udiv) {
    const KGeo G = kgeo(K);
    const long long n = (long long)G.nx * G.ny;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int i = (int)(t / G.ny) + 1, j = (int)(t % G.ny) + 1;
    udiv[(long long)i * G.NYp + j] = (U_(i, j) - U_(i + 1, j)) * K.dy + (V_(i, j + 1) - V_(i, j)) * K.dx;
}

#undef CT
#undef U_
#undef V_
#undef P_

static int check_k(const kc_karman* K) {
    if (!K) return set_error("kc_karman is null"), KC_ERR_ARG;
    if (K->nx < 3 || K->ny < 3) return set_error("kc_karman: nx=%d ny=%d too small", K->nx, K->ny), KC_ERR_ARG;
    return KC_OK;
}

static inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace kc

using namespace kc;

extern "C" {

int kc_karman_fill_u(const kc_karman* K, const int* ct, const double* u, const double* v, const double* p,
                     const double* u0, double* coef, double* b, double* M, void* stream) {
    int rc = check_k(K);
    if (rc) return rc;
    if (!ct || !u || !v || !p || !u0 || !coef || !b || !M) return set_error("kc_karman_fill_u: null argument"), KC_ERR_ARG;
    long long n = (long long)(K->nx + 1) * K->ny;
    k_karman_fill_u<<<nblk(n, 256), 256, 0, as_stream(stream)>>>(*K, ct, u, v, p, u0, coef, b, M);
    KC_LAUNCH_CHECK("k_karman_fill_u");
    return KC_OK;
}

int kc_karman_fill_v(const kc_karman* K, const int* ct, const double* u, const double* v, const double* p,
                     const double* v0, double* coef, double* b, double* M, void* stream) {
    int rc = check_k(K);
    if (rc) return rc;
    if (!ct || !u || !v || !p || !v0 || !coef || !b || !M) return set_error("kc_karman_fill_v: null argument"), KC_ERR_ARG;
    long long n = (long long)K->nx * (K->ny + 1);
    k_karman_fill_v<<<nblk(n, 256), 256, 0, as_stream(stream)>>>(*K, ct, u, v, p, v0, coef, b, M);
    KC_LAUNCH_CHECK("k_karman_fill_v");
    return KC_OK;
}

int kc_karman_fill_p(const kc_karman* K, const int* ct, const double* u, const double* v, const double* coef_u,
                     const double* coef_v, double* coef, double* b, double* M, void* stream) {
    int rc = check_k(K);
    if (rc) return rc;
    if (!ct || !u || !v || !coef_u || !coef_v || !coef || !b || !M)
        return set_error("kc_karman_fill_p: null argument"), KC_ERR_ARG;
    long long n = (long long)K->nx * K->ny;
    k_karman_fill_p<<<nblk(n, 256), 256, 0, as_stream(stream)>>>(*K, ct, u, v, coef_u, coef_v, coef, b, M);
    KC_LAUNCH_CHECK("k_karman_fill_p");
    return KC_OK;
}

int kc_karman_back(const kc_karman* K, int which, const double* x, double* field, void* stream) {
    int rc = check_k(K);
    if (rc) return rc;
    if (which < 0 || which > 2 || !x || !field) return set_error("kc_karman_back: bad arguments"), KC_ERR_ARG;
    long long n = which == 0 ? (long long)(K->nx + 1) * K->ny
                             : (which == 1 ? (long long)K->nx * (K->ny + 1) : (long long)K->nx * K->ny);
    k_karman_back<<<nblk(n, 256), 256, 0, as_stream(stream)>>>(*K, which, x, field);
    KC_LAUNCH_CHECK("k_karman_back");
    return KC_OK;
}

int kc_karman_puv_correction(const kc_karman* K, const int* ct, const double* pcor, const double* coef_u,
                             const double* coef_v, double* u, double* v, double* p, double* pcor_max_dev,
                             void* ws, void* stream) {
    int rc = check_k(K);
    if (rc) return rc;
    if (!ct || !pcor || !coef_u || !coef_v || !u || !v || !p) return set_error("kc_karman_puv_correction: null argument"), KC_ERR_ARG;
    if (!ws) return set_error("kc_karman_puv_correction: null workspace"), KC_ERR_WORKSPACE;
    long long n = (long long)(K->nx + 2) * (K->ny + 2);
    unsigned g = std::min<unsigned>(nblk(n, 256 * 4), 1024u);
    k_karman_puv<<<dim3(g, 1, 3), 256, 0, as_stream(stream)>>>(*K, ct, pcor, coef_u, coef_v, u, v, p, (ReduceWs*)ws,
                                                               pcor_max_dev);
    KC_LAUNCH_CHECK("k_karman_puv");
    return KC_OK;
}

int kc_karman_correct_conserv(const kc_karman* K, double* u, const double* v, double* udiv, void* stream) {
    int rc = check_k(K);
    if (rc) return rc;
    if (!u || !v) return set_error("kc_karman_correct_conserv: null argument"), KC_ERR_ARG;
    k_karman_conserv<<<1, 256, 0, as_stream(stream)>>>(*K, u);
    KC_LAUNCH_CHECK("k_karman_conserv");
    if (udiv) {
        long long n = (long long)K->nx * K->ny;
        k_karman_udiv<<<nblk(n, 256), 256, 0, as_stream(stream)>>>(*K, u, v, udiv);
        KC_LAUNCH_CHECK("k_karman_udiv");
    }
    return KC_OK;
}

}  // extern "C"
