// SIMPLE assembly and correction kernels on staggered padded fields.
//
// Reference behaviour (houkensjtu/karman_taichi):
//   compute_coef_u / compute_coef_v   simple.py:77-110   (mid-point convection + diffusion)
//   set_bc                            simple.py:172-216  (east wall adds aW: simple.py:215;
//                                                         bicgsimp.py:196 adds aE)
//   compute_mdiv / compute_coef_p     simple.py:137-170, bicgsimp.py:114-151
//   correct_pressure/velocity         simple.py:218-230
//   update_velocity                   simple.py:232-238, bicgsimp.py:212-225
//   outlet zero gradient + rescale    karman_taichi.py:178-183, 586-601
//
// Field layout (row-major, j fastest): u [nx+3][ny+2], v [nx+2][ny+3],
// p [nx+2][ny+2]; coefficient outputs are 5 SoA planes over the same padded
// field followed by b.  One thread owns one face/cell; faces that are not
// unknowns become zero rows (so a solver over the whole padded field leaves
// them at 0, as the reference's full-field solves do), blocked faces in the
// channel mode become identity rows.
//
// This file is compiled with -fmad=false: the p' coefficients, the mass
// source, the relaxation and the correction keep the reference's
// left-to-right IEEE operation order, so the CPU restatement reproduces them
// bit for bit.  The momentum coefficients are the exception: their central
// part is evaluated in an algebraically reduced form with explicit fused
// multiply-adds (15 instead of 36 FP64 operations per face; see u_row), which
// agrees with the reference's expression to a few units in the last place.
#include "kc_simple.cuh"
#include <algorithm>

namespace kc {

#define U_(a, bb) u[(long long)(a) * D.NYu + (bb)]
#define V_(a, bb) v[(long long)(a) * D.NYv + (bb)]
#define P_(a, bb) p[(long long)(a) * D.NYp + (bb)]

struct MomOut {
    double *cu, *bu, *cv, *bv;
    float *cu32, *bu32, *cv32, *bv32;
};

// Block layout of the field kernels: 256 threads as 8 rows of 32 lanes, lanes
// along j (coalesced), rows strided by the grid.
__device__ __forceinline__ int fk_lane() { return threadIdx.x & 31; }
__device__ __forceinline__ int fk_row() { return threadIdx.x >> 5; }

__global__ void __launch_bounds__(256)
    k_assemble_momentum(kc_phys P, SimpleK K, const double* u, const double* v, const double* p, const double* u0,
                        const double* v0, const unsigned char* solid, MomOut O) {
    const Dims D = dims_of(P);
    const Solid S{solid, D.NYp};
    const bool isv = blockIdx.z == 1;
    const int NX = isv ? D.nx + 2 : D.nx + 3, NY = isv ? D.NYv : D.NYu;
    const long long n = (long long)NX * NY;
    const int j = blockIdx.x * 32 + fk_lane();
    if (j >= NY) return;
    for (int i = blockIdx.y * 8 + fk_row(); i < NX; i += gridDim.y * 8) {
        double c[5], b;
        const long long k = (long long)i * NY + j;
        if (isv) {
            v_row(P, K, D, S, u, v, p, v0, i, j, c, b);
#pragma unroll
            for (int q = 0; q < 5; ++q) O.cv[q * n + k] = c[q];
            O.bv[k] = b;
            if (O.cv32) {
#pragma unroll
                for (int q = 0; q < 5; ++q) O.cv32[q * n + k] = f64_to_f32(c[q]);
                O.bv32[k] = f64_to_f32(b);
            }
        } else {
            u_row(P, K, D, S, u, v, p, u0, i, j, c, b);
#pragma unroll
            for (int q = 0; q < 5; ++q) O.cu[q * n + k] = c[q];
            O.bu[k] = b;
            if (O.cu32) {
#pragma unroll
                for (int q = 0; q < 5; ++q) O.cu32[q * n + k] = f64_to_f32(c[q]);
                O.bu32[k] = f64_to_f32(b);
            }
        }
    }
}

// Each block leaves its partials in ws->partials[z][block]; the last block of
// the grid to arrive folds them with every thread (a strided pass, then a
// block reduction) and resets the ticket.  Max is exact in any order; a sum is
// folded in a fixed order, so it is reproducible run to run.
__device__ __forceinline__ int fk_block() { return blockIdx.y * gridDim.x + blockIdx.x; }
__device__ __forceinline__ int fk_blocks_z() { return gridDim.x * gridDim.y; }

__global__ void k_apply_bc_values(kc_phys P, double* u, double* v) {
    const Dims D = dims_of(P);
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 1 && t <= D.ny) {
        u[(long long)1 * D.NYu + t] = P.bc[0][0];
        u[(long long)(D.nx + 1) * D.NYu + t] = P.bc[1][0];
    }
    if (t >= 1 && t <= D.nx) {
        v[(long long)t * D.NYv + 1] = P.bc[3][0];
        v[(long long)t * D.NYv + D.ny + 1] = P.bc[2][0];
    }
}

// ---- under-relaxation --------------------------------------------------------
__global__ void __launch_bounds__(256)
    k_relax(kc_phys P, SimpleK K, const unsigned char* solid, const double* um, const double* vm, double* u,
            double* v, ReduceWs* ws, double* diff_out) {
    const Dims D = dims_of(P);
    const Solid S{solid, D.NYp};
    const bool isv = blockIdx.z == 1;
    const int NX = isv ? D.nx + 2 : D.nx + 3, NY = isv ? D.NYv : D.NYu;
    const double a = P.alpha_m;
    const int j = blockIdx.x * 32 + fk_lane();
    double dm[1] = {0.0};
    if (j < NY) {
        const double* mid = isv ? vm : um;
        double* f = isv ? v : u;
        for (int i = blockIdx.y * 8 + fk_row(); i < NX; i += gridDim.y * 8) {
            const long long k = (long long)i * NY + j;
            if (isv ? unk_v(P, S, i, j) : unk_u(P, S, i, j)) {
                const double m = mid[k], old = f[k];
                dm[0] = fmax(dm[0], fabs(m - old));
                f[k] = a * m + K.one_m_am * old;
            }
        }
    }
    block_max<1>(dm);
    if (threadIdx.x == 0) ws->partials[blockIdx.z][fk_block()] = dm[0];
    if (!arrive_last(&ws->ticket[0], fk_blocks_z() * gridDim.z)) return;
    double o[2];
    reduce_partials_max<2>(&ws->partials[0][0], kReduceMaxBlocks, fk_blocks_z(), o);
    if (threadIdx.x == 0) {
        if (diff_out) *diff_out = sqrt(o[0] * o[0] + o[1] * o[1]);
        ws->ticket[0] = 0;
    }
}

// ---- channel outlet: zero gradient + mass-flow rescale (single block) --------
__global__ void __launch_bounds__(256) k_outlet_conserve(kc_phys P, double* u) {
    const Dims D = dims_of(P);
    double acc[2] = {0.0, 0.0};
    for (int j = 1 + threadIdx.x; j <= D.ny; j += blockDim.x) {
        const double w = u[(long long)D.nx * D.NYu + j];
        u[(long long)(D.nx + 1) * D.NYu + j] = w;
        acc[0] += u[(long long)1 * D.NYu + j];
        acc[1] += w;
    }
    block_sum<2>(acc);
    __shared__ double coef;
    if (threadIdx.x == 0) coef = acc[0] / acc[1];
    __syncthreads();
    for (int j = 1 + threadIdx.x; j <= D.ny; j += blockDim.x) {
        double* o = u + (long long)(D.nx + 1) * D.NYu + j;
        *o = coef * *o;
    }
}

// ---- pressure correction -----------------------------------------------------
// A warp covers 31 cells of a row (lane 31 evaluates the halo column) and a
// run of kPcRows consecutive rows.  Each face's link value -rho dy^2 / aP_u
// (resp. -rho dx^2 / aP_v) is divided once and shared by the two cells on
// either side of it -- through the row carry for u faces, a lane shuffle for
// v faces -- instead of once per cell: half the FP64 divisions.
constexpr int kPcRows = 4;
constexpr int kPcCols = 31;

__device__ __forceinline__ void finish_max_sum(double mx, double sq, ReduceWs* ws, double* mass_out) {
    double a[1] = {mx}, b[1] = {sq};
    block_max<1>(a);
    block_sum<1>(b);
    if (threadIdx.x == 0) {
        ws->partials[0][fk_block()] = a[0];
        ws->partials[1][fk_block()] = b[0];
    }
    if (!arrive_last(&ws->ticket[0], fk_blocks_z())) return;
    reduce_partials_max<1>(&ws->partials[0][0], kReduceMaxBlocks, fk_blocks_z(), a);
    reduce_partials<1>(&ws->partials[1][0], kReduceMaxBlocks, fk_blocks_z(), b);
    if (threadIdx.x == 0) {
        if (mass_out) {
            mass_out[0] = a[0];
            mass_out[1] = b[0];
        }
        ws->ticket[0] = 0;
    }
}

__global__ void __launch_bounds__(256)
    k_assemble_pcorr(kc_phys P, SimpleK K, const double* u, const double* v, const double* apu, const double* apv,
                     const unsigned char* solid, double* cp, double* bp, float* cp32, float* bp32,
                     double* mdiv_out, ReduceWs* ws, double* mass_out) {
    const Dims D = dims_of(P);
    const Solid S{solid, D.NYp};
    const int NX = D.nx + 2, NY = D.NYp;
    const long long n = (long long)NX * NY;
    const int nx = D.nx, ny = D.ny;
    const double rho = P.rho, dx = P.dx, dy = P.dy;
    const bool channel = P.mode == KC_MODE_CHANNEL;
    const int lane = fk_lane();
    const int j = blockIdx.x * kPcCols + lane;
    const bool own = lane < kPcCols && j < NY;
    double mx = 0.0, sq = 0.0;
    // rows of u faces: 0..nx+2 (NX + 1 of them); columns of v faces: 0..ny+2
    for (int rg = blockIdx.y * 8 + fk_row(); rg * kPcRows < NX; rg += gridDim.y * 8) {
        const int i0 = rg * kPcRows;
        double tw = j < NY ? K.nrdy2 / apu[(long long)i0 * D.NYu + j] : 0.0;   // u face (i0, j)
        for (int r = 0; r < kPcRows; ++r) {
            const int i = i0 + r;
            if (i >= NX) break;   // uniform over the warp
            const double te = j < NY ? K.nrdy2 / apu[(long long)(i + 1) * D.NYu + j] : 0.0;   // u face (i+1, j)
            const double tv = j < D.NYv ? K.nrdx2 / apv[(long long)i * D.NYv + j] : 0.0;     // v face (i, j)
            const double tn = __shfl_down_sync(kFull, tv, 1);                                 // v face (i, j+1)
            if (own) {
                const long long k = (long long)i * NY + j;
                double c[5] = {0, 0, 0, 0, 0}, b = 0.0, xs = 0.0;
                if (i >= 1 && i <= nx && j >= 1 && j <= ny) {
                    const double md = rho * (U_(i, j) - U_(i + 1, j)) * dy + rho * (V_(i, j) - V_(i, j + 1)) * dx;
                    if (mdiv_out) mdiv_out[k] = md;
                    if (channel && S.cell(i, j)) {
                        c[0] = 1.0;
                    } else if (channel) {
                        double aW = 0.0, aE = 0.0, aN = 0.0, aS = 0.0;
                        if (unk_u(P, S, i, j)) aW = tw;
                        if (unk_u(P, S, i + 1, j)) aE = te;
                        if (i == nx && unk_u(P, S, nx, j)) aE = tw;   // the outlet row links to face nx again
                        if (unk_v(P, S, i, j + 1)) aN = tn;
                        if (unk_v(P, S, i, j)) aS = tv;
                        xs = aW + aE + aN + aS;
                        c[0] = -xs;
                        c[1] = aW;
                        c[2] = aE;
                        c[3] = aN;
                        c[4] = aS;
                        b = md;
                        mx = fmax(mx, fabs(md));
                        sq += md * md;
                    } else {
                        // compute_coef_p, simple.py:146-163 (bicgsimp.py:146-151 pins (1,1))
                        const double aW = i == 1 ? 0.0 : tw;
                        const double aE = i == nx ? 0.0 : te;
                        const double aN = j == ny ? 0.0 : tn;
                        const double aS = j == 1 ? 0.0 : tv;
                        xs = aW + aE + aN + aS;
                        c[0] = -xs;
                        c[1] = aW;
                        c[2] = aE;
                        c[3] = aN;
                        c[4] = aS;
                        b = md;
                        if (P.mode == KC_MODE_BICGSIMP && i == 1 && j == 1) {
                            c[1] = c[2] = c[3] = c[4] = 0.0;
                            c[0] = 1.0;
                            b = 0.0;
                            xs = 0.0;
                        }
                        mx = fmax(mx, fabs(md));
                        sq += md * md;
                    }
                }
#pragma unroll
                for (int q = 0; q < 5; ++q) cp[q * n + k] = c[q];
                bp[k] = b;
                if (cp32) {
                    // FP32 copy in Laplacian form: component 0 is the row sum
                    // c0 + (((c1 + c2) + c3) + c4) -- the link sum xs in the
                    // order aP was built in, so it is exactly 0 on every fluid
                    // row (see KC_FORM_LAPLACIAN)
                    cp32[k] = f64_to_f32(c[0] + xs);
#pragma unroll
                    for (int q = 1; q < 5; ++q) cp32[q * n + k] = f64_to_f32(c[q]);
                    bp32[k] = f64_to_f32(b);
                }
            }
            tw = te;
        }
    }
    finish_max_sum(mx, sq, ws, mass_out);
}

// ---- correction: z = 0 u faces, 1 v faces, 2 p cells --------------------------
__global__ void __launch_bounds__(256)
    k_correct(kc_phys P, const double* pc, const double* apu, const double* apv, const unsigned char* solid,
              double* u, double* v, double* p, ReduceWs* ws, double* pmax_out) {
    const Dims D = dims_of(P);
    const Solid S{solid, D.NYp};
    const int z = blockIdx.z;
    const int NX = z == 0 ? D.nx + 3 : D.nx + 2;
    const int NY = z == 0 ? D.NYu : (z == 1 ? D.NYv : D.NYp);
    const int nx = D.nx, ny = D.ny;
    const bool channel = P.mode == KC_MODE_CHANNEL;
    const double au = P.alpha_u, ap = P.alpha_p, dx = P.dx, dy = P.dy;
#define PC_(a, bb) pc[(long long)(a) * D.NYp + (bb)]
    const int j = blockIdx.x * 32 + fk_lane();
    double mx[1] = {0.0};
    if (j < NY) {
        for (int i = blockIdx.y * 8 + fk_row(); i < NX; i += gridDim.y * 8) {
            const long long k = (long long)i * NY + j;
            if (z == 0) {
                if (unk_u(P, S, i, j)) {
                    u[k] = u[k] + au * (PC_(i - 1, j) - PC_(i, j)) * dy / apu[k];
                } else if (channel && i == nx + 1 && j >= 1 && j <= ny && unk_u(P, S, nx, j)) {
                    u[k] = u[k] + au * (PC_(nx, j) - PC_(nx + 1, j)) * dy / apu[(long long)nx * D.NYu + j];
                }
            } else if (z == 1) {
                if (unk_v(P, S, i, j)) v[k] = v[k] + au * (PC_(i, j - 1) - PC_(i, j)) * dx / apv[k];
            } else {
                const double q = pc[k];
                mx[0] = fmax(mx[0], fabs(q));
                if (i >= 1 && i <= nx && j >= 1 && j <= ny && !(channel && S.cell(i, j))) p[k] = p[k] + ap * q;
            }
        }
    }
    block_max<1>(mx);
    if (threadIdx.x == 0) ws->partials[z][fk_block()] = mx[0];
    if (!arrive_last(&ws->ticket[0], fk_blocks_z() * gridDim.z)) return;
    reduce_partials_max<1>(&ws->partials[2][0], kReduceMaxBlocks, fk_blocks_z(), mx);
    if (threadIdx.x == 0) {
        if (pmax_out) *pmax_out = mx[0];
        ws->ticket[0] = 0;
    }
}

__global__ void __launch_bounds__(256)
    k_mass_residual(kc_phys P, const double* u, const double* v, const unsigned char* solid, double* mdiv_out,
                    ReduceWs* ws, double* mass_out) {
    const Dims D = dims_of(P);
    const Solid S{solid, D.NYp};
    const int NX = D.nx + 2, NY = D.NYp;
    const double rho = P.rho, dx = P.dx, dy = P.dy;
    const bool channel = P.mode == KC_MODE_CHANNEL;
    const int j = blockIdx.x * 32 + fk_lane();
    double mx = 0.0, sq = 0.0;
    if (j >= 1 && j <= D.ny) {
        for (int i = blockIdx.y * 8 + fk_row(); i < NX; i += gridDim.y * 8) {
            if (i < 1 || i > D.nx) continue;
            const long long k = (long long)i * NY + j;
            double md = rho * (U_(i, j) - U_(i + 1, j)) * dy + rho * (V_(i, j) - V_(i, j + 1)) * dx;
            if (mdiv_out) mdiv_out[k] = md;
            if (channel && S.cell(i, j)) continue;
            mx = fmax(mx, fabs(md));
            sq += md * md;
        }
    }
    finish_max_sum(mx, sq, ws, mass_out);
}
#undef U_
#undef V_
#undef P_
#undef PC_

static dim3 field_grid(int NX, int NY, int zdim) {
    int gx = (NY + 31) / 32;
    int gy = (NX + 7) / 8;
    int cap = std::max(1, kReduceMaxBlocks / (gx > 0 ? gx : 1));
    if (gy > cap) gy = cap;
    if (gy > 64) gy = 64;
    return dim3(gx, gy, zdim);
}
// k_assemble_pcorr: kPcCols cells per warp row, kPcRows rows per warp, 8 warps
static dim3 pcorr_grid(int NX, int NY) {
    int gx = (NY + kPcCols - 1) / kPcCols;
    int gy = (NX + 8 * kPcRows - 1) / (8 * kPcRows);
    int cap = std::max(1, kReduceMaxBlocks / (gx > 0 ? gx : 1));
    if (gy > cap) gy = cap;
    return dim3(gx, gy, 1);
}

static int check_phys(const kc_phys* P) {
    if (!P) return set_error("kc_phys is null"), KC_ERR_ARG;
    if (P->nx < 2 || P->ny < 2) return set_error("kc_phys: nx=%d ny=%d must be >= 2", P->nx, P->ny), KC_ERR_ARG;
    if (P->mode < KC_MODE_SIMPLE || P->mode > KC_MODE_CHANNEL)
        return set_error("kc_phys: unknown mode %d", P->mode), KC_ERR_ARG;
    if ((long long)(P->ny + 3 + kPcCols - 1) / kPcCols > kReduceMaxBlocks)
        return set_error("kc_phys: ny=%d too large", P->ny), KC_ERR_ARG;
    return KC_OK;
}

}  // namespace kc

using namespace kc;

extern "C" {

size_t kc_reduce_ws_bytes(void) { return sizeof(ReduceWs); }

int kc_assemble_momentum(const kc_phys* P, const double* u, const double* v, const double* p, const double* u0,
                         const double* v0, const unsigned char* solid, double* coef_u, double* b_u,
                         double* coef_v, double* b_v, float* coef_u32, float* b_u32, float* coef_v32,
                         float* b_v32, void* stream) {
    int rc = check_phys(P);
    if (rc) return rc;
    if (!u || !v || !p || !u0 || !v0 || !coef_u || !b_u || !coef_v || !b_v)
        return set_error("kc_assemble_momentum: null field"), KC_ERR_ARG;
    if (P->mode == KC_MODE_CHANNEL && !solid) solid = nullptr;
    if ((coef_u32 == nullptr) != (b_u32 == nullptr) || (coef_v32 == nullptr) != (b_v32 == nullptr))
        return set_error("kc_assemble_momentum: FP32 outputs must be given in pairs"), KC_ERR_ARG;
    MomOut O{coef_u, b_u, coef_v, b_v, coef_u32, b_u32, coef_v32, b_v32};
    dim3 g = field_grid(P->nx + 3, P->ny + 3, 2);
    k_assemble_momentum<<<g, 256, 0, as_stream(stream)>>>(*P, consts_of(*P), u, v, p, u0, v0, solid, O);
    KC_LAUNCH_CHECK("k_assemble_momentum");
    return KC_OK;
}

int kc_apply_bc_values(const kc_phys* P, double* u, double* v, void* stream) {
    int rc = check_phys(P);
    if (rc) return rc;
    if (!u || !v) return set_error("kc_apply_bc_values: null field"), KC_ERR_ARG;
    int m = std::max(P->nx, P->ny) + 1;
    k_apply_bc_values<<<(m + 255) / 256, 256, 0, as_stream(stream)>>>(*P, u, v);
    KC_LAUNCH_CHECK("k_apply_bc_values");
    return KC_OK;
}

int kc_relax_velocity(const kc_phys* P, const unsigned char* solid, const double* u_mid, const double* v_mid,
                      double* u, double* v, double* diff_dev, void* ws, void* stream) {
    int rc = check_phys(P);
    if (rc) return rc;
    if (!u_mid || !v_mid || !u || !v) return set_error("kc_relax_velocity: null field"), KC_ERR_ARG;
    if (!ws) return set_error("kc_relax_velocity: null workspace"), KC_ERR_WORKSPACE;
    dim3 g = field_grid(P->nx + 3, P->ny + 3, 2);
    k_relax<<<g, 256, 0, as_stream(stream)>>>(*P, consts_of(*P), solid, u_mid, v_mid, u, v, (ReduceWs*)ws,
                                           diff_dev);
    KC_LAUNCH_CHECK("k_relax");
    return KC_OK;
}

int kc_outlet_conserve(const kc_phys* P, double* u, void* stream) {
    int rc = check_phys(P);
    if (rc) return rc;
    if (!u) return set_error("kc_outlet_conserve: null u"), KC_ERR_ARG;
    k_outlet_conserve<<<1, 256, 0, as_stream(stream)>>>(*P, u);
    KC_LAUNCH_CHECK("k_outlet_conserve");
    return KC_OK;
}

int kc_assemble_pcorr(const kc_phys* P, const double* u, const double* v, const double* coef_u,
                      const double* coef_v, const unsigned char* solid, double* coef_p, double* b_p,
                      float* coef_p32, float* b_p32, double* mdiv, double* mass_dev, void* ws, void* stream) {
    int rc = check_phys(P);
    if (rc) return rc;
    if (!u || !v || !coef_u || !coef_v || !coef_p || !b_p)
        return set_error("kc_assemble_pcorr: null field"), KC_ERR_ARG;
    if ((coef_p32 == nullptr) != (b_p32 == nullptr))
        return set_error("kc_assemble_pcorr: FP32 outputs must be given in pairs"), KC_ERR_ARG;
    if (!ws) return set_error("kc_assemble_pcorr: null workspace"), KC_ERR_WORKSPACE;
    dim3 g = pcorr_grid(P->nx + 2, P->ny + 2);
    k_assemble_pcorr<<<g, 256, 0, as_stream(stream)>>>(*P, consts_of(*P), u, v, coef_u, coef_v, solid, coef_p, b_p,
                                                               coef_p32, b_p32, mdiv, (ReduceWs*)ws, mass_dev);
    KC_LAUNCH_CHECK("k_assemble_pcorr");
    return KC_OK;
}

int kc_correct(const kc_phys* P, const double* pcor, const double* coef_u, const double* coef_v,
               const unsigned char* solid, double* u, double* v, double* p, double* pcor_max_dev, void* ws,
               void* stream) {
    int rc = check_phys(P);
    if (rc) return rc;
    if (!pcor || !coef_u || !coef_v || !u || !v || !p) return set_error("kc_correct: null field"), KC_ERR_ARG;
    if (!ws) return set_error("kc_correct: null workspace"), KC_ERR_WORKSPACE;
    dim3 g = field_grid(P->nx + 3, P->ny + 3, 3);
    k_correct<<<g, 256, 0, as_stream(stream)>>>(*P, pcor, coef_u, coef_v, solid, u, v, p, (ReduceWs*)ws,
                                                        pcor_max_dev);
    KC_LAUNCH_CHECK("k_correct");
    return KC_OK;
}

int kc_mass_residual(const kc_phys* P, const double* u, const double* v, const unsigned char* solid,
                     double* mdiv, double* mass_dev, void* ws, void* stream) {
    int rc = check_phys(P);
    if (rc) return rc;
    if (!u || !v || !mass_dev) return set_error("kc_mass_residual: null argument"), KC_ERR_ARG;
    if (!ws) return set_error("kc_mass_residual: null workspace"), KC_ERR_WORKSPACE;
    dim3 g = field_grid(P->nx + 2, P->ny + 2, 1);
    k_mass_residual<<<g, 256, 0, as_stream(stream)>>>(*P, u, v, solid, mdiv, (ReduceWs*)ws, mass_dev);
    KC_LAUNCH_CHECK("k_mass_residual");
    return KC_OK;
}

}  // extern "C"

// ---- lexicographic relaxation sweep (jacosimp.py) -------------------------------------------
// jacosimp.py:210-238 relaxes u, v and p' in Python scope, in place, i outer
// and j inner: cell (i, j) reads its west (i-1, j) and south (i, j-1)
// neighbours already updated in this sweep and its east and north neighbours
// not yet updated.  Cells on one anti-diagonal i + j = d depend only on
// diagonal d - 1, so one block sweeping the diagonals in order, with a barrier
// between them, produces the serial sweep's values exactly; every cell's
// arithmetic is the reference's expression in its order (this unit is
// compiled without FMA contraction).
namespace kc {
__global__ void __launch_bounds__(1024)
    k_lex_sweep(const double* __restrict__ c, long long cs, long long es, int NY, int i0, int i1, int j0, int j1,
                const double* __restrict__ b, double* x, double* x_mid, double omega, int relax) {
    const int ni = i1 - i0, nj = j1 - j0;
    for (int d = 0; d < ni + nj - 1; ++d) {
        const int a_lo = d - nj + 1 > 0 ? d - nj + 1 : 0, a_hi = d < ni - 1 ? d : ni - 1;
        for (int a = a_lo + (int)threadIdx.x; a <= a_hi; a += (int)blockDim.x) {
            const long long i = i0 + a, j = j0 + (d - a);
            const long long k = i * NY + j;
            const double* ck = c + k * es;
            const double xm =
                ((((-ck[cs] * x[k - NY]) - ck[2 * cs] * x[k + NY]) - ck[3 * cs] * x[k + 1]) - ck[4 * cs] * x[k - 1] +
                 b[k]) / ck[0];
            if (relax) {
                x_mid[k] = xm;
                x[k] = (1.0 - omega) * x[k] + omega * xm;
            } else {
                x[k] = xm;
            }
        }
        __syncthreads();
    }
}
}  // namespace kc

extern "C" {

int kc_lex_sweep(const double* coef, long long cs, long long es, int NX, int NY, int i0, int i1, int j0, int j1,
                 const double* b, double* x, double* x_mid, double omega, int relax, void* stream) {
    if (!coef || !b || !x || (relax && !x_mid)) return set_error("kc_lex_sweep: null argument"), KC_ERR_ARG;
    if (NX < 3 || NY < 3 || cs < 1 || es < 1)
        return set_error("kc_lex_sweep: bad grid %d x %d or strides", NX, NY), KC_ERR_ARG;
    if (i0 < 1 || i1 > NX - 1 || j0 < 1 || j1 > NY - 1 || i0 >= i1 || j0 >= j1)
        return set_error("kc_lex_sweep: box [%d, %d) x [%d, %d) must lie inside the 1-cell ring of %d x %d", i0, i1,
                         j0, j1, NX, NY),
               KC_ERR_ARG;
    k_lex_sweep<<<1, 1024, 0, as_stream(stream)>>>(coef, cs, es, NY, i0, i1, j0, j1, b, x, x_mid, omega, relax);
    KC_LAUNCH_CHECK("k_lex_sweep");
    return KC_OK;
}

}  // extern "C"
