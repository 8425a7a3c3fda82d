// Flexible conjugate gradients for the pressure-correction system, with the
// trained network as a preconditioner application.
//
// The reference solves p' with BiCGSTAB whose right-preconditioner hooks
// p^ = M^-1 p and s^ = M^-1 s are the identity (bicgsolver.py:48-58) or Jacobi
// (karman_taichi.py:398-399, 418-419).  Here the preconditioner changes from
// one application to the next -- the first is the U-Net's prediction of
// A^-1 r (kc_unet_predict), every later one a multigrid-preconditioned FP32 CG
// pass on A z = r (kc_pcg_refined, one refinement sweep) -- so the outer
// iteration is a flexible Krylov method: FCG(1) in FP64 (Notay, "Flexible
// conjugate gradients", SIAM J. Sci. Comput. 22, 2000).  With z_k = P_k(r_k)
// and w_k = A z_k:
//     beta_k = (z_k, q_{k-1}) / (p_{k-1}, q_{k-1})       (0 for k = 0)
//     p_k = z_k - beta_k p_{k-1},  q_k = A p_k = w_k - beta_k q_{k-1}
//     alpha_k = (p_k, r_k) / (p_k, q_k)
//     x += alpha_k p_k,  r -= alpha_k q_k
// so every direction is A-orthogonal to the previous one and every step
// length minimises the error's A-norm along its direction: a poor network
// prediction costs one short step, not a worse iterate.  A network
// direction that is not finite, or not a descent direction ((p, q) <= 0), is
// rejected and replaced by a multigrid pass (counted in kc_flex_info).
// Stall detection: two outer iterations in a row that reduce ||r|| by less
// than 10 % end the solve with KC_STALL (x the last iterate), so the caller
// can fall back to the plain BiCGSTAB.  Convergence is confirmed on the true
// residual b - A x before KC_OK is returned.
//
// All outer vectors are FP64; each pointwise pass accumulates its inner
// products per block and sums the block partials in a fixed order in a
// second one-block kernel, so results repeat bitwise.
#include "kc_common.cuh"
#include <algorithm>
#include <cmath>
#include <cstring>

namespace kc {
namespace {

constexpr int kFxThreads = 256;
constexpr int kFxMaxBlocks = 1024;
constexpr int kFxSums = 4;

struct FlexLayout {
    size_t r, z, w, p, q, partials, out, total;
};
FlexLayout flex_layout(long long n) {
    FlexLayout L{};
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o = align256(o + bytes);
        return at;
    };
    L.r = take((size_t)n * 8);
    L.z = take((size_t)n * 8);
    L.w = take((size_t)n * 8);
    L.p = take((size_t)n * 8);
    L.q = take((size_t)n * 8);
    L.partials = take((size_t)kFxSums * kFxMaxBlocks * 8);
    L.out = take(8 * 8);
    L.total = o;
    return L;
}

int fx_blocks(long long n) {
    return (int)std::max<long long>(1, std::min<long long>((n + kFxThreads * 4 - 1) / (kFxThreads * 4), kFxMaxBlocks));
}

// per-block sums of NS values into partials[s * kFxMaxBlocks + block]
template <int NS>
__device__ __forceinline__ void fx_block_store(double (&v)[NS], double* partials) {
    block_sum<NS>(v);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int s = 0; s < NS; ++s) partials[s * kFxMaxBlocks + blockIdx.x] = v[s];
    }
}

// one block: out[s] = sum over blocks of partials[s][.], in block order
template <int NS>
__global__ void __launch_bounds__(kFxThreads) k_fx_finish(const double* __restrict__ partials, int nb,
                                                          double* __restrict__ out) {
    double v[NS];
    reduce_partials<NS>(partials, kFxMaxBlocks, nb, v);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int s = 0; s < NS; ++s) out[s] = v[s];
    }
}

// r = b - w (w = A x); sums (r, r), (b, b)
__global__ void __launch_bounds__(kFxThreads) k_fx_resid(long long n, const double* __restrict__ b,
                                                         const double* __restrict__ w, double* __restrict__ r,
                                                         double* partials) {
    double v[2] = {0.0, 0.0};
    for (long long k = blockIdx.x * (long long)kFxThreads + threadIdx.x; k < n; k += (long long)gridDim.x * kFxThreads) {
        const double bk = __ldg(b + k);
        const double rk = bk - __ldg(w + k);
        r[k] = rk;
        v[0] = fma(rk, rk, v[0]);
        v[1] = fma(bk, bk, v[1]);
    }
    fx_block_store<2>(v, partials);
}

// sums (z, q_prev), (z, r), (z, w), (p_prev, r)
__global__ void __launch_bounds__(kFxThreads) k_fx_dots(long long n, const double* __restrict__ z,
                                                        const double* __restrict__ w, const double* __restrict__ r,
                                                        const double* __restrict__ p, const double* __restrict__ q,
                                                        int first, double* partials) {
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (long long k = blockIdx.x * (long long)kFxThreads + threadIdx.x; k < n; k += (long long)gridDim.x * kFxThreads) {
        const double zk = __ldg(z + k), rk = __ldg(r + k);
        v[1] = fma(zk, rk, v[1]);
        v[2] = fma(zk, __ldg(w + k), v[2]);
        if (!first) {
            v[0] = fma(zk, __ldg(q + k), v[0]);
            v[3] = fma(__ldg(p + k), rk, v[3]);
        }
    }
    fx_block_store<4>(v, partials);
}

// p = z - beta p, q = w - beta q, x += alpha p, r -= alpha q; sums (r, r), (p, r)
__global__ void __launch_bounds__(kFxThreads) k_fx_update(long long n, const double* __restrict__ z,
                                                          const double* __restrict__ w, double* __restrict__ p,
                                                          double* __restrict__ q, double* __restrict__ x,
                                                          double* __restrict__ r, double alpha, double beta,
                                                          double* partials) {
    double v[2] = {0.0, 0.0};
    for (long long k = blockIdx.x * (long long)kFxThreads + threadIdx.x; k < n; k += (long long)gridDim.x * kFxThreads) {
        const double pk = fma(-beta, p[k], __ldg(z + k));
        const double qk = fma(-beta, q[k], __ldg(w + k));
        p[k] = pk;
        q[k] = qk;
        x[k] = fma(alpha, pk, x[k]);
        const double rk = fma(-alpha, qk, r[k]);
        r[k] = rk;
        v[0] = fma(rk, rk, v[0]);
        v[1] = fma(pk, rk, v[1]);
    }
    fx_block_store<2>(v, partials);
}

__global__ void k_fx_zero(long long n, double* __restrict__ a) {
    for (long long k = blockIdx.x * (long long)kFxThreads + threadIdx.x; k < n; k += (long long)gridDim.x * kFxThreads)
        a[k] = 0.0;
}

// sums of the last pass, read back to the host
int fx_read(const double* partials, int nb, double* out_dev, int ns, double* host, cudaStream_t s) {
    if (ns == 2)
        k_fx_finish<2><<<1, kFxThreads, 0, s>>>(partials, nb, out_dev);
    else
        k_fx_finish<4><<<1, kFxThreads, 0, s>>>(partials, nb, out_dev);
    KC_LAUNCH_CHECK("k_fx_finish");
    const void* hp = readback(out_dev, (size_t)ns * sizeof(double), s);
    if (!hp) return KC_ERR_CUDA;
    memcpy(host, hp, (size_t)ns * sizeof(double));
    return KC_OK;
}

}  // namespace
}  // namespace kc

using namespace kc;

extern "C" {

size_t kc_pcg_flexible_ws_bytes(long long n) { return n > 0 ? flex_layout(n).total : 0; }

int kc_pcg_flexible(const kc_system* A64, const kc_system* A32, const double* b, double* x,
                    const kc_unet_net* net, void* mg_ws, const kc_mg_opts* mg_opts, void* inner_ws,
                    size_t inner_ws_bytes, void* ws, size_t ws_bytes, const kc_solve_opts* opts, double eps_inner,
                    int max_outer, kc_solve_info* info, kc_flex_info* finfo, void* stream) {
    if (!A64 || !A32 || !b || !x || !opts || !mg_ws || !mg_opts)
        return set_error("kc_pcg_flexible: null argument"), KC_ERR_ARG;
    if (A64->dtype != KC_F64 || A32->dtype != KC_F32 || A64->n != A32->n || A64->stride != A32->stride)
        return set_error("kc_pcg_flexible: need matching FP64 and FP32 systems"), KC_ERR_ARG;
    if (A32->es != 1 || A32->cs != A32->n)
        return set_error("kc_pcg_flexible: the FP32 system must be SoA planes"), KC_ERR_ARG;
    if (net && (net->NX < 1 || (long long)net->NX * net->NY != A64->n || net->NY != A64->stride))
        return set_error("kc_pcg_flexible: network grid %d x %d does not match the system", net ? net->NX : 0,
                         net ? net->NY : 0),
               KC_ERR_ARG;
    const long long n = A64->n;
    const FlexLayout L = flex_layout(n);
    if (!ws || ws_bytes < L.total || ((uintptr_t)ws & 255))
        return set_error("kc_pcg_flexible: workspace %zu bytes (256-aligned) < required %zu", ws_bytes, L.total),
               KC_ERR_WORKSPACE;
    cudaStream_t s = as_stream(stream);
    char* base = (char*)ws;
    double *r = (double*)(base + L.r), *z = (double*)(base + L.z), *w = (double*)(base + L.w);
    double *p = (double*)(base + L.p), *q = (double*)(base + L.q);
    double* partials = (double*)(base + L.partials);
    double* out = (double*)(base + L.out);
    const int nb = fx_blocks(n);
    kc_flex_info F{};
    kc_solve_info I{};
    I.status = KC_MAXITER;
    int rc = KC_OK;

    if (opts->x0 != KC_X0_WARM) {
        k_fx_zero<<<nb, kFxThreads, 0, s>>>(n, x);
        KC_LAUNCH_CHECK("k_fx_zero");
    }
    // r = b - A x, ||r||^2, ||b||^2
    auto true_residual = [&](double* rr, double* bb) -> int {
        int e = kc_spmv(A64, x, w, stream);
        if (e) return e;
        k_fx_resid<<<nb, kFxThreads, 0, s>>>(n, b, w, r, partials);
        KC_LAUNCH_CHECK("k_fx_resid");
        double h[2];
        e = fx_read(partials, nb, out, 2, h, s);
        if (e) return e;
        *rr = h[0];
        if (bb) *bb = h[1];
        return KC_OK;
    };
    double rr = 0.0, bb = 0.0;
    if ((rc = true_residual(&rr, &bb))) return rc;
    I.r0 = std::sqrt(rr);
    double rel = bb > 0 ? std::sqrt(rr / bb) : 0.0, prev_rel = INFINITY, pq_prev = 0.0, pr_prev = 0.0;
    int stalls = 0;
    bool first = true;   // no previous direction (start, or after a restart on the true residual)
    long long inner_total = 0;
    for (int k = 0;; ++k) {
        if (!std::isfinite(rr) || !std::isfinite(bb)) {
            I.status = KC_NONFINITE;
            break;
        }
        if (bb == 0.0 || rel < opts->eps) {
            // confirm on the true residual (the recurrence can drift from it)
            double rt = 0.0;
            if ((rc = true_residual(&rt, nullptr))) return rc;
            rel = bb > 0 ? std::sqrt(rt / bb) : 0.0;
            rr = rt;
            if (bb == 0.0 || rel < opts->eps) {
                I.status = KC_OK;
                break;
            }
            first = true;   // restart the recurrence from the true residual
        }
        if (rel > 0.9 * prev_rel) {
            if (++stalls >= 2) {
                I.status = KC_STALL;
                break;
            }
        } else {
            stalls = 0;
        }
        if (k >= max_outer || inner_total >= opts->max_iter) {
            I.status = KC_MAXITER;
            break;
        }
        prev_rel = rel;
        // ---- preconditioner application z = P_k(r)
        bool learned = false;
        if (k == 0 && net) {
            if ((rc = kc_unet_predict(net, r, (const float*)A32->coef, z, stream))) return rc;
            learned = true;
            F.learned_used = 1;
        }
        for (int attempt = 0; attempt < 2; ++attempt) {
            if (!learned) {
                k_fx_zero<<<nb, kFxThreads, 0, s>>>(n, z);
                KC_LAUNCH_CHECK("k_fx_zero");
                kc_solve_opts io = *opts;
                io.x0 = KC_X0_ZERO;
                io.rel_to = KC_REL_B;
                io.eps = std::max(eps_inner, 0.5 * opts->eps / std::max(rel, 1e-300));
                io.max_iter = opts->max_iter - inner_total;
                io.history = nullptr;
                io.history_len = 0;
                kc_solve_info ii{};
                rc = kc_pcg_refined(A64, A32, r, z, nullptr, mg_ws, mg_opts, inner_ws, inner_ws_bytes, &io, eps_inner,
                                    1, &ii, stream);
                if (rc < 0) return rc;
                inner_total += ii.iters;
            }
            // ---- w = A z and the inner products of the new direction
            if ((rc = kc_spmv(A64, z, w, stream))) return rc;
            k_fx_dots<<<nb, kFxThreads, 0, s>>>(n, z, w, r, p, q, first ? 1 : 0, partials);
            KC_LAUNCH_CHECK("k_fx_dots");
            double d[4];
            if ((rc = fx_read(partials, nb, out, 4, d, s))) return rc;
            const double beta = first ? 0.0 : d[0] / pq_prev;
            const double pr = d[1] - beta * (first ? 0.0 : d[3]);
            const double pqv = d[2] - 2.0 * beta * d[0] + beta * beta * (first ? 0.0 : pq_prev);
            const bool ok = std::isfinite(beta) && std::isfinite(pr) && std::isfinite(pqv) && pqv > 0.0;
            if (!ok) {
                if (learned) {          // a useless network direction: a multigrid pass instead
                    F.learned_rejected = 1;
                    learned = false;
                    continue;
                }
                I.status = std::isfinite(pqv) ? KC_BREAKDOWN_RHO : KC_NONFINITE;
                break;
            }
            const double alpha = pr / pqv;
            k_fx_update<<<nb, kFxThreads, 0, s>>>(n, z, w, p, q, x, r, alpha, beta, partials);
            KC_LAUNCH_CHECK("k_fx_update");
            double u[2];
            if ((rc = fx_read(partials, nb, out, 2, u, s))) return rc;
            rr = u[0];
            pr_prev = u[1];
            pq_prev = pqv;
            first = false;
            rel = bb > 0 ? std::sqrt(rr / bb) : 0.0;
            F.outer += 1;
            break;
        }
        if (I.status == KC_BREAKDOWN_RHO || I.status == KC_NONFINITE) break;
    }
    (void)pr_prev;
    I.iters = inner_total;
    I.refinements = F.outer;
    I.rel_res = rel;
    if (info) *info = I;
    if (finfo) *finfo = F;
    return I.status;
}

}  // extern "C"
