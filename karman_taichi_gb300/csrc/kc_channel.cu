// Native SIMPLE time step and the batched executor.
//
// kc_channel_step runs one time step of the channel case entirely in C++:
// the outer loop of karman_taichi.py:633-659 / simple.py:270-281 over the
// library's own entry points (assembly, linear solves, relaxation, outlet,
// pressure correction, correction), reading back one scalar (the mass
// residual) per outer iteration, then u0 <- u, v0 <- v (time_forward,
// karman_taichi.py:617-622).  It makes exactly the calls, with the same
// options, as karman_taichi_gb300.channel.ChannelSolver.step, so both give
// bitwise identical fields.
//
// kc_channel_batch_step steps many independent instances with a pool of
// native threads, each instance on its own stream: no interpreter between the
// launches of small instances, and their kernels overlap on the GPU.
#include "kc_common.cuh"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

using namespace kc;

namespace {

kc_system sys_of(long long NX, long long NY, const void* coef, int dtype, int form) {
    kc_system A{};
    A.n = NX * NY;
    A.cs = NX * NY;
    A.es = 1;
    A.coef = coef;
    A.stride = (int)NY;
    A.dtype = dtype;
    A.form = form;
    return A;
}

// sweeps the Gauss-Seidel momentum solves may take before the refined BiCGSTAB takes over
constexpr long long kMomentumSweeps = 200;
// inner tolerance of the one-sweep Gauss-Seidel path of the refined momentum solve (systems whose
// rows link across their ends; the padded channel systems take 12 sweeps per pass, no inner test)
constexpr double kEpsInnerGs = 1e-5;

kc_solve_opts opts_of(double eps, long long max_iter, int rel_to, int check_every, int use_graph, int persistent) {
    kc_solve_opts o{};
    o.eps = eps;
    o.max_iter = max_iter;
    o.x0 = KC_X0_ZERO;
    o.precond = KC_PRECOND_NONE;
    o.omega_break = 0;
    o.rel_to = rel_to;
    o.check_every = check_every;
    o.use_graph = use_graph;
    o.persistent = persistent;
    o.history = nullptr;
    o.history_len = 0;
    return o;
}

// One momentum / plain system solve as ChannelSolver._solve does it; *fell_back
// is set when the Gauss-Seidel solve missed eps and the refined BiCGSTAB took over.
int solve_sys(const kc_channel* c, const kc_system& A64, const kc_system& A32, const double* b, double* x, void* ws,
              size_t ws_bytes, kc_solve_info* info, bool* fell_back, cudaStream_t s) {
    *fell_back = false;
    if (c->precision == KC_F64) {
        const kc_solve_opts o = opts_of(c->eps, A64.n, KC_REL_R0, 0, c->use_graph, c->persistent);
        return kc_bicgstab(&A64, b, x, nullptr, ws, ws_bytes, &o, info, s);
    }
    long long before = 0;
    if (c->momentum == KC_MOMENTUM_RBGS_REFINED) {
        // FP32 red-black Gauss-Seidel sweeps in FP64 refinement from the previous outer
        // iteration's u*, v*; the refined BiCGSTAB takes over, from where they stopped, if they miss eps
        kc_solve_opts og = opts_of(c->eps, kMomentumSweeps, KC_REL_R0, 0, c->use_graph, 0);
        og.x0 = KC_X0_WARM;
        const int rc = kc_rbgs_refined(&A64, &A32, b, x, ws, ws_bytes, &og, kEpsInnerGs, 30, info, s);
        if (rc < 0 || info->status == KC_OK) return rc;
        before = info->iters;
        *fell_back = true;
    } else if (c->momentum == KC_MOMENTUM_RBGS) {
        // red-black Gauss-Seidel from the previous outer iteration's u*, v*; the
        // refined BiCGSTAB takes over, from where it stopped, if it misses eps
        kc_solve_opts og = opts_of(c->eps, kMomentumSweeps, KC_REL_B, 0, c->use_graph, 0);
        og.x0 = KC_X0_WARM;
        const int rc = kc_rbgs(&A64, b, x, ws, ws_bytes, &og, info, s);
        if (rc < 0 || info->status == KC_OK) return rc;
        before = info->iters;
        *fell_back = true;
    }
    kc_solve_opts o = opts_of(c->eps, 50 * A64.n, KC_REL_R0, 0, c->use_graph, c->persistent);
    o.x0 = KC_X0_WARM;   // from the previous outer iteration's u*, v*
    const int rc = kc_bicgstab_refined(&A64, &A32, b, x, ws, ws_bytes, &o, c->eps_inner, 30, info, s);
    info->iters += before;
    return rc;
}

// ring of the last p' solutions in ws_recycle: slot q at q * n doubles
double* ring_slot(const kc_channel* c, int q) {
    const long long n = (long long)(c->phys.nx + 2) * (c->phys.ny + 2);
    return (double*)c->ws_recycle + (size_t)q * n;
}
// the stored solutions, newest first
int ring_vectors(const kc_channel* c, const double** Z) {
    const int m = c->rstate->count;
    for (int i = 0; i < m; ++i) Z[i] = ring_slot(c, ((c->rstate->head - 1 - i) % c->recycle + c->recycle) % c->recycle);
    return m;
}

// A second stream per host thread and device: the multigrid setup of a p'
// solve (launch-latency-bound: one small launch per level and a one-block
// coarsest inverse) runs on it while the recycled guess (FP64-pipe-bound)
// runs on the caller's stream; the caller's stream then waits for it.
struct SideStream {
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    ~SideStream() {
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        if (s) cudaStreamDestroy(s);
    }
};
SideStream* side_stream() {
    static thread_local SideStream side[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        set_error("side stream: no current device below 64");
        return nullptr;
    }
    SideStream& d = side[dev];
    if (!d.s) {
        cudaError_t e = cudaStreamCreateWithFlags(&d.s, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&d.fork, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&d.join, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            cuda_status(e, "side stream");
            return nullptr;
        }
    }
    return &d;
}

}  // namespace

extern "C" {

size_t kc_channel_recycle_ws_bytes(long long n_p, int recycle) {
    if (n_p < 1 || recycle < 1 || recycle > KC_RECYCLE_MAX) return 0;
    return align256((size_t)recycle * n_p * sizeof(double)) + align256((size_t)n_p * sizeof(double)) +
           kc_recycle_ws_bytes(n_p, recycle);
}

int kc_channel_step(const kc_channel* c, kc_channel_stats* st, void* stream) {
    if (!c) return set_error("kc_channel_step: null channel"), KC_ERR_ARG;
    if (c->phys.mode != KC_MODE_CHANNEL) return set_error("kc_channel_step: phys.mode must be KC_MODE_CHANNEL"), KC_ERR_ARG;
    if (c->precision != KC_F64 && c->precision != KC_F32) return set_error("kc_channel_step: bad precision"), KC_ERR_ARG;
    if (c->momentum != KC_MOMENTUM_BICGSTAB && c->momentum != KC_MOMENTUM_RBGS &&
        c->momentum != KC_MOMENTUM_RBGS_REFINED)
        return set_error("kc_channel_step: bad momentum solver %d", c->momentum), KC_ERR_ARG;
    const bool mixed = c->precision == KC_F32;
    if (mixed && (!c->coef_u32 || !c->coef_v32 || !c->coef_p32 || !c->b_u32 || !c->b_v32 || !c->b_p32 || !c->mg_ws))
        return set_error("kc_channel_step: mixed precision needs the FP32 systems and a multigrid workspace"),
               KC_ERR_ARG;
    cudaStream_t s = as_stream(stream);
    const kc_phys* P = &c->phys;
    const long long nx = P->nx, ny = P->ny;
    const kc_system Au = sys_of(nx + 3, ny + 2, c->coef_u, KC_F64, KC_FORM_STANDARD);
    const kc_system Av = sys_of(nx + 2, ny + 3, c->coef_v, KC_F64, KC_FORM_STANDARD);
    const kc_system Ap = sys_of(nx + 2, ny + 2, c->coef_p, KC_F64, KC_FORM_STANDARD);
    const kc_system Au32 = sys_of(nx + 3, ny + 2, c->coef_u32, KC_F32, KC_FORM_STANDARD);
    const kc_system Av32 = sys_of(nx + 2, ny + 3, c->coef_v32, KC_F32, KC_FORM_STANDARD);
    const kc_system Ap32 = sys_of(nx + 2, ny + 2, c->coef_p32, KC_F32, KC_FORM_LAPLACIAN);
    kc_channel_stats S{};
    int rc = KC_OK;
    double mass = 0.0;
    const bool recycling = mixed && !c->learned && c->recycle > 0;
    double* rc_x0 = nullptr;
    void* rc_ws = nullptr;
    size_t rc_ws_bytes = 0;
    if (recycling) {
        if (c->recycle > KC_RECYCLE_MAX || !c->rstate || !c->ws_recycle ||
            c->ws_recycle_bytes < kc_channel_recycle_ws_bytes(Ap.n, c->recycle) || ((uintptr_t)c->ws_recycle & 255))
            return set_error("kc_channel_step: recycle = %d needs rstate and a 256-aligned ws_recycle of %zu bytes",
                             c->recycle, kc_channel_recycle_ws_bytes(Ap.n, c->recycle)),
                   KC_ERR_WORKSPACE;
        rc_x0 = (double*)((char*)c->ws_recycle + align256((size_t)c->recycle * Ap.n * sizeof(double)));
        rc_ws = (char*)rc_x0 + align256((size_t)Ap.n * sizeof(double));
        rc_ws_bytes = kc_recycle_ws_bytes(Ap.n, c->recycle);
    }
    for (int outer = 0; outer < c->max_outer; ++outer) {
        rc = kc_assemble_momentum(P, c->u, c->v, c->p, c->u0, c->v0, c->solid, c->coef_u, c->b_u, c->coef_v, c->b_v,
                                  c->coef_u32, c->b_u32, c->coef_v32, c->b_v32, s);
        if (rc < 0) return rc;
        kc_solve_info iu{}, iv{}, ip{};
        bool fu = false, fv = false;
        rc = solve_sys(c, Au, Au32, c->b_u, c->u_mid, c->ws_u, c->ws_u_bytes, &iu, &fu, s);
        if (rc < 0) return rc;
        rc = solve_sys(c, Av, Av32, c->b_v, c->v_mid, c->ws_v, c->ws_v_bytes, &iv, &fv, s);
        if (rc < 0) return rc;
        S.fallbacks += (int)fu + (int)fv;
        rc = kc_relax_velocity(P, c->solid, c->u_mid, c->v_mid, c->u, c->v, nullptr, c->rws, s);
        if (rc < 0) return rc;
        rc = kc_outlet_conserve(P, c->u, s);
        if (rc < 0) return rc;
        rc = kc_assemble_pcorr(P, c->u, c->v, c->coef_u, c->coef_v, c->solid, c->coef_p, c->b_p, c->coef_p32,
                               c->b_p32, nullptr, c->mass, c->rws, s);
        if (rc < 0) return rc;
        if (mixed) {
            const double* Z[KC_RECYCLE_MAX];
            const int m = recycling ? ring_vectors(c, Z) : 0;
            if (m > 0) {
                // the hierarchy on the side stream while the guess forms on this one: the
                // projection onto the last solutions (kc_recycle_guess)
                SideStream* sd = side_stream();
                if (!sd) return KC_ERR_CUDA;
                KC_CUDA(cudaEventRecord(sd->fork, s));
                KC_CUDA(cudaStreamWaitEvent(sd->s, sd->fork, 0));
                rc = kc_mg_setup(&Ap32, c->mg_ws, c->mg_ws_bytes, &c->mg_opts, sd->s);
                if (rc < 0) return rc;
                KC_CUDA(cudaEventRecord(sd->join, sd->s));
                rc = kc_recycle_guess(&Ap, c->b_p, Z, m, rc_x0, rc_ws, rc_ws_bytes, nullptr, s);
                if (rc < 0) return rc;
                KC_CUDA(cudaStreamWaitEvent(s, sd->join, 0));
            } else {
                rc = kc_mg_setup(&Ap32, c->mg_ws, c->mg_ws_bytes, &c->mg_opts, s);
                if (rc < 0) return rc;
            }
            const kc_solve_opts o =
                opts_of(c->eps, 50 * Ap.n, KC_REL_B, c->check_every_p > 0 ? c->check_every_p : 4, c->use_graph, 0);
            if (c->learned) {
                // the network as the first preconditioner application of a flexible CG
                kc_flex_info fi{};
                rc = kc_pcg_flexible(&Ap, &Ap32, c->b_p, c->pcor, c->learned, c->mg_ws, &c->mg_opts, c->ws_p,
                                     c->ws_p_bytes, c->ws_flex, c->ws_flex_bytes, &o, c->eps_inner_p, 30, &ip, &fi, s);
                if (rc < 0) return rc;
                S.learned += fi.learned_used;
                S.learned_rejected += fi.learned_rejected;
            } else {
                const double* x0 = m > 0 ? rc_x0 : nullptr;
                rc = kc_pcg_refined(&Ap, &Ap32, c->b_p, c->pcor, x0, c->mg_ws, &c->mg_opts, c->ws_p,
                                    c->ws_p_bytes, &o, c->eps_inner_p, 30, &ip, s);
                if (rc < 0) return rc;
            }
            if (ip.status != KC_OK) {   // accelerated solve stalled: plain BiCGSTAB is the fallback
                ++S.fallbacks;
                const long long before = ip.iters;
                const kc_solve_opts of = opts_of(c->eps, Ap.n, KC_REL_R0, 0, c->use_graph, c->persistent);
                rc = kc_bicgstab(&Ap, c->b_p, c->pcor, nullptr, c->ws_p, c->ws_p_bytes, &of, &ip, s);
                if (rc < 0) return rc;
                ip.iters += before;
            }
        } else {
            const kc_solve_opts o = opts_of(c->eps, Ap.n, KC_REL_R0, 0, c->use_graph, c->persistent);
            rc = kc_bicgstab(&Ap, c->b_p, c->pcor, nullptr, c->ws_p, c->ws_p_bytes, &o, &ip, s);
            if (rc < 0) return rc;
        }
        if (recycling) {   // the solution joins the ring (the oldest leaves)
            rc = kc_copy(ring_slot(c, c->rstate->head), c->pcor, (size_t)Ap.n * sizeof(double), s);
            if (rc < 0) return rc;
            c->rstate->head = (c->rstate->head + 1) % c->recycle;
            c->rstate->count = std::min(c->rstate->count + 1, c->recycle);
        }
        rc = kc_correct(P, c->pcor, c->coef_u, c->coef_v, c->solid, c->u, c->v, c->p, c->pmax, c->rws, s);
        if (rc < 0) return rc;
        S.outer += 1;
        S.it_u += iu.iters;
        S.it_v += iv.iters;
        S.it_p += ip.iters;
        const bool nonfinite = iu.status == KC_NONFINITE || iv.status == KC_NONFINITE || ip.status == KC_NONFINITE;
        if (nonfinite)
            S.status = KC_NONFINITE;
        else if ((iu.status != KC_OK || iv.status != KC_OK || ip.status != KC_OK) && S.status == KC_OK)
            S.status = KC_MAXITER;
        const void* hp = readback(c->mass, sizeof(double), s);
        if (!hp) return KC_ERR_CUDA;
        memcpy(&mass, hp, sizeof(double));
        S.mass = mass;
        // a NaN or Inf in the fields (the reference has no such check) ends the step: the outer
        // loop would only repeat it; the status tells the caller
        if (nonfinite || !std::isfinite(mass)) {
            S.status = KC_NONFINITE;
            break;
        }
        if (mass <= c->mass_tol) break;
    }
    rc = kc_copy(c->u0, c->u, (size_t)((nx + 3) * (ny + 2)) * sizeof(double), s);
    if (rc < 0) return rc;
    rc = kc_copy(c->v0, c->v, (size_t)((nx + 2) * (ny + 3)) * sizeof(double), s);
    if (rc < 0) return rc;
    if (st) *st = S;
    return KC_OK;
}

int kc_channel_batch_step(const kc_channel* const* chs, int n, void* const* streams, int workers, int steps,
                          kc_channel_stats* stats) {
    if (!chs || !streams || n < 0 || steps < 0) return set_error("kc_channel_batch_step: bad arguments"), KC_ERR_ARG;
    if (n == 0 || steps == 0) return KC_OK;
    int dev = 0;
    KC_CUDA(cudaGetDevice(&dev));
    workers = std::max(1, std::min(workers, n));
    // the first failing instance's status and message are recorded together,
    // under one lock, so the message always belongs to the returned status
    std::atomic<int> first_err{0};
    std::mutex err_mu;
    std::string first_msg;
    auto record = [&](int code, const std::string& msg) {
        std::lock_guard<std::mutex> lk(err_mu);
        if (first_err.load() == 0) {
            first_msg = msg;
            first_err.store(code);
        }
    };
    std::vector<std::thread> pool;
    pool.reserve(workers);
    for (int w = 0; w < workers; ++w) {
        pool.emplace_back([&, w] {
            if (cudaSetDevice(dev) != cudaSuccess) {
                record(KC_ERR_CUDA, "cudaSetDevice failed in a batch worker");
                return;
            }
            for (int k = w; k < n; k += workers) {
                for (int t = 0; t < steps && first_err.load() == 0; ++t) {
                    const int rc = kc_channel_step(chs[k], stats ? &stats[k] : nullptr, streams[k]);
                    if (rc < 0) {
                        record(rc, "instance " + std::to_string(k) + ": " + kc_last_error());
                        return;
                    }
                }
            }
        });
    }
    for (auto& t : pool) t.join();
    const int rc = first_err.load();
    if (rc) set_error("kc_channel_batch_step: %s", first_msg.c_str());
    return rc;
}

}  // extern "C"
