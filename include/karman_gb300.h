/*
 * karman_gb300.h -- C ABI of libkarman_gb300.so, the GB300 (sm_103a) kernels
 * behind the karman_taichi SIMPLE hot path.
 *
 * Everything crossing this boundary is a plain pointer, size or POD struct:
 * device arrays are caller-owned (allocated by the caller, e.g. from torch),
 * the stream is a cudaStream_t passed as void*, and no exception, abort or
 * device trap crosses the ABI.  Every entry point returns an int status:
 *     0          success (for solvers: converged)
 *     > 0        a solver outcome (KC_MAXITER, KC_BREAKDOWN_*, KC_NONFINITE, KC_STALL)
 *     < 0        an argument or CUDA error (KC_ERR_*); kc_last_error() explains it.
 * Calls are stream ordered.  A workspace must not be shared by calls that can
 * run concurrently; otherwise the functions are reentrant.
 *
 * Linear systems are 5-point stencils on a flat index k in [0, n) with far
 * stride S (for a padded 2-D field [NX][NY], k = i*NY + j and S = NY):
 *     y[k] = c0 x[k] + c1 x[k-S] + c2 x[k+S] + c3 x[k+1] + c4 x[k-1]
 * with reads outside [0, n) returning 0.  Component c is read at
 * coef[c*cs + k*es]: SoA planes use (cs = n, es = 1); the reference's
 * coef[i,j,0..4] array-of-structs layout is (cs = 1, es = 5).
 */
#ifndef KARMAN_GB300_H
#define KARMAN_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define KC_OK               0
#define KC_MAXITER          1   /* iteration cap reached                           */
#define KC_BREAKDOWN_RHO    2   /* rho = (r, r~) == 0   (bicgsolver.py:96-98)      */
#define KC_BREAKDOWN_OMEGA  3   /* omega == 0           (karman_taichi.py:451-454) */
#define KC_NONFINITE        4   /* a NaN/Inf appeared in a scalar of the recurrence */
#define KC_STALL            5   /* preconditioned residual stopped decreasing      */
#define KC_ERR_ARG        (-1)
#define KC_ERR_CUDA       (-2)
#define KC_ERR_WORKSPACE  (-3)
#define KC_ERR_UNSUPPORTED (-4)

#define KC_F64 0
#define KC_F32 1

#define KC_X0_ZERO 0   /* cold start x = 0, r = b          (bicgsolver.py:21-36)     */
#define KC_X0_WARM 1   /* warm start r = b - A x           (karman_taichi.py:362-371) */

#define KC_PRECOND_NONE   0   /* M = I                    (bicgsolver.py:48-58)          */
#define KC_PRECOND_JACOBI 1   /* right Jacobi, p^ = M^-1 p (karman_taichi.py:398-399,418) */

#define KC_REL_R0 0   /* stop when ||r|| / ||r0|| < eps (reference definition) */
#define KC_REL_B  1   /* stop when ||r|| / ||b||  < eps                         */

/* Coefficient forms.  KC_FORM_STANDARD: component 0 is aP and
 *   y = aP x + sum_nb a_nb x_nb.
 * KC_FORM_LAPLACIAN: component 0 holds the row sum rs = aP + sum_nb a_nb and
 *   y = rs x + sum_nb a_nb (x_nb - x)   (the same operator, written so that
 * rounding the links to FP32 cannot perturb the row sums -- zero for every
 * fluid row of the pressure-correction system, whose only Dirichlet
 * condition is the outlet). */
#define KC_FORM_STANDARD  0
#define KC_FORM_LAPLACIAN 1

typedef struct {
    long long n;          /* number of unknowns                                 */
    long long cs, es;     /* coefficient component stride, element stride       */
    const void* coef;     /* 5 components aP|rs, aW(k-S), aE(k+S), aN(k+1), aS(k-1) */
    int stride;           /* far stride S                                       */
    int dtype;            /* KC_F64 or KC_F32 (vectors and coefficients)        */
    int form;             /* KC_FORM_STANDARD or KC_FORM_LAPLACIAN              */
    int pad_;
} kc_system;

typedef struct {
    double eps;           /* relative residual tolerance                        */
    long long max_iter;   /* iteration cap (reference: NX*NY or 100*n)          */
    int x0;               /* KC_X0_ZERO | KC_X0_WARM                             */
    int precond;          /* KC_PRECOND_NONE | KC_PRECOND_JACOBI                 */
    int omega_break;      /* stop on omega == 0 (karman_taichi.py:451)           */
    int rel_to;           /* KC_REL_R0 | KC_REL_B                                */
    int check_every;      /* host polls convergence every N iterations (0: auto)*/
    int use_graph;        /* capture iteration chunks in a CUDA graph            */
    int persistent;       /* 1: one cooperative launch runs the whole solve      */
    int pad_;
    double* history;      /* device array or NULL: history[k] = ||r_k||_2       */
    long long history_len;/* capacity of history (entries beyond are dropped)   */
} kc_solve_opts;

typedef struct {
    int status;           /* KC_OK or a solver outcome                          */
    int refinements;      /* refinement sweeps (kc_bicgstab_refined only)       */
    long long iters;      /* completed iterations (summed over sweeps)          */
    double rel_res;       /* final relative residual                            */
    double r0;            /* ||r0|| (2-norm)                                     */
} kc_solve_info;

/* ---- library ------------------------------------------------------------- */
int         kc_version(void);
const char* kc_status_str(int status);
const char* kc_last_error(void);
int         kc_device_count(void);
/* Kernels launched by this library in this process (graph nodes included). */
long long   kc_launch_count(void);
/* sizeof of an ABI struct by name ("kc_system", "kc_channel", ...; 0 if unknown). */
size_t      kc_struct_size(const char* name);
/* Solves that run in captured chunks of iterations (opts->use_graph) keep the
 * instantiated graphs in a process-wide cache keyed by every pointer and
 * parameter a graph bakes in.  No counterpart in the reference (it has no
 * graphs).  kc_graph_cache_size: entries held.  kc_graph_cache_limit(cap):
 * sets the most entries kept (least recently used evicted first; cap = 0
 * only queries) and returns the previous limit (default 1024).  A graph
 * evicted while another thread launches it is destroyed after that launch. */
size_t      kc_graph_cache_size(void);
size_t      kc_graph_cache_limit(size_t cap);
/* Failure testing.  The persistent (cooperative) solvers meet at grid
 * barriers whose waits give up after a bounded number of polls (about 0.5 s);
 * the solve then ends with KC_ERR_CUDA ("grid barrier timed out") and the
 * context stays usable.  This sets that bound for later launches (0: the
 * default) and returns the previous setting, so a test can make a wait run
 * out without any block hanging.  No counterpart in the reference. */
unsigned    kc_debug_barrier_spin_limit(unsigned polls);
/* The multigrid-CG refinement (kc_pcg_refined with opts->use_graph) runs as
 * one CUDA graph launch: a conditional WHILE node over the refinement passes
 * (FP64 residual, the pass's decisions in a one-thread kernel, the inner
 * solve) whose body holds a nested WHILE node over the CG iterations; one
 * readback at the end.  enable = 0 runs the refinement passes from the host
 * and the CG iterations in graph-captured chunks with a host check between
 * chunks (the same kernels, decisions and results; profilers list kernels of
 * such graphs, not those under a conditional node), 1 the device loops;
 * returns the previous setting; enable < 0 only queries: bit 0 the CG loop,
 * bit 1 the refinement loop (each cleared once the driver refuses it).  No
 * counterpart in the reference. */
int         kc_device_loop(int enable);

/* ---- stencil linear algebra --------------------------------------------- */
/* y = A x.  Replaces BICGSolver.compute_Ap/compute_As (bicgsolver.py:65-76),
 * CGSolver.compute_Ap/compute_Ax (cgsolver.py:56-66) and the 7-offset gather
 * of karman_taichi.py:362-366, 403-407. */
int kc_spmv(const kc_system* A, const void* x, void* y, void* stream);

/* out_dev[0] = sum_k p[k] q[k] in FP64 with a deterministic two-stage
 * reduction.  Replaces CGSolver.reduce (cgsolver.py:49-54). */
size_t kc_dot_ws_bytes(long long n);
int kc_dot(int dtype, long long n, const void* p, const void* q, double* out_dev,
           void* ws, size_t ws_bytes, void* stream);

/* BiCGSTAB.  Replaces BICGSolver.solve (bicgsolver.py:88-135) and the
 * bicgstab kernel of karman_taichi.py:342-456.  x is overwritten (cold start)
 * or used as the initial guess (warm start).  M is the Jacobi diagonal (may
 * differ from A's, as in karman_taichi.py:218) or NULL. */
size_t kc_bicgstab_ws_bytes(long long n, int stride, int dtype);
int kc_bicgstab(const kc_system* A, const void* b, void* x, const void* M,
                void* ws, size_t ws_bytes, const kc_solve_opts* opts,
                kc_solve_info* info, void* stream);

/* BiCGSTAB that allocates nothing.  No counterpart in the reference: it is
 * for callers that cannot allocate device memory for a workspace -- a plugin
 * inside a host framework whose allocator owns all device memory, or a loop
 * in which cudaMalloc/cudaFree (which can synchronise the device) are not
 * acceptable.  Same arguments and results as kc_bicgstab, minus the
 * workspace: scratch comes from a static device array built into the library
 * (about 4.5 MB, held on every GPU that loads the library until exit), which
 * limits the system to KC_NOALLOC_MAX_N unknowns; larger systems are
 * rejected with KC_ERR_ARG and an explanation in kc_last_error().
 * The first call on a device looks up that array's device address (once per
 * device, with the device current); the address is kept for the life of the
 * process and is not looked up again after cudaDeviceReset.  Every call
 * synchronises with the host (it reads the solver state back), so no call can
 * be captured into a CUDA graph.  Every call uses the same array and each
 * call clears the state it needs, but calls that overlap on the GPU
 * (concurrent streams, threads or processes sharing a context) race on it.
 * Iterations are launched directly (opts->use_graph is ignored).  Each call
 * waits on the host for its solve: the solver state is copied back into a
 * static pageable host buffer (no pinned host memory is allocated either). */
#define KC_NOALLOC_MAX_N 65536
int kc_bicgstab_noalloc(const kc_system* A, const void* b, void* x, const void* M,
                        const kc_solve_opts* opts, kc_solve_info* info, void* stream);

/* Conjugate gradients.  Replaces CGSolver.solve (cgsolver.py:83-114). */
size_t kc_cg_ws_bytes(long long n, int stride, int dtype);
int kc_cg(const kc_system* A, const void* b, void* x, void* ws, size_t ws_bytes,
          const kc_solve_opts* opts, kc_solve_info* info, void* stream);

/* Mixed precision: FP64 residual r = b - A64 x, FP32 BiCGSTAB correction on
 * A32 (FP64 inner products), x += d, until ||r||/||b|| < opts->eps.  Each
 * sweep solves to eps_inner, or only as far as the target needs
 * (0.5 eps / the current ||r||/||b||) when that is looser.  opts->x0 =
 * KC_X0_WARM starts from x (a warm start, as karman_taichi.py:362-371 does);
 * otherwise x = 0.  The momentum solves of the mixed SIMPLE path. */
size_t kc_refined_ws_bytes(long long n, int stride);
int kc_bicgstab_refined(const kc_system* A64, const kc_system* A32, const double* b,
                        double* x, void* ws, size_t ws_bytes, const kc_solve_opts* opts,
                        double eps_inner, int max_refine, kc_solve_info* info, void* stream);
/* The same refinement with FP32 red-black Gauss-Seidel sweeps as the inner
 * solver (the Gauss-Seidel counterpart of the reference's Jacobi solves,
 * pressure_valid.py:192-233), for diagonally dominant systems such as the
 * momentum rows.  Systems whose rows never link across their ends (checked
 * on the device): opts->check_every sweeps per refinement pass (0: 12), two
 * per launch on staged tiles, no inner residual test; others: one sweep per
 * launch, each pass to eps_inner.  opts->max_iter caps the sweeps in all.
 * info->iters counts sweeps.  Workspace: kc_refined_ws_bytes. */
int kc_rbgs_refined(const kc_system* A64, const kc_system* A32, const double* b,
                    double* x, void* ws, size_t ws_bytes, const kc_solve_opts* opts,
                    double eps_inner, int max_refine, kc_solve_info* info, void* stream);

/* One Jacobi sweep (FP64, standard form): x_mid = (b - sum_nb a_nb x_nb) / aP,
 * y = (1 - omega) x + omega x_mid on the cells (i, j) of the [n/stride][stride]
 * view with i0 <= i < i1, j0 <= j < j1 (y = x elsewhere and where aP = 0);
 * max_diff_dev[0] = max |x_mid - x| there.  Replaces jacobian_solve_u /
 * jacobian_solve_p (pressure_valid.py:192-233: region i in [2, nx] or [1, nx],
 * j in [1, ny], omega = alpha_u or 1) and quick_jacobian
 * (debug/20210828_karman_taihi.py:375-393: whole range, omega = 1).  Those
 * overwrite the iterate inside a parallel loop, an order the reference leaves
 * undefined; here every cell reads the previous iterate x (x != y).
 * ws: kc_jacobi_ws_bytes() bytes, zeroed before the first call. */
size_t kc_jacobi_ws_bytes(void);
int kc_jacobi(const kc_system* A, const double* b, const double* x, double* y, double omega,
              int i0, int i1, int j0, int j1, double* max_diff_dev, void* ws, size_t ws_bytes,
              void* stream);

/* Red-black Gauss-Seidel solve of an FP64 system (standard or Laplacian
 * form): the Gauss-Seidel counterpart of the reference's Jacobi solves
 * (pressure_valid.py:192-233; debug/20210828_karman_taihi.py:375-393), used
 * for the channel's momentum systems, whose time term makes them strongly
 * diagonally dominant.  One launch per sweep (the red cells, then the black
 * ones, of a tile; colour = parity of i + j of the [n/stride][stride] view),
 * which also sums the residual of the iterate it starts from: the stopping
 * test ||b - A x|| < eps * (||b|| for rel_to = KC_REL_B, else ||b - A x0||)
 * is checked one sweep late, after chunks of sweeps (check_every, or 4 up to
 * 16) launched as CUDA graphs.  opts: eps, max_iter (sweeps), x0, rel_to,
 * check_every, use_graph; precond must be KC_PRECOND_NONE.  Rows with a zero
 * diagonal keep their x.  ws: kc_rbgs_ws_bytes(n, stride) bytes.
 * info->iters: sweeps applied; info->rel_res: the last residual checked. */
size_t kc_rbgs_ws_bytes(long long n, int stride);
int kc_rbgs(const kc_system* A, const double* b, double* x, void* ws, size_t ws_bytes,
            const kc_solve_opts* opts, kc_solve_info* info, void* stream);

/* ---- multigrid preconditioner (FP32) --------------------------------------
 * The reference names multigrid as its missing next step (README.md:31;
 * debug/note.md:6); it has Jacobi only (karman_taichi.py:398-399).
 * Aggregation multigrid V-cycle for 2-D 5-point operators: 2x2 Galerkin
 * coarsening, red-black Gauss-Seidel smoothing with per-level weights
 * omega[l], coarse corrections scaled by alpha[l].  Links across the end of a
 * row of [n/stride][stride] are treated as links to a zero cell.
 * nu_pre / nu_post are the sweeps on level 0, nu_coarse (1..3 in the fused
 * cycle; <= 0 reads as 1) those on every level below; nu_pre = nu_post = 1
 * selects the fused cycle (two launches per level).
 * coarsest_sweeps = 0: coarsening stops at <= 128 cells, whose dense
 * operator is inverted at setup (exact coarsest solve; a non-positive pivot
 * falls back to 64 Jacobi sweeps); > 0: coarsening stops at <= 1024 cells,
 * solved by that many Jacobi sweeps.  tail > 0 (with the fused cycle and the
 * exact coarsest solve) runs the levels of at most `tail` cells and the
 * coarsest solve in one single-block launch, their arithmetic unchanged,
 * when their arrays fit the block's shared memory; 0 launches every level
 * separately.  The fused cycle's levels below level 0 with at least
 * big_cells cells use 64-wide tiles (16 x 60 owned cells at one sweep,
 * 12 x 56 at two, 8 x 52 at three), smaller ones 32-wide tiles (8 x 28,
 * 8 x 24, 8 x 20).  Neither
 * changes the result.  kc_mg_default_opts: nu 1/1 on level 0 and 2 below,
 * exact coarsest solve, omega 1.0 on level 0 and 1.5 below, alpha 1.9 on
 * level 0 and 2.0 below (the tuned setting for the channel's pressure
 * correction), tail 1536, big_cells 200000. */
#define KC_MG_MAX_LEVELS 16
typedef struct {
    int nu_pre, nu_post;          /* red-black sweeps before / after the coarse correction */
    int coarsest_sweeps;          /* 0: exact coarsest solve; > 0: Jacobi sweeps            */
    int max_levels;
    int tail;                     /* levels of at most this many cells in one launch (0: off) */
    int big_cells;                /* levels of at least this many cells use the large tiles */
    int nu_coarse;                /* red-black sweeps before / after on the levels below 0  */
    float omega[KC_MG_MAX_LEVELS];/* smoother weight per level                            */
    float alpha[KC_MG_MAX_LEVELS];/* coarse-correction scale per level                    */
} kc_mg_opts;
void   kc_mg_default_opts(kc_mg_opts* opts);
size_t kc_mg_ws_bytes(long long n, int stride, const kc_mg_opts* opts);
/* Builds the coarse levels of A32 (FP32) into mg_ws; re-run when A changes. */
int kc_mg_setup(const kc_system* A32, void* mg_ws, size_t mg_ws_bytes, const kc_mg_opts* opts, void* stream);
/* z = M r: one V-cycle (r, z: n floats). */
int kc_mg_apply(const kc_system* A32, void* mg_ws, const kc_mg_opts* opts, const float* r, float* z,
                void* stream);

/* Mixed precision with the multigrid preconditioner: FP64 residual
 * refinement around an FP32 right-preconditioned BiCGSTAB (FP32 vectors, FP64
 * iterate and inner products), stopping when ||b - A64 x|| / ||b|| <
 * opts->eps.  Each inner solve runs to a relative residual eps_inner; at most
 * max_refine of them.  x0 (nullable, FP64) is an initial guess; kc_mg_setup
 * must have been run on mg_ws.  No reference counterpart: the reference's
 * pressure solve is the plain or Jacobi BiCGSTAB above.  A correction that
 * raises the true residual is undone and the call returns KC_STALL with x
 * the best iterate. */
size_t kc_pbicgstab_ws_bytes(long long n, int stride);
int kc_pbicgstab_refined(const kc_system* A64, const kc_system* A32, const double* b, double* x,
                         const double* x0, void* mg_ws, const kc_mg_opts* mg_opts, void* ws,
                         size_t ws_bytes, const kc_solve_opts* opts, double eps_inner,
                         int max_refine, kc_solve_info* info, void* stream);
/* The same with multigrid-preconditioned CG as the inner solver, for
 * symmetric systems (the pressure correction: its links are the face
 * coefficients rho*dy^2/aP_face, shared by both cells of a face) -- one
 * operator and one V-cycle per iteration.  Workspace: kc_pbicgstab_ws_bytes.
 * A non-positive (p, A p) or (r, M r) ends the inner solve with
 * KC_BREAKDOWN_RHO.  The pressure-correction solve of the accelerated SIMPLE
 * path. */
int kc_pcg_refined(const kc_system* A64, const kc_system* A32, const double* b, double* x,
                   const double* x0, void* mg_ws, const kc_mg_opts* mg_opts, void* ws,
                   size_t ws_bytes, const kc_solve_opts* opts, double eps_inner,
                   int max_refine, kc_solve_info* info, void* stream);

/* Initial guess for the next system of a sequence by Galerkin projection onto
 * earlier solutions: x0 = Z y with (Z^T A Z) y = Z^T b, Z = [Z[0] .. Z[m-1]]
 * (FP64 n-vectors, newest first).  x0 minimises the error's A-norm over
 * span(Z), so for a symmetric positive definite A it starts no further from
 * the solution than x0 = 0.  The SIMPLE loop solves one p' system per outer
 * iteration (karman_taichi.py:633-659; simple.py:270-281) and successive
 * corrections keep their shape: with the last four solutions the guess's
 * relative residual is ~1e-4.  A vector whose Cholesky pivot falls below
 * 1e-12 of its diagonal is dropped with the older ones; *used (nullable)
 * gets the count kept.  m = 0 gives x0 = 0.  ws: kc_recycle_ws_bytes(n, m),
 * 256-byte aligned.  No counterpart in the reference. */
#define KC_RECYCLE_MAX 4
size_t kc_recycle_ws_bytes(long long n, int m);
int kc_recycle_guess(const kc_system* A64, const double* b, const double* const* Z, int m,
                     double* x0, void* ws, size_t ws_bytes, int* used, void* stream);
/* Ring of earlier solutions kept by a driver: count stored (<= capacity), head
 * the slot the next solution goes to. */
typedef struct {
    int count, head;
} kc_recycle_state;

/* The trained network applied from native code: features of A x = b (the p'
 * system: b FP64 [NX][NY], coef32 its FP32 Laplacian-form SoA planes), the
 * U-Net forward pass at half resolution, and x0 = the upsampled prediction
 * (FP64 [NX][NY]) -- the same kernels, in the same order, as the Python
 * trainer's forward pass.  params: the kc_unet_param_count() FP32
 * parameters, layer by layer (w [9][cout][cin], b [cout]; head w [16], b [1]);
 * params16: their BF16 copy.  ws: kc_unet_predict_ws_bytes(NX, NY), 256-byte
 * aligned (features and activations).  No counterpart in the reference (it
 * has no learned component). */
typedef struct {
    int NX, NY;
    const void* params;
    const void* params16;
    void* ws;
    size_t ws_bytes;
} kc_unet_net;
long long kc_unet_param_count(void);
size_t kc_unet_predict_ws_bytes(int NX, int NY);
int kc_unet_predict(const kc_unet_net* net, const double* b, const float* coef32, double* x0,
                    void* stream);

/* Flexible CG (FCG(1), FP64 outer vectors) for the symmetric pressure-correction
 * system with a changing preconditioner: its first application is the trained
 * network's prediction of A^-1 r (kc_unet_predict; net may be NULL), every
 * later one a multigrid-preconditioned FP32 CG pass on A z = r (one sweep of
 * kc_pcg_refined to eps_inner, inner_ws of kc_pbicgstab_ws_bytes).  This is the
 * network in the role of the reference's right-preconditioner hooks
 * p^ = M^-1 p, s^ = M^-1 s (bicgsolver.py:48-58; karman_taichi.py:398-399,
 * 418-419), with M changing between iterations.  Each direction is
 * A-orthogonalised against the previous one and its step length minimises
 * the error's A-norm, so a poor prediction costs one short step.  A network
 * direction that is not finite or not a descent direction is replaced by a
 * multigrid pass (finfo->learned_rejected).  Two outer iterations in a row
 * that cut ||b - A x|| by less than 10 % end the solve with KC_STALL (x the
 * last iterate): the caller falls back to the plain BiCGSTAB.  KC_OK once
 * ||b - A x|| / ||b|| < opts->eps on the true residual.  opts->x0:
 * KC_X0_WARM starts from x; opts->max_iter caps the inner CG iterations;
 * max_outer the outer ones.  info->iters: inner CG iterations;
 * info->refinements: outer iterations.  ws: kc_pcg_flexible_ws_bytes(n)
 * (5 FP64 vectors), 256-byte aligned; kc_mg_setup must have run on mg_ws. */
typedef struct {
    int learned_used;      /* the network's prediction was applied            */
    int learned_rejected;  /* ... and replaced: not finite or not descending  */
    int outer;             /* outer (flexible) iterations                     */
    int pad_;
} kc_flex_info;
size_t kc_pcg_flexible_ws_bytes(long long n);
int kc_pcg_flexible(const kc_system* A64, const kc_system* A32, const double* b, double* x,
                    const kc_unet_net* net, void* mg_ws, const kc_mg_opts* mg_opts, void* inner_ws,
                    size_t inner_ws_bytes, void* ws, size_t ws_bytes, const kc_solve_opts* opts,
                    double eps_inner, int max_outer, kc_solve_info* info, kc_flex_info* finfo,
                    void* stream);

/* ---- SIMPLE assembly and correction (staggered padded fields) ----------- */
#define KC_MODE_SIMPLE   0   /* simple.py set_bc incl. the east-wall aW term (simple.py:215) */
#define KC_MODE_BICGSIMP 1   /* bicgsimp.py: east-wall fix (:196), p' pinned at (1,1) (:146-151) */
#define KC_MODE_CHANNEL  2   /* velocity inlet, zero-gradient outlet, walls, blocked cells */

typedef struct {
    int nx, ny;               /* interior cells; u [nx+3][ny+2], v [nx+2][ny+3], p [nx+2][ny+2] */
    int mode;                 /* KC_MODE_*                                                       */
    int pad_;
    double dx, dy, rho, mu, dt;
    double U;                 /* channel inlet velocity                                          */
    double bc[4][2];          /* simple.py bc dict order w, e, n, s: [normal, tangential]        */
    double alpha_m, alpha_u, alpha_p;
} kc_phys;

/* Size of the small reduction workspace used by the kernels below. */
size_t kc_reduce_ws_bytes(void);

/* Momentum coefficients a_P..a_S and source for u and v faces with the
 * boundary conditions folded in.  Replaces compute_coef_u/compute_coef_v +
 * set_bc (simple.py:77-110, 172-216).  solid may be NULL.  The optional
 * FP32 outputs (NULL to skip) receive a rounded copy for the mixed path. */
int kc_assemble_momentum(const kc_phys* P, const double* u, const double* v,
                         const double* p, const double* u0, const double* v0,
                         const unsigned char* solid,
                         double* coef_u, double* b_u, double* coef_v, double* b_v,
                         float* coef_u32, float* b_u32, float* coef_v32, float* b_v32,
                         void* stream);

/* Boundary velocities written by set_bc (simple.py:181, 186, 192, 196). */
int kc_apply_bc_values(const kc_phys* P, double* u, double* v, void* stream);

/* u = a*u_mid + (1-a)*u on unknown faces (simple.py:232-238; bicgsimp.py:212-225);
 * diff_dev (nullable) receives sqrt(max|du|^2 + max|dv|^2). */
int kc_relax_velocity(const kc_phys* P, const unsigned char* solid, const double* u_mid,
                      const double* v_mid, double* u, double* v, double* diff_dev,
                      void* ws, void* stream);

/* Channel outlet: zero-gradient copy then mass-flow rescale
 * (karman_taichi.py:178-183, 586-601). */
int kc_outlet_conserve(const kc_phys* P, double* u, void* stream);

/* Pressure-correction coefficients and mass source.  Replaces compute_coef_p
 * (simple.py:143-170; bicgsimp.py:124-151).  mass_dev[0] = max|mdiv| over
 * fluid cells, mass_dev[1] = sum mdiv^2.  The optional FP32 copy coef_p32 is
 * written in KC_FORM_LAPLACIAN (component 0 = row sum). */
int kc_assemble_pcorr(const kc_phys* P, const double* u, const double* v,
                      const double* coef_u, const double* coef_v, const unsigned char* solid,
                      double* coef_p, double* b_p, float* coef_p32, float* b_p32,
                      double* mdiv, double* mass_dev, void* ws, void* stream);

/* Velocity and pressure correction.  Replaces correct_velocity and
 * correct_pressure (simple.py:218-230); pcor_max_dev = max|p'|. */
int kc_correct(const kc_phys* P, const double* pcor, const double* coef_u,
               const double* coef_v, const unsigned char* solid, double* u, double* v,
               double* p, double* pcor_max_dev, void* ws, void* stream);

/* mdiv and max|mdiv| of the current field (simple.py:137-141; bicgsimp.py:114-122). */
/* One in-place lexicographic relaxation sweep of A x = b over the box
 * i in [i0, i1), j in [j0, j1) of a [NX][NY] field, i outer and j inner, as
 * jacosimp.py:226-247 runs it in Python scope:
 *   x_mid = (-aW x[i-1,j] - aE x[i+1,j] - aN x[i,j+1] - aS x[i,j-1] + b) / aP
 *   relax: x_mid[i,j] = x_mid, x = (1 - omega) x + omega x_mid;  else x = x_mid
 * where the west and south neighbours already hold this sweep's values.  One
 * block sweeps the anti-diagonals in order: the serial sweep's values exactly
 * (FP64, the reference's operation order).  Coefficient c of (i, j) at
 * coef[c*cs + (i*NY + j)*es]; the box must leave a 1-cell ring. */
int kc_lex_sweep(const double* coef, long long cs, long long es, int NX, int NY, int i0, int i1,
                 int j0, int j1, const double* b, double* x, double* x_mid, double omega, int relax,
                 void* stream);
int kc_mass_residual(const kc_phys* P, const double* u, const double* v,
                     const unsigned char* solid, double* mdiv, double* mass_dev,
                     void* ws, void* stream);

/* ---- karman_taichi.py assembled-matrix path ----------------------------- */
typedef struct {
    int nx, ny;
    double dx, dy, rho, mu, dt, velo_rel, p_rel;
} kc_karman;

/* Rows of fill_Au (karman_taichi.py:162-248), fill_Av (:251-294) and
 * fill_Ap (:297-339) as flat 5-point planes (cs = n, es = 1) + b + Jacobi
 * diagonal M.  u: n = (nx+1)*ny, S = ny; v: n = nx*(ny+1), S = ny+1;
 * p: n = nx*ny, S = ny.  ct is the int32 cell-type field [nx+2][ny+2]. */
int kc_karman_fill_u(const kc_karman* K, const int* ct, const double* u, const double* v,
                     const double* p, const double* u0, double* coef, double* b, double* M,
                     void* stream);
int kc_karman_fill_v(const kc_karman* K, const int* ct, const double* u, const double* v,
                     const double* p, const double* v0, double* coef, double* b, double* M,
                     void* stream);
int kc_karman_fill_p(const kc_karman* K, const int* ct, const double* u, const double* v,
                     const double* coef_u, const double* coef_v, double* coef, double* b,
                     double* M, void* stream);
/* xu_back / xv_back / xp_back (karman_taichi.py:459-478); which = 0, 1, 2. */
int kc_karman_back(const kc_karman* K, int which, const double* x, double* field, void* stream);
/* puv_correction (karman_taichi.py:507-542); pcor_max_dev = max|pcor|. */
int kc_karman_puv_correction(const kc_karman* K, const int* ct, const double* pcor,
                             const double* coef_u, const double* coef_v, double* u,
                             double* v, double* p, double* pcor_max_dev, void* ws,
                             void* stream);
/* correct_conserv (karman_taichi.py:586-614); udiv may be NULL. */
int kc_karman_correct_conserv(const kc_karman* K, double* u, const double* v, double* udiv,
                              void* stream);

/* ---- learned initial guess (U-Net) ---------------------------------------- */
/* No reference counterpart: the learned row of the accelerated path.
 * Activations are NHWC bfloat16 [H][W][C] with C a multiple of 16; 3x3
 * weights are bfloat16 [9][cout][cin] (tap = 3*ky + kx); biases FP32.
 * y = act(conv3x3(x, w) + bias) with zero padding, act 0 = none, 1 = ReLU,
 * cout in {16, 32, 48, 64}; weight (tap, co, ci) at w[tap*wtap + co*cin + ci]
 * (wtap 0: cout*cin) and output (px, co) at y[px*ldy + co] (ldy 0: cout) --
 * a channel group of a wider tensor.  mask (nullable, indexed like y): y = 0
 * where mask <= 0 (the ReLU derivative of the layer below, when the call
 * computes a data gradient with flipped weights).  Tensor cores (BF16
 * operands, FP32 accumulation). */
int kc_unet_conv3x3(const void* x, int H, int W, int cin, const void* w, long long wtap,
                    const float* bias, int cout, int act, const void* mask, void* y, int ldy,
                    void* stream);
/* dw[9][cout][cin] += sum_px dy[px][co] x[px + tap][ci]; db[cout] += sum_px dy (db nullable). */
int kc_unet_conv3x3_wgrad(const void* x, const void* dy, int H, int W, int cin, int cout, float* dw,
                          float* db, void* stream);
/* wt[9][cin][cout] = w[8 - tap][cout][cin] (input channels >= cin_real zeroed): the weights
 * of the data-gradient convolution. */
int kc_unet_flip_weights(const void* w, int cout, int cin, int cin_real, void* wt, void* stream);
/* 2x2 average pooling and its gradient (dx = or += dy / 4). */
int kc_unet_pool2(const void* x, int H, int W, int C, void* y, void* stream);
int kc_unet_pool2_bwd(const void* dy, int H, int W, int C, void* dx, int accumulate, void* stream);
/* y[H][W][cu + cs] = concat(nearest 2x upsampling of u[H/2][W/2][cu], s[H][W][cs]) and its gradient. */
int kc_unet_up2_concat(const void* u, int cu, const void* s, int cs, int H, int W, void* y, void* stream);
int kc_unet_up2_concat_bwd(const void* dy, int cu, int cs, int H, int W, void* du, void* ds,
                           int accumulate_s, void* stream);
/* dy = 0 where y <= 0 (in place). */
int kc_unet_relu_bwd(void* dy, const void* y, long long n, void* stream);
/* 1x1 head C -> 1 (FP32 out, C <= 64) and its gradient (dw, db accumulated). */
int kc_unet_head(const void* x, int C, long long npx, const float* w, const float* b, float* out,
                 void* stream);
int kc_unet_head_bwd(const void* x, int C, long long npx, const float* w, const float* dout, void* dx,
                     float* dw, float* db, void* stream);
/* loss += sum (weight (out - target))^2 * inv_count; dout = 2 weight^2 (out - target) inv_count. */
int kc_unet_mse(const float* out, const float* target, const float* weight, long long npx,
                float inv_count, float* dout, float* loss, void* stream);
/* Adam step (bias-corrected, step >= 1) on FP32 parameters; p_bf16 (nullable) receives a copy. */
int kc_unet_adam(float* p, const float* g, float* m, float* v, long long n, float lr, float b1,
                 float b2, float eps, int step, void* p_bf16, void* stream);
int kc_unet_to_bf16(const float* a, void* b, long long n, void* stream);
/* Network input of the p' system A x = b (b FP64 [NX][NY], coef32 its FP32
 * Laplacian-form planes, SoA): feat[H][W][16] bf16 (H >= NX, W >= NY; zero
 * outside the fluid) with channels b/s_b, fluid, d/mean(d), P1/s_p, where P1
 * is the 1-D solution of the column-summed system (Neumann at i = 0,
 * Dirichlet beyond i = NX-1); fluid (nullable) FP32 [NX][NY]; scales[4] =
 * {s_b, mean d, s_p, fluid count} (device).  ws: kc_unet_features_ws_bytes(NX). */
size_t kc_unet_features_ws_bytes(int NX);
int kc_unet_features(const double* b, const float* coef32, int NX, int NY, int H, int W, void* feat,
                     float* fluid, double* scales, void* ws, size_t ws_bytes, void* stream);
/* x0 = s_p * bilinear 2x upsampling of the half-resolution prediction out[Hh][Wh] on fluid cells
 * (0 elsewhere), FP64 [NX][NY]. */
int kc_unet_guess_up2(const float* out, int Hh, int Wh, const float* coef32, int NX, int NY,
                      const double* scales, double* x0, void* stream);
/* Half-resolution training target: 2x2 fluid average of p / s_p and the fluid share as weight. */
int kc_unet_target_down2(const double* p, const float* coef32, int NX, int NY, const double* scales,
                         int Hh, int Wh, float* target, float* weight, void* stream);


/* ---- native SIMPLE step and the batched executor --------------------------- */
/* One channel instance (caller-owned device buffers, shapes as kc_assemble_*).
 * precision KC_F64: the plain method (every solve FP64 BiCGSTAB, cold start,
 * rel. tol eps, cap n); KC_F32: the accelerated path (momentum:
 * KC_MOMENTUM_BICGSTAB, FP32 BiCGSTAB in FP64 refinement, inner tol
 * eps_inner; KC_MOMENTUM_RBGS_REFINED (the Python ChannelSolver's default),
 * FP32 red-black Gauss-Seidel in FP64 refinement (kc_rbgs_refined, 12
 * sweeps per refinement pass, at most 200 sweeps); or
 * KC_MOMENTUM_RBGS, FP64 red-black Gauss-Seidel (kc_rbgs, at most 200
 * sweeps); the Gauss-Seidel variants hand over to the refined BiCGSTAB if
 * they miss eps; all from the previous outer iteration's u*, v* to
 * ||b - A x|| / ||b|| < eps; p': multigrid CG in FP64 refinement
 * on coef_p32 in Laplacian form, inner tol eps_inner_p, with the plain FP64
 * BiCGSTAB as fallback).  Workspaces: ws_u / ws_v of kc_bicgstab_ws_bytes
 * (F64) or the larger of kc_refined_ws_bytes and kc_rbgs_ws_bytes (F32)
 * bytes; ws_p of kc_bicgstab_ws_bytes (F64) or the larger of that and
 * kc_pbicgstab_ws_bytes (F32); mg_ws of kc_mg_ws_bytes (F32 only); rws of
 * kc_reduce_ws_bytes. */
#define KC_MOMENTUM_BICGSTAB 0
#define KC_MOMENTUM_RBGS 1
#define KC_MOMENTUM_RBGS_REFINED 2
typedef struct {
    kc_phys phys;                       /* mode must be KC_MODE_CHANNEL */
    int precision, max_outer, use_graph;
    int persistent;                     /* 1: BiCGSTAB solves as one cooperative launch, 0: graph chunks */
    int momentum;                       /* KC_F32 momentum solver: KC_MOMENTUM_* */
    int check_every_p;                  /* KC_F32 p' solve: CG iterations per graph chunk between checks (0: 4) */
    double mass_tol, eps, eps_inner, eps_inner_p;
    double *u, *v, *p, *u0, *v0, *pcor, *u_mid, *v_mid;
    const unsigned char* solid;         /* [nx+2][ny+2], 1 = blocked cell */
    double *coef_u, *b_u, *coef_v, *b_v, *coef_p, *b_p;
    float *coef_u32, *b_u32, *coef_v32, *b_v32, *coef_p32, *b_p32;
    double *mass, *pmax;                /* device scalars: [2] and [1] */
    void* rws;
    void *ws_u, *ws_v, *ws_p;
    size_t ws_u_bytes, ws_v_bytes, ws_p_bytes;
    void* mg_ws;
    size_t mg_ws_bytes;
    kc_mg_opts mg_opts;
    /* KC_F32 only, nullable: with a network, every p' solve is kc_pcg_flexible
     * (the network's prediction as the first preconditioner application, then
     * multigrid CG passes), in ws_flex of kc_pcg_flexible_ws_bytes(n_p) */
    const kc_unet_net* learned;
    void* ws_flex;
    size_t ws_flex_bytes;
    /* KC_F32 without a network: recycle > 0 starts every p' solve from the
     * Galerkin projection onto the last `recycle` (<= KC_RECYCLE_MAX) p'
     * solutions (kc_recycle_guess).  ws_recycle: kc_channel_recycle_ws_bytes
     * (the ring of solutions, the guess, the projection's scratch); rstate:
     * the caller's ring bookkeeping, {0, 0} for an empty ring (reset it when
     * the fields are reset). */
    int recycle;
    int pad2_;
    void* ws_recycle;
    size_t ws_recycle_bytes;
    kc_recycle_state* rstate;
} kc_channel;
size_t kc_channel_recycle_ws_bytes(long long n_p, int recycle);

typedef struct {
    int outer, fallbacks, status, pad_;   /* status: KC_OK; KC_MAXITER if a solve missed eps;
                                             KC_NONFINITE if a solve or the mass residual met a
                                             NaN/Inf, which also ends the step's outer loop */
    long long it_u, it_v, it_p;
    double mass;                          /* max|mdiv| of the last outer iteration */
    int learned, learned_rejected;        /* p' solves that applied / rejected the network */
} kc_channel_stats;

/* One time step: SIMPLE outer iterations (karman_taichi.py:633-659, simple.py:270-281)
 * until max|mdiv| <= mass_tol or max_outer, then u0 = u, v0 = v (karman_taichi.py:617-622).
 * No reference counterpart as a single call: the reference drives these stages from Python. */
int kc_channel_step(const kc_channel* ch, kc_channel_stats* stats, void* stream);
/* steps time steps of n independent instances, instance k on streams[k], driven by
 * `workers` native threads (instance k by thread k mod workers); stats[k] (nullable) gets
 * instance k's last step.  The first error stops all workers and is returned. */
int kc_channel_batch_step(const kc_channel* const* chs, int n, void* const* streams, int workers,
                          int steps, kc_channel_stats* stats);

/* n instances advanced by `steps` time steps in ONE kernel launch, block k
 * running instance k's whole time steps (the mixed path: momentum by FP32
 * red-black Gauss-Seidel in FP64 refinement, p' by multigrid CG in FP64
 * refinement from p' = 0, the instance's mg_opts omega / alpha / nu_coarse;
 * outer loop to mass_tol or max_outer, then u0 = u, v0 = v).  Every instance
 * must be KC_F32 in KC_MODE_CHANNEL; of its buffers only the fields, the
 * FP64 systems and their FP32 copies are used (ws_* and mg_ws are not).  An
 * instance computes bit for bit what it computes in a batch of one.  ws:
 * kc_channel_batch_fused_ws_bytes(chs, n), 256-byte aligned.  last / total
 * (host arrays of n, nullable): each instance's last step, and the sums over
 * the steps (mass: the largest last-outer mass residual).  A momentum solve
 * whose Gauss-Seidel sweeps miss eps, and a p' solve whose multigrid CG
 * stalls, continue with FP32 BiCGSTAB in FP64 refinement (counted in
 * `fallbacks`).  Blocks until the launch has finished.  The reference's
 * drivers have no batched counterpart. */
size_t kc_channel_batch_fused_ws_bytes(const kc_channel* const* chs, int n);
int kc_channel_batch_fused(const kc_channel* const* chs, int n, int steps, void* ws, size_t ws_bytes,
                           kc_channel_stats* last, kc_channel_stats* total, void* stream);

/* ---- output post-processing ----------------------------------------------- */
/* post_process_field (karman_taichi.py:545-583) on the padded staggered fields
 * (u [nx+3][ny+2], v [nx+2][ny+3], p and pcor [nx+2][ny+2]):
 *   u_post[i][j] = (u[i][j] + u[i+1][j]) / 2, v_post[i][j] = (v[i][j] + v[i][j+1]) / 2,
 *   udiv[i][j] = (u[i][j] - u[i+1][j]) dy + (v[i][j+1] - v[i][j]) dx for i in [1,nx], j in [1,ny]
 *   (other entries of udiv untouched);
 *   minmax[2f], minmax[2f+1] = min, max of field f in (u_post, v_post, p, pcor, udiv), starting
 *   from max 0 and min 1e9 as scale_field does (karman_taichi.py:573-583);
 *   disp (nullable, FP32 [5][3(nx+2)][3(ny+2)]): the display canvases, field f at cell (I/3, J/3)
 *   scaled by (x - min) / (max - min + 1e-9).
 * minmax is device memory (10 doubles); ws: kc_post_process_ws_bytes() bytes, zeroed before the
 * first call. */
size_t kc_post_process_ws_bytes(void);
int kc_post_process(int nx, int ny, double dx, double dy, const double* u, const double* v,
                    const double* p, const double* pcor, double* u_post, double* v_post,
                    double* udiv, double* minmax, float* disp, void* ws, size_t ws_bytes,
                    void* stream);

/* ---- utilities ------------------------------------------------------------ */
/* dst = src (device to device), e.g. time_forward (karman_taichi.py:617-622). */
int kc_copy(void* dst, const void* src, size_t bytes, void* stream);
/* dst[k] = (float)src[k], k < n (device FP64 -> device FP32), rounded to nearest, ties to even:
 * the conversion every FP32 copy of an FP64 system in this library uses (the mixed-precision
 * coefficient planes, right-hand sides and refinement residuals). */
int kc_to_f32(const double* src, float* dst, long long n, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* KARMAN_GB300_H */
