/*
 * kc_cpu.c -- TEST INFRASTRUCTURE / TIMED CPU BASELINE ONLY.
 *
 * A C17 + OpenMP FP64 restatement of the channel SIMPLE plain path, the same
 * algorithm as oracle/np_oracle.py's ChannelOracle (which the tests pin
 * against the reference's known-answer tests):
 *   momentum coefficients   simple.py:77-110 with set_bc-style folding (simple.py:172-216)
 *   outlet                  karman_taichi.py:178-183 (zero gradient), 586-601 (mass rescale)
 *   pressure correction     simple.py:143-170, correction simple.py:218-230
 *   BiCGSTAB                bicgsolver.py:88-135 (M = I, cold start, rel tol)
 * Only bench.py's CPU-baseline / reference legs and the tests load it; the
 * product never does.  Loops are OpenMP-parallel; reductions use OpenMP's
 * (unordered) reduction clauses.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

typedef struct {
    int nx, ny;
    double dx, dy, rho, mu, dt, U, alpha_m, alpha_u, alpha_p, eps, mass_tol;
    int max_outer;
} cpu_params;

#define IDU(i, j) ((long)(i) * (ny + 2) + (j))
#define IDV(i, j) ((long)(i) * (ny + 3) + (j))
#define IDP(i, j) ((long)(i) * (ny + 2) + (j))

static int blk_u(const unsigned char* s, int ny, int i, int j) { return s[IDP(i - 1, j)] || s[IDP(i, j)]; }
static int blk_v(const unsigned char* s, int ny, int i, int j) { return s[IDP(i, j - 1)] || s[IDP(i, j)]; }
static int unk_u(const unsigned char* s, int nx, int ny, int i, int j) {
    return i >= 2 && i <= nx && j >= 1 && j <= ny && !blk_u(s, ny, i, j);
}
static int unk_v(const unsigned char* s, int nx, int ny, int i, int j) {
    return i >= 1 && i <= nx && j >= 2 && j <= ny && !blk_v(s, ny, i, j);
}

/* flat 5-point stencil y = A x, reads outside [0, n) are 0 */
static void spmv(const double* c, long n, long S, const double* x, double* y) {
#pragma omp parallel for schedule(static)
    for (long k = 0; k < n; ++k) {
        double v = c[k] * x[k];
        if (k >= S) v += c[n + k] * x[k - S];
        if (k + S < n) v += c[2 * n + k] * x[k + S];
        if (k + 1 < n) v += c[3 * n + k] * x[k + 1];
        if (k >= 1) v += c[4 * n + k] * x[k - 1];
        y[k] = v;
    }
}

static double dot(const double* a, const double* b, long n) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (long k = 0; k < n; ++k) s += a[k] * b[k];
    return s;
}

/* BiCGSTAB (bicgsolver.py:88-135); returns iterations, x overwritten */
static long bicgstab(const double* c, long n, long S, const double* b, double* x, double eps, long max_iter,
                     double* work) {
    double *r = work, *rt = work + n, *p = work + 2 * n, *v = work + 3 * n, *s = work + 4 * n, *t = work + 5 * n;
#pragma omp parallel for schedule(static)
    for (long k = 0; k < n; ++k) {
        r[k] = b[k];
        rt[k] = b[k];
        x[k] = 0.0;
        p[k] = 0.0;
        v[k] = 0.0;
    }
    const double r0 = dot(r, r, n);
    if (r0 == 0.0) return 0;
    double rho_1 = 1.0, alpha = 1.0, omega = 1.0;
    long it = 0;
    for (long i = 0; i < max_iter; ++i) {
        const double rho = dot(r, rt, n);
        if (rho == 0.0) break;
        if (i == 0) {
            memcpy(p, r, n * sizeof(double));
        } else {
            const double beta = (rho / rho_1) * (alpha / omega);
#pragma omp parallel for schedule(static)
            for (long k = 0; k < n; ++k) p[k] = r[k] + beta * (p[k] - omega * v[k]);
        }
        spmv(c, n, S, p, v);
        alpha = rho / dot(rt, v, n);
#pragma omp parallel for schedule(static)
        for (long k = 0; k < n; ++k) s[k] = r[k] - alpha * v[k];
        spmv(c, n, S, s, t);
        omega = dot(t, s, n) / dot(t, t, n);
        double rr = 0.0;
#pragma omp parallel for reduction(+ : rr) schedule(static)
        for (long k = 0; k < n; ++k) {
            x[k] += alpha * p[k] + omega * s[k];
            r[k] = s[k] - omega * t[k];
            rr += r[k] * r[k];
        }
        it = i + 1;
        if (sqrt(rr / r0) < eps || !isfinite(rr)) break;
        rho_1 = rho;
    }
    return it;
}

static void assemble_momentum(const cpu_params* P, const unsigned char* sol, const double* u, const double* v,
                              const double* p, const double* u0, const double* v0, double* cu, double* bu,
                              double* cv, double* bv) {
    const int nx = P->nx, ny = P->ny;
    const double dx = P->dx, dy = P->dy, rho = P->rho, mu = P->mu, dt = P->dt;
    const long nu = (long)(nx + 3) * (ny + 2), nv = (long)(nx + 2) * (ny + 3);
    memset(cu, 0, 5 * nu * sizeof(double));
    memset(bu, 0, nu * sizeof(double));
    memset(cv, 0, 5 * nv * sizeof(double));
    memset(bv, 0, nv * sizeof(double));
#pragma omp parallel for schedule(static)
    for (int i = 2; i <= nx; ++i) {
        for (int j = 1; j <= ny; ++j) {
            const long k = IDU(i, j);
            if (blk_u(sol, ny, i, j)) {
                cu[k] = 1.0;
                continue;
            }
            const double ui = u[IDU(i, j)], uw = u[IDU(i - 1, j)], ue = u[IDU(i + 1, j)];
            const double vnw = v[IDV(i - 1, j + 1)], vne = v[IDV(i, j + 1)], vsw = v[IDV(i - 1, j)], vse = v[IDV(i, j)];
            double aW = -(mu * dy / dx + 0.5 * rho * 0.5 * (ui + uw) * dy);
            double aE = -(mu * dy / dx - 0.5 * rho * 0.5 * (ui + ue) * dy);
            double aN = -(mu * dx / dy - 0.5 * rho * 0.5 * (vnw + vne) * dx);
            double aS = -(mu * dx / dy + 0.5 * rho * 0.5 * (vsw + vse) * dx);
            double aP = -(aW + aE + aN + aS) + rho * 0.5 * (ui + ue) * dy - rho * 0.5 * (ui + uw) * dy +
                        rho * 0.5 * (vnw + vne) * dx - rho * 0.5 * (vsw + vse) * dx + rho * dx * dy / dt;
            double b = (p[IDP(i - 1, j)] - p[IDP(i, j)]) * dy + rho * dx * dy / dt * u0[k];
            const double wall = 2 * mu * dx / dy;
            if (i == 2) { b += -aW * P->U; aW = 0.0; }
            else if (blk_u(sol, ny, i - 1, j)) aW = 0.0;
            if (i == nx) { aP = aP + aE; aE = 0.0; }
            else if (blk_u(sol, ny, i + 1, j)) aE = 0.0;
            if (j == 1 || blk_u(sol, ny, i, j - 1)) { aP = aP + (aS + wall); aS = 0.0; }
            if (j == ny || blk_u(sol, ny, i, j + 1)) { aP = aP + (aN + wall); aN = 0.0; }
            cu[k] = aP; cu[nu + k] = aW; cu[2 * nu + k] = aE; cu[3 * nu + k] = aN; cu[4 * nu + k] = aS;
            bu[k] = b;
        }
    }
#pragma omp parallel for schedule(static)
    for (int i = 1; i <= nx; ++i) {
        for (int j = 2; j <= ny; ++j) {
            const long k = IDV(i, j);
            if (blk_v(sol, ny, i, j)) {
                cv[k] = 1.0;
                continue;
            }
            const double uc = u[IDU(i, j)], us = u[IDU(i, j - 1)], uec = u[IDU(i + 1, j)], ues = u[IDU(i + 1, j - 1)];
            const double vc = v[IDV(i, j)], vn = v[IDV(i, j + 1)], vs = v[IDV(i, j - 1)];
            double aW = -(mu * dy / dx + 0.5 * rho * 0.5 * (uc + us) * dy);
            double aE = -(mu * dy / dx - 0.5 * rho * 0.5 * (ues + uec) * dy);
            double aN = -(mu * dx / dy - 0.5 * rho * 0.5 * (vn + vc) * dx);
            double aS = -(mu * dx / dy + 0.5 * rho * 0.5 * (vs + vc) * dx);
            double aP = -(aW + aE + aN + aS) + rho * 0.5 * (ues + uec) * dy - rho * 0.5 * (uc + us) * dy +
                        rho * 0.5 * (vn + vc) * dx - rho * 0.5 * (vs + vc) * dx + rho * dx * dy / dt;
            double b = (p[IDP(i, j - 1)] - p[IDP(i, j)]) * dx + rho * dx * dy / dt * v0[k];
            const double wall = 2 * mu * dy / dx;
            if (j == 2 || blk_v(sol, ny, i, j - 1)) aS = 0.0;
            if (j == ny || blk_v(sol, ny, i, j + 1)) aN = 0.0;
            if (i == 1 || blk_v(sol, ny, i - 1, j)) { aP = aP + (aW + wall); aW = 0.0; }
            if (i == nx) { aP = aP + aE; aE = 0.0; }
            else if (blk_v(sol, ny, i + 1, j)) { aP = aP + (aE + wall); aE = 0.0; }
            cv[k] = aP; cv[nv + k] = aW; cv[2 * nv + k] = aE; cv[3 * nv + k] = aN; cv[4 * nv + k] = aS;
            bv[k] = b;
        }
    }
}

static void relax_outlet(const cpu_params* P, const unsigned char* sol, const double* um, const double* vm, double* u,
                         double* v) {
    const int nx = P->nx, ny = P->ny;
    const double a = P->alpha_m;
#pragma omp parallel for schedule(static)
    for (int i = 2; i <= nx; ++i)
        for (int j = 1; j <= ny; ++j)
            if (unk_u(sol, nx, ny, i, j)) u[IDU(i, j)] = a * um[IDU(i, j)] + (1 - a) * u[IDU(i, j)];
#pragma omp parallel for schedule(static)
    for (int i = 1; i <= nx; ++i)
        for (int j = 2; j <= ny; ++j)
            if (unk_v(sol, nx, ny, i, j)) v[IDV(i, j)] = a * vm[IDV(i, j)] + (1 - a) * v[IDV(i, j)];
    double min = 0.0, mout = 0.0;
    for (int j = 1; j <= ny; ++j) {
        u[IDU(nx + 1, j)] = u[IDU(nx, j)];
        min += u[IDU(1, j)];
        mout += u[IDU(nx + 1, j)];
    }
    const double coef = min / mout;
    for (int j = 1; j <= ny; ++j) u[IDU(nx + 1, j)] = coef * u[IDU(nx + 1, j)];
}

static double assemble_p(const cpu_params* P, const unsigned char* sol, const double* u, const double* v,
                         const double* cu, const double* cv, double* cp, double* bp) {
    const int nx = P->nx, ny = P->ny;
    const double dx = P->dx, dy = P->dy, rho = P->rho;
    const long np = (long)(nx + 2) * (ny + 2);
    memset(cp, 0, 5 * np * sizeof(double));
    memset(bp, 0, np * sizeof(double));
    double mx = 0.0;
#pragma omp parallel for reduction(max : mx) schedule(static)
    for (int i = 1; i <= nx; ++i) {
        for (int j = 1; j <= ny; ++j) {
            const long k = IDP(i, j);
            if (sol[k]) {
                cp[k] = 1.0;
                continue;
            }
            const double md = rho * (u[IDU(i, j)] - u[IDU(i + 1, j)]) * dy + rho * (v[IDV(i, j)] - v[IDV(i, j + 1)]) * dx;
            double aW = 0.0, aE = 0.0, aN = 0.0, aS = 0.0;
            if (unk_u(sol, nx, ny, i, j)) aW = -rho * dy * dy / cu[IDU(i, j)];
            if (unk_u(sol, nx, ny, i + 1, j)) aE = -rho * dy * dy / cu[IDU(i + 1, j)];
            if (i == nx && unk_u(sol, nx, ny, nx, j)) aE = -rho * dy * dy / cu[IDU(nx, j)];
            if (unk_v(sol, nx, ny, i, j + 1)) aN = -rho * dx * dx / cv[IDV(i, j + 1)];
            if (unk_v(sol, nx, ny, i, j)) aS = -rho * dx * dx / cv[IDV(i, j)];
            cp[k] = -(aW + aE + aN + aS);
            cp[np + k] = aW; cp[2 * np + k] = aE; cp[3 * np + k] = aN; cp[4 * np + k] = aS;
            bp[k] = md;
            if (fabs(md) > mx) mx = fabs(md);
        }
    }
    return mx;
}

static void correct(const cpu_params* P, const unsigned char* sol, const double* pc, const double* cu,
                    const double* cv, double* u, double* v, double* p) {
    const int nx = P->nx, ny = P->ny;
    const double dx = P->dx, dy = P->dy, au = P->alpha_u, ap = P->alpha_p;
#pragma omp parallel for schedule(static)
    for (int i = 2; i <= nx + 1; ++i)
        for (int j = 1; j <= ny; ++j) {
            if (unk_u(sol, nx, ny, i, j))
                u[IDU(i, j)] = u[IDU(i, j)] + au * (pc[IDP(i - 1, j)] - pc[IDP(i, j)]) * dy / cu[IDU(i, j)];
            else if (i == nx + 1 && unk_u(sol, nx, ny, nx, j))
                u[IDU(i, j)] = u[IDU(i, j)] + au * (pc[IDP(nx, j)] - pc[IDP(nx + 1, j)]) * dy / cu[IDU(nx, j)];
        }
#pragma omp parallel for schedule(static)
    for (int i = 1; i <= nx; ++i)
        for (int j = 2; j <= ny; ++j)
            if (unk_v(sol, nx, ny, i, j))
                v[IDV(i, j)] = v[IDV(i, j)] + au * (pc[IDP(i, j - 1)] - pc[IDP(i, j)]) * dx / cv[IDV(i, j)];
#pragma omp parallel for schedule(static)
    for (int i = 1; i <= nx; ++i)
        for (int j = 1; j <= ny; ++j)
            if (!sol[IDP(i, j)]) p[IDP(i, j)] = p[IDP(i, j)] + ap * pc[IDP(i, j)];
}

int kc_cpu_threads(void) { return omp_get_max_threads(); }

/* sets the OpenMP thread count of later calls (n < 1: leave it) */
void kc_cpu_set_threads(int n) {
    if (n >= 1) omp_set_num_threads(n);
}

/*
 * Runs SIMPLE outer iterations of the channel case (time steps of up to
 * max_outer iterations, stopping a step when the predicted field's max|mdiv|
 * <= mass_tol), in place on u, v, p, u0, v0.  Stops after n_steps time steps
 * or after max_total_outer outer iterations, whichever comes first; every
 * BiCGSTAB solve is capped at max_solver_iter iterations (bounded samples).
 * stats[0] = outer iterations run, [1] = time steps completed, [2] = BiCGSTAB
 * iterations (all solves), [3] = last mass residual, [4] = wall seconds.
 */
int kc_cpu_channel_run(const cpu_params* P, const unsigned char* sol, double* u, double* v, double* p, double* u0,
                       double* v0, int n_steps, long max_total_outer, long max_solver_iter, double* stats) {
    const int nx = P->nx, ny = P->ny;
    const long nu = (long)(nx + 3) * (ny + 2), nv = (long)(nx + 2) * (ny + 3), np = (long)(nx + 2) * (ny + 2);
    long nmax = nu > nv ? nu : nv;
    double* cu = malloc(5 * nu * sizeof(double));
    double* bu = malloc(nu * sizeof(double));
    double* cv = malloc(5 * nv * sizeof(double));
    double* bv = malloc(nv * sizeof(double));
    double* cp = malloc(5 * np * sizeof(double));
    double* bp = malloc(np * sizeof(double));
    double* um = malloc(nu * sizeof(double));
    double* vm = malloc(nv * sizeof(double));
    double* pc = malloc(np * sizeof(double));
    double* work = malloc(6 * nmax * sizeof(double));
    if (!cu || !bu || !cv || !bv || !cp || !bp || !um || !vm || !pc || !work) return -1;
    double t0 = omp_get_wtime();
    long outer = 0, its = 0;
    int steps = 0;
    double mass = 0.0;
    for (int st = 0; st < n_steps && outer < max_total_outer; ++st) {
        int done_step = 0;
        for (int k = 0; k < P->max_outer && outer < max_total_outer; ++k) {
            assemble_momentum(P, sol, u, v, p, u0, v0, cu, bu, cv, bv);
            its += bicgstab(cu, nu, ny + 2, bu, um, P->eps, nu < max_solver_iter ? nu : max_solver_iter, work);
            its += bicgstab(cv, nv, ny + 3, bv, vm, P->eps, nv < max_solver_iter ? nv : max_solver_iter, work);
            relax_outlet(P, sol, um, vm, u, v);
            mass = assemble_p(P, sol, u, v, cu, cv, cp, bp);
            its += bicgstab(cp, np, ny + 2, bp, pc, P->eps, np < max_solver_iter ? np : max_solver_iter, work);
            correct(P, sol, pc, cu, cv, u, v, p);
            ++outer;
            if (mass <= P->mass_tol) {
                done_step = 1;
                break;
            }
            if (k == P->max_outer - 1) done_step = 1;
        }
        if (!done_step) break;
        memcpy(u0, u, nu * sizeof(double));
        memcpy(v0, v, nv * sizeof(double));
        ++steps;
    }
    stats[0] = (double)outer;
    stats[1] = (double)steps;
    stats[2] = (double)its;
    stats[3] = mass;
    stats[4] = omp_get_wtime() - t0;
    free(cu); free(bu); free(cv); free(bv); free(cp); free(bp); free(um); free(vm); free(pc); free(work);
    return 0;
}
