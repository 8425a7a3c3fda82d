"""CPU oracle for the karman_taichi SIMPLE hot path -- TEST INFRASTRUCTURE ONLY.

A NumPy FP64 restatement of the reference algorithms. Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import this
module, and only as the checker; the product (``karman_taichi_gb300``) never
imports anything under ``oracle/``.

Parity status
-------------
* Linear solvers (``bicgstab``, ``cg``, ``spmv``) are pinned against the
  reference's own known-answer tests, restated with seeded inputs in
  ``tests/test_oracle_kat.py``: debug/ti_bicg_test.py:21-98 (random
  diagonally dominant 5-diagonal matrix vs ``np.linalg.solve``),
  benchmark/cg_to_sparse/validation.py:7-45 and test_cg_sparse.py:10-41
  (Laplacian + offset vs a direct sparse solve / SciPy BiCGSTAB).
* SIMPLE fields (u, v, p after N steps): **parity unpinned**. Taichi 0.9.0 is
  not importable here and the reference commits no field fixtures, so this
  restatement is the only field oracle.

Conventions shared with the CUDA library
----------------------------------------
Every linear system is a 5-point stencil on a *flat* index ``k in [0, n)``
with far stride ``S``: ``y[k] = c0 x[k] + cW x[k-S] + cE x[k+S] + cN x[k+1]
+ cS x[k-1]``; reads outside ``[0, n)`` return 0 (Taichi reads of unwritten
sparse entries return 0: debug/ti_sparse_test.py:38-39). Coefficients are
planes ``coef[0..4] = aP, aW, aE, aN, aS`` -- the component order of the
reference's ``coef[i,j,0..4]`` (simple.py:42-47). For a padded 2-D field
``[NX, NY]`` the flat stride is ``S = NY`` and ``(i, j)`` is ``k = i*NY + j``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# Solver status codes (mirrors include/karman_gb300.h)
OK, MAXITER, BREAKDOWN_RHO, BREAKDOWN_OMEGA, NONFINITE, STALL = 0, 1, 2, 3, 4, 5


# ----------------------------------------------------------------------------
# Stencil operator and solvers
# ----------------------------------------------------------------------------
def spmv(coef, x, S, order="simple"):
    """y = A x for a flat 5-point stencil (bicgsolver.py:65-76, cgsolver.py:56-66).

    ``order='simple'`` adds the terms as bicgsolver.py:75-76 writes them
    (P, W, E, N, S); ``order='karman'`` follows the gather order of
    karman_taichi.py:403-407 (k-S, k-1, k, k+1, k+S).
    """
    coef = coef.reshape(5, -1)
    x = x.reshape(-1)
    n = x.size
    xW = np.zeros(n); xE = np.zeros(n); xN = np.zeros(n); xS = np.zeros(n)
    if S < n:
        xW[S:] = x[:n - S]
        xE[:n - S] = x[S:]
    xS[1:] = x[:-1]
    xN[:-1] = x[1:]
    if order == "simple":
        y = coef[0] * x + coef[1] * xW + coef[2] * xE + coef[3] * xN + coef[4] * xS
    else:
        y = 0.0 + coef[1] * xW
        y = y + coef[4] * xS
        y = y + coef[0] * x
        y = y + coef[3] * xN
        y = y + coef[2] * xE
    return y


def dot(p, q):
    """CGSolver.reduce (cgsolver.py:49-54): FP64 sum of p*q over the whole field."""
    return float(np.dot(p.reshape(-1), q.reshape(-1)))


@dataclass
class SolveResult:
    x: np.ndarray
    status: int
    iters: int
    rel_res: float
    history: list = field(default_factory=list)


def bicgstab(coef, b, S, eps=1e-8, max_iter=None, x0=None, M=None,
             omega_break=False, order="simple", rel_to="r0"):
    """BiCGSTAB restated from bicgsolver.py:88-135 and karman_taichi.py:342-456.

    * ``x0=None``: cold start, x = 0, r = b (bicgsolver.py:21-36).
    * ``x0`` array: warm start, r = b - A x0 (karman_taichi.py:362-371).
    * ``M``: right-Jacobi diagonal, p_hat = (1/M) p, s_hat = (1/M) s
      (karman_taichi.py:398-399, 418-419); None means M = I (bicgsolver.py:52).
    * stop when sqrt(rTr / r0Tr) < eps (bicgsolver.py:130; karman :446), on
      rho == 0 (bicgsolver.py:96-98) and, for karman, on omega == 0 (:451-454).
    * ``rel_to='b'`` measures the residual against ||b|| instead of ||r0||.
    """
    b = b.reshape(-1).astype(np.float64)
    n = b.size
    if max_iter is None:
        max_iter = n
    if x0 is None:
        x = np.zeros(n)
        r = b.copy()
    else:
        x = np.array(x0, dtype=np.float64).reshape(-1).copy()
        r = b - spmv(coef, x, S, order)
    rt = r.copy()
    r0 = dot(r, r)
    den = dot(b, b) if rel_to == "b" else r0
    invM = None if M is None else 1.0 / M.reshape(-1)
    rho_1 = alpha = omega = 1.0
    p = np.zeros(n); v = np.zeros(n)
    status, it, rel = MAXITER, 0, (0.0 if den == 0 else math.sqrt(r0 / den))
    if r0 == 0.0:
        return SolveResult(x, OK, 0, 0.0)
    if rel_to == "b" and rel < eps:
        return SolveResult(x, OK, 0, rel)
    with np.errstate(all="ignore"):
        for i in range(max_iter):
            rho = dot(r, rt)
            if rho == 0.0:
                status = BREAKDOWN_RHO
                break
            if i == 0:
                p = r.copy()
            else:
                beta = (rho / rho_1) * (alpha / omega)
                p = r + beta * (p - omega * v)
            ph = p if invM is None else invM * p
            v = spmv(coef, ph, S, order)
            alpha = rho / dot(rt, v)
            s = r - alpha * v
            sh = s if invM is None else invM * s
            t = spmv(coef, sh, S, order)
            omega = dot(t, s) / dot(t, t)
            x = x + (alpha * ph + omega * sh)
            r = s - omega * t
            rTr = dot(r, r)
            it = i + 1
            rel = math.sqrt(rTr / den) if den > 0 else 0.0
            if rel < eps:
                status = OK
                break
            if not np.isfinite(rTr):
                status = NONFINITE
                break
            if omega_break and omega == 0.0:
                status = BREAKDOWN_OMEGA
                break
            rho_1 = rho
    return SolveResult(x, status, it, rel)


def cg(coef, b, S, eps=1e-8, max_iter=None):
    """Conjugate gradients restated from cgsolver.py:83-114 (cold start, x = 0;
    stop when sqrt(new_rTr) < sqrt(r0Tr) * eps, cgsolver.py:102)."""
    b = b.reshape(-1).astype(np.float64)
    n = b.size
    if max_iter is None:
        max_iter = n
    x = np.zeros(n)
    r = b.copy()
    r0 = dot(r, r)
    hist = [math.sqrt(r0)]
    if r0 == 0.0:
        return SolveResult(x, OK, 0, 0.0, hist)
    old = r0
    p = r.copy()
    status, it, rel = MAXITER, 0, 1.0
    with np.errstate(all="ignore"):
        for i in range(max_iter):
            Ap = spmv(coef, p, S)
            alpha = old / dot(p, Ap)
            x = x + alpha * p
            r = r - alpha * Ap
            new = dot(r, r)
            it = i + 1
            rel = math.sqrt(new) / math.sqrt(r0)
            if math.sqrt(new) < math.sqrt(r0) * eps:
                status = OK
                break
            if not np.isfinite(new):
                status = NONFINITE
                break
            beta = new / old
            p = r + beta * p
            old = new
            hist.append(math.sqrt(new))
    return SolveResult(x, status, it, rel, hist)


def bicgstab_refined(coef, b, S, eps=1e-8, eps_inner=1e-4, max_refine=20,
                     max_iter=None):
    """Mixed-precision iterative refinement: FP64 residual, FP32 BiCGSTAB
    correction with FP64 inner products (emulated by rounding the vectors and
    coefficients to float32 after every update)."""
    b = b.reshape(-1).astype(np.float64)
    n = b.size
    max_iter = max_iter or n
    c32 = coef.reshape(5, -1).astype(np.float32).astype(np.float64)
    x = np.zeros(n)
    bn = math.sqrt(dot(b, b))
    total = 0
    if bn == 0:
        return SolveResult(x, OK, 0, 0.0)
    for _ in range(max_refine):
        r = b - spmv(coef, x, S)
        rel = math.sqrt(dot(r, r)) / bn
        if rel < eps:
            return SolveResult(x, OK, total, rel)
        r32 = r.astype(np.float32).astype(np.float64)
        res = _bicgstab_f32(c32, r32, S, eps_inner, max_iter)
        total += res.iters
        x = x + res.x
    r = b - spmv(coef, x, S)
    rel = math.sqrt(dot(r, r)) / bn
    return SolveResult(x, OK if rel < eps else MAXITER, total, rel)


def _f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def _bicgstab_f32(c32, b, S, eps, max_iter):
    n = b.size
    x = np.zeros(n); r = b.copy(); rt = r.copy()
    r0 = dot(r, r)
    rho_1 = alpha = omega = 1.0
    p = np.zeros(n); v = np.zeros(n)
    it = 0
    for i in range(max_iter):
        rho = dot(r, rt)
        if rho == 0:
            break
        if i == 0:
            p = r.copy()
        else:
            beta = (rho / rho_1) * (alpha / omega)
            p = _f32(r + _f32(beta) * (p - _f32(omega) * v))
        v = _f32(spmv(c32, p, S))
        alpha = rho / dot(rt, v)
        s = _f32(r - _f32(alpha) * v)
        t = _f32(spmv(c32, s, S))
        omega = dot(t, s) / dot(t, t)
        x = _f32(x + _f32(alpha) * p + _f32(omega) * s)
        r = _f32(s - _f32(omega) * t)
        it = i + 1
        if math.sqrt(dot(r, r) / r0) < eps:
            break
        rho_1 = rho
    return SolveResult(x, OK, it, 0.0)


def to_laplacian32(coef):
    """FP32 copy of a standard-form stencil in Laplacian form: component 0 is
    the row sum aP + (((aW + aE) + aN) + aS), formed in FP64 and rounded once
    (the FP32 pressure-correction output of kc_assemble_pcorr)."""
    c = np.asarray(coef, dtype=np.float64).reshape(5, -1)
    out = c.astype(np.float32)
    out[0] = (c[0] + (((c[1] + c[2]) + c[3]) + c[4])).astype(np.float32)
    return out.reshape(np.shape(coef))


def to_csr(coef, S):
    """Assemble the flat 5-point stencil as a scipy CSR matrix (test helper)."""
    import scipy.sparse as sp
    coef = coef.reshape(5, -1)
    n = coef.shape[1]
    rows, cols, vals = [], [], []
    for c, off in ((0, 0), (1, -S), (2, S), (3, 1), (4, -1)):
        k = np.arange(n)
        m = (k + off >= 0) & (k + off < n) & (coef[c] != 0)
        rows.append(k[m]); cols.append(k[m] + off); vals.append(coef[c][m])
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))


# ----------------------------------------------------------------------------
# simple.py: matrix-free SIMPLESolver (cavity / generic bc dict)
# ----------------------------------------------------------------------------
class SimpleOracle:
    """Restatement of simple.py:11-285 (and the bicgsimp.py:114-151, 196
    variant when ``bicgsimp=True``: p' pinned at (1,1), east-wall fix)."""

    def __init__(self, lx, ly, nx, ny, bicgsimp=False):
        self.lx, self.ly, self.nx, self.ny = lx, ly, nx, ny
        self.dx, self.dy = lx / nx, ly / ny
        self.rho, self.mu, self.dt = 1.0, 0.01, 10000.0
        self.alpha_p = self.alpha_u = self.alpha_m = 0.001
        self.bicgsimp = bicgsimp
        if bicgsimp:   # bicgsimp.py:18-25
            self.dt, self.alpha_p, self.alpha_u, self.alpha_m = 1e12, 0.1, 0.8, 0.05
        z = np.zeros
        self.u = z((nx + 3, ny + 2)); self.v = z((nx + 2, ny + 3))
        self.u_mid = z((nx + 3, ny + 2)); self.v_mid = z((nx + 2, ny + 3))
        self.u0 = z((nx + 3, ny + 2)); self.v0 = z((nx + 2, ny + 3))
        self.p = z((nx + 2, ny + 2)); self.pcor = z((nx + 2, ny + 2)); self.mdiv = z((nx + 2, ny + 2))
        self.bc = {"w": [0.0, 0.0], "e": [0.0, 0.0], "n": [0.0, 0.0], "s": [0.0, 0.0]}
        self.coef_u = z((5, nx + 3, ny + 2)); self.b_u = z((nx + 3, ny + 2))
        self.coef_v = z((5, nx + 2, ny + 3)); self.b_v = z((nx + 2, ny + 3))
        self.coef_p = z((5, nx + 2, ny + 2)); self.b_p = z((nx + 2, ny + 2))

    def compute_coef_u(self):  # simple.py:77-92
        nx, ny, dx, dy, dt, rho, mu = self.nx, self.ny, self.dx, self.dy, self.dt, self.rho, self.mu
        u, v, p, u0, c = self.u, self.v, self.p, self.u0, self.coef_u
        I, J = slice(2, nx + 1), slice(1, ny + 1)
        ui, uw, ue = u[I, J], u[1:nx, J], u[3:nx + 2, J]
        vnw, vne, vsw, vse = v[1:nx, 2:ny + 2], v[2:nx + 1, 2:ny + 2], v[1:nx, J], v[2:nx + 1, J]
        c[1, I, J] = -(mu * dy / dx + 0.5 * rho * 0.5 * (ui + uw) * dy)
        c[2, I, J] = -(mu * dy / dx - 0.5 * rho * 0.5 * (ui + ue) * dy)
        c[3, I, J] = -(mu * dx / dy - 0.5 * rho * 0.5 * (vnw + vne) * dx)
        c[4, I, J] = -(mu * dx / dy + 0.5 * rho * 0.5 * (vsw + vse) * dx)
        c[0, I, J] = (-(c[1, I, J] + c[2, I, J] + c[3, I, J] + c[4, I, J])
                      + rho * 0.5 * (ui + ue) * dy - rho * 0.5 * (ui + uw) * dy
                      + rho * 0.5 * (vnw + vne) * dx - rho * 0.5 * (vsw + vse) * dx
                      + rho * dx * dy / dt)
        self.b_u[I, J] = (p[1:nx, J] - p[2:nx + 1, J]) * dy + rho * dx * dy / dt * u0[I, J]

    def compute_coef_v(self):  # simple.py:95-110
        nx, ny, dx, dy, dt, rho, mu = self.nx, self.ny, self.dx, self.dy, self.dt, self.rho, self.mu
        u, v, p, v0, c = self.u, self.v, self.p, self.v0, self.coef_v
        I, J = slice(1, nx + 1), slice(2, ny + 1)
        uc, us = u[I, J], u[I, 1:ny]
        uec, ues = u[2:nx + 2, J], u[2:nx + 2, 1:ny]
        vc, vn, vs = v[I, J], v[I, 3:ny + 2], v[I, 1:ny]
        c[1, I, J] = -(mu * dy / dx + 0.5 * rho * 0.5 * (uc + us) * dy)
        c[2, I, J] = -(mu * dy / dx - 0.5 * rho * 0.5 * (ues + uec) * dy)
        c[3, I, J] = -(mu * dx / dy - 0.5 * rho * 0.5 * (vn + vc) * dx)
        c[4, I, J] = -(mu * dx / dy + 0.5 * rho * 0.5 * (vs + vc) * dx)
        c[0, I, J] = (-(c[1, I, J] + c[2, I, J] + c[3, I, J] + c[4, I, J])
                      + rho * 0.5 * (ues + uec) * dy - rho * 0.5 * (uc + us) * dy
                      + rho * 0.5 * (vn + vc) * dx - rho * 0.5 * (vs + vc) * dx
                      + rho * dx * dy / dt)
        self.b_v[I, J] = (p[I, 1:ny] - p[I, J]) * dx + rho * dx * dy / dt * self.v0[I, J]

    def set_bc(self):  # simple.py:172-216 (bicgsimp.py:153-197 when bicgsimp)
        nx, ny, bc, mu, dx, dy = self.nx, self.ny, self.bc, self.mu, self.dx, self.dy
        cu, bu, cv, bv = self.coef_u, self.b_u, self.coef_v, self.b_v
        J = slice(1, ny + 1)
        bu[2, J] += -cu[1, 2, J] * bc["w"][0]; cu[1, 2, J] = 0.0; self.u[1, J] = bc["w"][0]
        bu[nx, J] += -cu[2, nx, J] * bc["e"][0]; cu[2, nx, J] = 0.0; self.u[nx + 1, J] = bc["e"][0]
        I = slice(1, nx + 1)
        bv[I, 2] += -cv[4, I, 2] * bc["s"][0]; cv[4, I, 2] = 0.0; self.v[I, 1] = bc["s"][0]
        bv[I, ny] += -cv[3, I, ny] * bc["n"][0]; cv[3, I, ny] = 0.0; self.v[I, ny + 1] = bc["n"][0]
        I = slice(2, nx + 1)
        bu[I, 1] += 2 * mu * bc["s"][1] * dx / dy
        cu[0, I, 1] += (cu[4, I, 1] + 2 * mu * dx / dy); cu[4, I, 1] = 0.0
        bu[I, ny] += 2 * mu * bc["n"][1] * dx / dy
        cu[0, I, ny] += (cu[3, I, ny] + 2 * mu * dx / dy); cu[3, I, ny] = 0.0
        J = slice(2, ny + 1)
        bv[1, J] += 2 * mu * bc["w"][1] * dy / dx
        cv[0, 1, J] += (cv[1, 1, J] + 2 * mu * dy / dx); cv[1, 1, J] = 0.0
        bv[nx, J] += 2 * mu * bc["e"][1] * dy / dx
        # simple.py:215 adds aW (component 1) here; bicgsimp.py:196 adds aE.
        cv[0, nx, J] += (cv[2 if self.bicgsimp else 1, nx, J] + 2 * mu * dy / dx); cv[2, nx, J] = 0.0

    def compute_mdiv(self):  # simple.py:137-141; bicgsimp.py:114-122 returns max|mdiv|
        nx, ny, dx, dy, rho = self.nx, self.ny, self.dx, self.dy, self.rho
        u, v = self.u, self.v
        I, J = slice(1, nx + 1), slice(1, ny + 1)
        self.mdiv[I, J] = rho * (u[I, J] - u[2:nx + 2, J]) * dy + rho * (v[I, J] - v[I, 2:ny + 2]) * dx
        return float(np.abs(self.mdiv[I, J]).max())

    def compute_coef_p(self):  # simple.py:143-170 (bicgsimp.py:124-151)
        nx, ny, dx, dy, rho = self.nx, self.ny, self.dx, self.dy, self.rho
        self.compute_mdiv()
        I, J = slice(1, nx + 1), slice(1, ny + 1)
        c, cu, cv = self.coef_p, self.coef_u, self.coef_v
        self.b_p[I, J] = self.mdiv[I, J]
        with np.errstate(divide="ignore"):
            c[1, I, J] = -rho * dy * dy / cu[0, I, J]
            c[2, I, J] = -rho * dy * dy / cu[0, 2:nx + 2, J]
            c[3, I, J] = -rho * dx * dx / cv[0, I, 2:ny + 2]
            c[4, I, J] = -rho * dx * dx / cv[0, I, J]
        c[1, 1, J] = 0.0; c[2, nx, J] = 0.0; c[4, I, 1] = 0.0; c[3, I, ny] = 0.0
        c[0, I, J] = -(c[1, I, J] + c[2, I, J] + c[3, I, J] + c[4, I, J])
        if self.bicgsimp:
            c[1:5, 1, 1] = 0.0; c[0, 1, 1] = 1.0; self.b_p[1, 1] = 0.0

    def correct_pressure(self):  # simple.py:218-222
        nx, ny = self.nx, self.ny
        self.p[1:nx + 1, 1:ny + 1] += self.alpha_p * self.pcor[1:nx + 1, 1:ny + 1]

    def correct_velocity(self):  # simple.py:224-230
        nx, ny, dx, dy = self.nx, self.ny, self.dx, self.dy
        pc = self.pcor
        I, J = slice(2, nx + 1), slice(1, ny + 1)
        self.u[I, J] += self.alpha_u * (pc[1:nx, J] - pc[I, J]) * dy / self.coef_u[0, I, J]
        I, J = slice(1, nx + 1), slice(2, ny + 1)
        self.v[I, J] += self.alpha_u * (pc[I, 1:ny] - pc[I, J]) * dx / self.coef_v[0, I, J]

    def update_velocity(self):  # simple.py:232-238 (bicgsimp.py:212-225 returns max diff)
        nx, ny, a = self.nx, self.ny, self.alpha_m
        I, J = slice(2, nx + 1), slice(1, ny + 1)
        du = np.abs(self.u_mid[I, J] - self.u[I, J]).max(initial=0.0)
        self.u[I, J] = a * self.u_mid[I, J] + (1 - a) * self.u[I, J]
        I, J = slice(1, nx + 1), slice(2, ny + 1)
        dv = np.abs(self.v_mid[I, J] - self.v[I, J]).max(initial=0.0)
        self.v[I, J] = a * self.v_mid[I, J] + (1 - a) * self.v[I, J]
        return math.sqrt(du ** 2 + dv ** 2)

    def solve_momentum_eqn(self, n_iter=1, eps=1e-1):  # simple.py:241-250
        for _ in range(n_iter):
            self.compute_coef_u(); self.compute_coef_v(); self.set_bc()
            ru = bicgstab(self.coef_u, self.b_u, self.b_u.shape[1], eps=eps)
            rv = bicgstab(self.coef_v, self.b_v, self.b_v.shape[1], eps=eps)
            self.u_mid[...] = ru.x.reshape(self.u_mid.shape)
            self.v_mid[...] = rv.x.reshape(self.v_mid.shape)
            # bicgsimp.py:209-210 returns update_velocity's max-change residual
            self.last_momentum_residual = self.update_velocity()
        return ru, rv

    def solve_pcorrection_eqn(self, eps=1e-2):  # simple.py:252-255
        self.compute_coef_p()
        res = cg(self.coef_p, self.b_p, self.b_p.shape[1], eps=eps)
        self.pcor[...] = res.x.reshape(self.pcor.shape)
        return res

    def init(self):  # simple.py:257-264
        self.u[...] = 0.0; self.v[...] = 0.0; self.p[...] = 0.0

    def solve(self, n_steps=2000):  # simple.py:266-285 without the CSV/PNG dumps
        self.init()
        for _ in range(n_steps):
            self.solve_momentum_eqn(1)
            self.compute_mdiv()
            self.solve_pcorrection_eqn()
            self.correct_pressure(); self.correct_velocity()
            self.compute_mdiv()


# ----------------------------------------------------------------------------
# Channel preset: velocity inlet, zero-gradient outlet, no-slip walls,
# blocked-cell cylinder (the benchmark configurations)
# ----------------------------------------------------------------------------
def channel_solid_mask(nx, ny, obstacles):
    """uint8 [nx+2, ny+2]; 1 = blocked cell.  ``obstacles`` is a list of
    ``(shape, ci, cj, D)`` in padded cell indices.  'square': cells
    [c - D//2, c - D//2 + D - 1] in i and j.  'circle': the reference's
    rule (i - ci)^2 + (j - cj)^2 < (D/2)^2 (karman_taichi.py:148-150)."""
    m = np.zeros((nx + 2, ny + 2), dtype=np.uint8)
    ii, jj = np.meshgrid(np.arange(nx + 2), np.arange(ny + 2), indexing="ij")
    inside = (ii >= 1) & (ii <= nx) & (jj >= 1) & (jj <= ny)
    for shape, ci, cj, D in obstacles:
        if shape == "square":
            lo_i, lo_j = ci - D // 2, cj - D // 2
            sel = (ii >= lo_i) & (ii <= lo_i + D - 1) & (jj >= lo_j) & (jj <= lo_j + D - 1)
        else:
            r2 = (D * D) // 4 if D % 2 == 0 else (D * D) / 4.0
            sel = ((ii - ci) ** 2 + (jj - cj) ** 2) < r2
        m[sel & inside] = 1
    return m


@dataclass
class ChannelParams:
    nx: int
    ny: int
    dx: float
    dy: float
    rho: float
    mu: float
    dt: float
    U: float = 1.0
    alpha_m: float = 0.7
    alpha_u: float = 1.0
    alpha_p: float = 0.3
    eps: float = 1e-8
    mass_tol: float = 1e-6
    max_outer: int = 50


class ChannelOracle:
    """FP64 restatement of the channel SIMPLE step.  The discretisation is
    simple.py's mid-point scheme (simple.py:77-110) with set_bc's wall and
    Dirichlet folding (simple.py:172-216); the outlet uses karman_taichi.py's
    zero-gradient row and mass-flow rescale (karman_taichi.py:178-183,
    586-614); blocked faces become identity rows (karman_taichi.py:225-229)."""

    def __init__(self, prm: ChannelParams, solid, u, v, p):
        self.P = prm
        nx, ny = prm.nx, prm.ny
        self.solid = solid.astype(bool)
        self.u = u.astype(np.float64).copy(); self.v = v.astype(np.float64).copy()
        self.p = p.astype(np.float64).copy()
        self.u0 = self.u.copy(); self.v0 = self.v.copy()
        self.pcor = np.zeros((nx + 2, ny + 2))
        s = self.solid
        bu = np.zeros((nx + 3, ny + 2), bool)
        bu[1:nx + 2, :] = s[0:nx + 1, :] | s[1:nx + 2, :]
        bv = np.zeros((nx + 2, ny + 3), bool)
        bv[:, 1:ny + 2] = s[:, 0:ny + 1] | s[:, 1:ny + 2]
        self.blk_u, self.blk_v = bu, bv
        unk_u = np.zeros_like(bu); unk_u[2:nx + 1, 1:ny + 1] = ~bu[2:nx + 1, 1:ny + 1]
        unk_v = np.zeros_like(bv); unk_v[1:nx + 1, 2:ny + 1] = ~bv[1:nx + 1, 2:ny + 1]
        self.unk_u, self.unk_v = unk_u, unk_v
        self.coef_u = np.zeros((5, nx + 3, ny + 2)); self.b_u = np.zeros((nx + 3, ny + 2))
        self.coef_v = np.zeros((5, nx + 2, ny + 3)); self.b_v = np.zeros((nx + 2, ny + 3))
        self.coef_p = np.zeros((5, nx + 2, ny + 2)); self.b_p = np.zeros((nx + 2, ny + 2))
        self.stats = []

    # -- momentum ----------------------------------------------------------
    def assemble_momentum(self):
        P = self.P
        nx, ny, dx, dy, dt, rho, mu = P.nx, P.ny, P.dx, P.dy, P.dt, P.rho, P.mu
        u, v, p = self.u, self.v, self.p
        c, b = self.coef_u, self.b_u
        c[...] = 0.0; b[...] = 0.0
        I, J = slice(2, nx + 1), slice(1, ny + 1)
        ui, uw, ue = u[I, J], u[1:nx, J], u[3:nx + 2, J]
        vnw, vne, vsw, vse = v[1:nx, 2:ny + 2], v[2:nx + 1, 2:ny + 2], v[1:nx, J], v[2:nx + 1, J]
        aW = -(mu * dy / dx + 0.5 * rho * 0.5 * (ui + uw) * dy)
        aE = -(mu * dy / dx - 0.5 * rho * 0.5 * (ui + ue) * dy)
        aN = -(mu * dx / dy - 0.5 * rho * 0.5 * (vnw + vne) * dx)
        aS = -(mu * dx / dy + 0.5 * rho * 0.5 * (vsw + vse) * dx)
        aP = (-(aW + aE + aN + aS) + rho * 0.5 * (ui + ue) * dy - rho * 0.5 * (ui + uw) * dy
              + rho * 0.5 * (vnw + vne) * dx - rho * 0.5 * (vsw + vse) * dx + rho * dx * dy / dt)
        bb = (p[1:nx, J] - p[I, J]) * dy + rho * dx * dy / dt * self.u0[I, J]
        ii = np.arange(2, nx + 1)[:, None] + 0 * np.arange(ny)[None, :]
        jj = np.arange(1, ny + 1)[None, :] + 0 * ii
        bu = self.blk_u
        wall_x = 2 * mu * dx / dy
        # west
        m = ii == 2
        bb = np.where(m, bb + (-aW * P.U), bb); aW = np.where(m, 0.0, aW)
        m = (ii > 2) & bu[1:nx, J]
        aW = np.where(m, 0.0, aW)
        # east
        m = ii == nx
        aP = np.where(m, aP + aE, aP); aE = np.where(m, 0.0, aE)
        m = (ii < nx) & bu[3:nx + 2, J]
        aE = np.where(m, 0.0, aE)
        # south
        m = (jj == 1) | bu[I, 0:ny]
        aP = np.where(m, aP + (aS + wall_x), aP); aS = np.where(m, 0.0, aS)
        # north
        m = (jj == ny) | bu[I, 2:ny + 2]
        aP = np.where(m, aP + (aN + wall_x), aP); aN = np.where(m, 0.0, aN)
        blk = bu[I, J]
        c[0, I, J] = np.where(blk, 1.0, aP)
        c[1, I, J] = np.where(blk, 0.0, aW); c[2, I, J] = np.where(blk, 0.0, aE)
        c[3, I, J] = np.where(blk, 0.0, aN); c[4, I, J] = np.where(blk, 0.0, aS)
        b[I, J] = np.where(blk, 0.0, bb)

        c, b = self.coef_v, self.b_v
        c[...] = 0.0; b[...] = 0.0
        I, J = slice(1, nx + 1), slice(2, ny + 1)
        uc, us = u[I, J], u[I, 1:ny]
        uec, ues = u[2:nx + 2, J], u[2:nx + 2, 1:ny]
        vc, vn, vs = v[I, J], v[I, 3:ny + 2], v[I, 1:ny]
        aW = -(mu * dy / dx + 0.5 * rho * 0.5 * (uc + us) * dy)
        aE = -(mu * dy / dx - 0.5 * rho * 0.5 * (ues + uec) * dy)
        aN = -(mu * dx / dy - 0.5 * rho * 0.5 * (vn + vc) * dx)
        aS = -(mu * dx / dy + 0.5 * rho * 0.5 * (vs + vc) * dx)
        aP = (-(aW + aE + aN + aS) + rho * 0.5 * (ues + uec) * dy - rho * 0.5 * (uc + us) * dy
              + rho * 0.5 * (vn + vc) * dx - rho * 0.5 * (vs + vc) * dx + rho * dx * dy / dt)
        bb = (p[I, 1:ny] - p[I, J]) * dx + rho * dx * dy / dt * self.v0[I, J]
        ii = np.arange(1, nx + 1)[:, None] + 0 * np.arange(ny - 1)[None, :]
        jj = np.arange(2, ny + 1)[None, :] + 0 * ii
        bv = self.blk_v
        wall_y = 2 * mu * dy / dx
        # south / north: Dirichlet v = 0 (walls and obstacle faces)
        m = (jj == 2) | bv[I, 1:ny]
        aS = np.where(m, 0.0, aS)
        m = (jj == ny) | bv[I, 3:ny + 2]
        aN = np.where(m, 0.0, aN)
        # west: inlet (tangential v = 0) or obstacle side -> wall
        m = (ii == 1) | bv[0:nx, J]
        aP = np.where(m, aP + (aW + wall_y), aP); aW = np.where(m, 0.0, aW)
        # east: outlet zero gradient, obstacle side -> wall
        m = ii == nx
        aP = np.where(m, aP + aE, aP); aE = np.where(m, 0.0, aE)
        m = (ii < nx) & bv[2:nx + 2, J]
        aP = np.where(m, aP + (aE + wall_y), aP); aE = np.where(m, 0.0, aE)
        blk = bv[I, J]
        c[0, I, J] = np.where(blk, 1.0, aP)
        c[1, I, J] = np.where(blk, 0.0, aW); c[2, I, J] = np.where(blk, 0.0, aE)
        c[3, I, J] = np.where(blk, 0.0, aN); c[4, I, J] = np.where(blk, 0.0, aS)
        b[I, J] = np.where(blk, 0.0, bb)

    def relax(self, u_mid, v_mid):
        """Explicit under-relaxation of the momentum solution (simple.py:232-238),
        then the zero-gradient outlet and the mass-flow rescale
        (karman_taichi.py:586-601)."""
        a = self.P.alpha_m
        m = self.unk_u
        self.u[m] = a * u_mid[m] + (1 - a) * self.u[m]
        m = self.unk_v
        self.v[m] = a * v_mid[m] + (1 - a) * self.v[m]
        nx, ny = self.P.nx, self.P.ny
        J = slice(1, ny + 1)
        self.u[nx + 1, J] = self.u[nx, J]
        mdot_in = float(np.sum(self.u[1, J]))
        mdot_out = float(np.sum(self.u[nx + 1, J]))
        self.u[nx + 1, J] = (mdot_in / mdot_out) * self.u[nx + 1, J]

    # -- pressure correction ------------------------------------------------
    def assemble_p(self):
        P = self.P
        nx, ny, dx, dy, rho = P.nx, P.ny, P.dx, P.dy, P.rho
        u, v = self.u, self.v
        c, b = self.coef_p, self.b_p
        c[...] = 0.0; b[...] = 0.0
        I, J = slice(1, nx + 1), slice(1, ny + 1)
        mdiv = rho * (u[I, J] - u[2:nx + 2, J]) * dy + rho * (v[I, J] - v[I, 2:ny + 2]) * dx
        apu, apv = self.coef_u[0], self.coef_v[0]
        uu, uv = self.unk_u, self.unk_v
        with np.errstate(divide="ignore", invalid="ignore"):
            aW = np.where(uu[I, J], -rho * dy * dy / apu[I, J], 0.0)
            aE = np.where(uu[2:nx + 2, J], -rho * dy * dy / apu[2:nx + 2, J], 0.0)
            out = np.zeros_like(aE, dtype=bool); out[nx - 1, :] = uu[nx, J]
            aE = np.where(out, -rho * dy * dy / apu[nx:nx + 1, J], aE)
            aN = np.where(uv[I, 2:ny + 2], -rho * dx * dx / apv[I, 2:ny + 2], 0.0)
            aS = np.where(uv[I, J], -rho * dx * dx / apv[I, J], 0.0)
        aP = -(aW + aE + aN + aS)
        sol = self.solid[I, J]
        c[0, I, J] = np.where(sol, 1.0, aP)
        c[1, I, J] = np.where(sol, 0.0, aW); c[2, I, J] = np.where(sol, 0.0, aE)
        c[3, I, J] = np.where(sol, 0.0, aN); c[4, I, J] = np.where(sol, 0.0, aS)
        b[I, J] = np.where(sol, 0.0, mdiv)
        return float(np.abs(np.where(sol, 0.0, mdiv)).max())

    def correct(self):
        """Velocity/pressure correction (simple.py:218-230 with alpha_u, and
        the outlet face corrected against p' = 0 beyond the outlet)."""
        P = self.P
        nx, ny, dx, dy = P.nx, P.ny, P.dx, P.dy
        pc = self.pcor
        apu, apv = self.coef_u[0], self.coef_v[0]
        I, J = slice(2, nx + 1), slice(1, ny + 1)
        m = self.unk_u[I, J]
        self.u[I, J] = np.where(m, self.u[I, J] + P.alpha_u * (pc[1:nx, J] - pc[I, J]) * dy
                                / np.where(m, apu[I, J], 1.0), self.u[I, J])
        m = self.unk_u[nx, J]
        self.u[nx + 1, J] = np.where(m, self.u[nx + 1, J] + P.alpha_u * (pc[nx, J] - pc[nx + 1, J]) * dy
                                     / np.where(m, apu[nx, J], 1.0), self.u[nx + 1, J])
        I, J = slice(1, nx + 1), slice(2, ny + 1)
        m = self.unk_v[I, J]
        self.v[I, J] = np.where(m, self.v[I, J] + P.alpha_u * (pc[I, 1:ny] - pc[I, J]) * dx
                                / np.where(m, apv[I, J], 1.0), self.v[I, J])
        I, J = slice(1, nx + 1), slice(1, ny + 1)
        fl = ~self.solid[I, J]
        self.p[I, J] = np.where(fl, self.p[I, J] + P.alpha_p * pc[I, J], self.p[I, J])
        return float(np.abs(pc).max())

    def mass_residual(self):
        """max |mdiv| over fluid cells of the current field (bicgsimp.py:114-122)."""
        P = self.P
        nx, ny, dx, dy, rho = P.nx, P.ny, P.dx, P.dy, P.rho
        I, J = slice(1, nx + 1), slice(1, ny + 1)
        mdiv = rho * (self.u[I, J] - self.u[2:nx + 2, J]) * dy + rho * (self.v[I, J] - self.v[I, 2:ny + 2]) * dx
        return float(np.abs(np.where(self.solid[I, J], 0.0, mdiv)).max())

    def outer_iteration(self):
        P = self.P
        self.assemble_momentum()
        ru = bicgstab(self.coef_u, self.b_u, self.b_u.shape[1], eps=P.eps)
        rv = bicgstab(self.coef_v, self.b_v, self.b_v.shape[1], eps=P.eps)
        self.relax(ru.x.reshape(self.u.shape), rv.x.reshape(self.v.shape))
        R = self.assemble_p()
        rp = bicgstab(self.coef_p, self.b_p, self.b_p.shape[1], eps=P.eps)
        self.pcor[...] = rp.x.reshape(self.pcor.shape)
        pmax = self.correct()
        return dict(mass=R, it_u=ru.iters, it_v=rv.iters, it_p=rp.iters,
                    st=(ru.status, rv.status, rp.status), pcor_max=pmax)

    def step(self):
        """One time step: SIMPLE outer iterations until the momentum-predicted
        mass residual is <= mass_tol or max_outer, then u0 <- u, v0 <- v
        (karman_taichi.py:617-622)."""
        rec = []
        for k in range(self.P.max_outer):
            s = self.outer_iteration()
            rec.append(s)
            if s["mass"] <= self.P.mass_tol:
                break
        self.u0 = self.u.copy(); self.v0 = self.v.copy()
        self.stats.append(rec)
        return rec


# ----------------------------------------------------------------------------
# karman_taichi.py: assembled-matrix driver, literal sparse emulation
# ----------------------------------------------------------------------------
class SparseRows:
    """Pointer-SNode stand-in: a persistent dict of written (row, col) entries;
    unwritten entries read 0 and writes outside [0, n) are dropped."""

    def __init__(self, n):
        self.n = n
        self.e = {}

    def __setitem__(self, rc, val):
        r, c = rc
        if 0 <= r < self.n and 0 <= c < self.n:
            self.e[(r, c)] = float(val)

    def __getitem__(self, rc):
        return self.e.get(rc, 0.0)

    def planes(self, S):
        """Convert to flat 5-point planes [P, W(-S), E(+S), N(+1), S(-1)];
        asserts that nothing else is stored on the stencil's 7-offset gather."""
        n = self.n
        c = np.zeros((5, n))
        slot = {0: 0, -S: 1, S: 2, 1: 3, -1: 4}
        for (r, col), val in self.e.items():
            off = col - r
            if off in slot:
                c[slot[off], r] = val
            elif abs(off) in (S - 1, S + 1) and val != 0.0:
                raise AssertionError(f"entry off the 5-point pattern: {(r, col)}")
        return c


class KarmanOracle:
    """Restatement of karman_taichi.py (channel + circle, pressure-driven).
    Geometry and constants follow karman_taichi.py:7-25; ``nx=320, ny=64`` is
    debug/karman_taichi.py:11-12."""

    def __init__(self, nx=640, ny=128, lx=0.5, ly=0.1, rho=1.0, mu=0.01, dt=1e-5,
                 velo_rel=0.8, p_rel=0.2, circle=(64, 32, 144)):
        self.nx, self.ny = nx, ny
        self.dx, self.dy = lx / nx, ly / ny
        self.rho, self.mu, self.dt = rho, mu, dt
        self.velo_rel, self.p_rel = velo_rel, p_rel
        self.circle = circle
        self.nu, self.nv, self.np_ = (nx + 1) * ny, nx * (ny + 1), nx * ny
        self.Au, self.Mu = SparseRows(self.nu), SparseRows(self.nu)
        self.Av, self.Mv = SparseRows(self.nv), SparseRows(self.nv)
        self.Ap, self.Mp = SparseRows(self.np_), SparseRows(self.np_)
        self.bu, self.xu = np.zeros(self.nu), np.zeros(self.nu)
        self.bv, self.xv = np.zeros(self.nv), np.zeros(self.nv)
        self.bp, self.xp = np.zeros(self.np_), np.zeros(self.np_)
        self.init()

    def init(self):  # karman_taichi.py:130-154
        nx, ny = self.nx, self.ny
        i = np.arange(nx + 2)[:, None] * np.ones((1, ny + 2))
        self.p = 100 - 4000.0 * i / nx
        self.pcor = np.zeros((nx + 2, ny + 2))
        self.u = np.zeros((nx + 3, ny + 2)); self.u0 = np.zeros((nx + 3, ny + 2))
        self.v = np.zeros((nx + 2, ny + 3)); self.v0 = np.zeros((nx + 2, ny + 3))
        ct = np.ones((nx + 2, ny + 2), dtype=np.int32)
        ct[1:nx + 1, 1:ny + 1] = -1
        ci, cj, r2 = self.circle
        ii, jj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
        sel = ((ii - ci) ** 2 + (jj - cj) ** 2) < r2
        ct[:nx, :ny][sel] = 1
        self.ct = ct
        self.udiv = np.zeros((nx + 2, ny + 2))

    def fill_Au(self):  # karman_taichi.py:162-248
        nx, ny, dx, dy, dt, rho, mu = self.nx, self.ny, self.dx, self.dy, self.dt, self.rho, self.mu
        ct, u, v, p, u0 = self.ct, self.u, self.v, self.p, self.u0
        A, M, b = self.Au, self.Mu, self.bu
        for i in range(1, nx + 2):
            for j in range(1, ny + 1):
                k = (i - 1) * ny + (j - 1)
                if ct[i - 1, j] == 1:
                    A[k, k] = 1.0; A[k, k + ny] = -1.0; b[k] = 0.0
                elif ct[i, j] == 1:
                    A[k, k] = 1.0; A[k, k - ny] = -1.0; b[k] = 0.0
                elif (ct[i, j] + ct[i, j - 1]) == 0:
                    A[k, k + 1] = -mu * dx / dy - rho * 0.5 * (v[i - 1, j + 1] + v[i, j + 1]) * dx
                    A[k, k - ny] = -mu * dy / dx - rho * 0.5 * (u[i, j] + u[i - 1, j]) * dy
                    A[k, k + ny] = -mu * dy / dx - (-rho * 0.5 * (u[i, j] + u[i + 1, j]) * dy)
                    A[k, k] = -A[k, k + 1] - A[k, k - ny] - A[k, k + ny] + rho * dx * dy / dt + 2 * mu * dx / dy
                    b[k] = (p[i - 1, j] - p[i, j]) * dy + rho * dx * dy / dt * u0[i, j]
                elif (ct[i, j] + ct[i, j + 1]) == 0:
                    A[k, k - 1] = -mu * dx / dy - (-rho * 0.5 * (v[i - 1, j] + v[i, j]) * dx)
                    A[k, k - ny] = -mu * dy / dx - rho * 0.5 * (u[i, j] + u[i - 1, j]) * dy
                    A[k, k + ny] = -mu * dy / dx - (-rho * 0.5 * (u[i, j] + u[i + 1, j]) * dy)
                    A[k, k] = -A[k, k - 1] - A[k, k - ny] - A[k, k + ny] + rho * dx * dy / dt + 2 * mu * dx / dy
                    b[k] = (p[i - 1, j] - p[i, j]) * dy + rho * dx * dy / dt * u0[i, j]
                else:
                    A[k, k - 1] = -mu * dx / dy - (-rho * 0.5 * (v[i - 1, j] + v[i, j]) * dx)
                    A[k, k + 1] = -mu * dx / dy - rho * 0.5 * (v[i - 1, j + 1] + v[i, j + 1]) * dx
                    A[k, k - ny] = -mu * dy / dx - rho * 0.5 * (u[i, j] + u[i - 1, j]) * dy
                    A[k, k + ny] = -mu * dy / dx - (-rho * 0.5 * (u[i, j] + u[i + 1, j]) * dy)
                    A[k, k] = -A[k, k - 1] - A[k, k + 1] - A[k, k - ny] - A[k, k + ny] + rho * dx * dy / dt
                    b[k] = (p[i - 1, j] - p[i, j]) * dy + rho * dx * dy / dt * u0[i, j]
                M[k, k] = A[k, k]
        for i in range(2, nx + 1):
            for j in range(2, ny):
                k = (i - 1) * ny + (j - 1)
                if (ct[i - 1, j] + ct[i, j]) == 0 or (ct[i - 1, j] + ct[i, j]) == 2:
                    for nb in (k - ny, k - 1, k + 1, k + ny):
                        A[k, nb] = 0.0
                    A[k, k] = 1.0; b[k] = 0.0
                elif (ct[i, j] + ct[i, j - 1]) == 0 or (ct[i - 1, j] + ct[i - 1, j - 1]) == 0:
                    A[k, k + 1] = -mu * dx / dy - rho * 0.5 * (v[i - 1, j + 1] + v[i, j + 1]) * dx
                    A[k, k - ny] = -mu * dy / dx - rho * 0.5 * (u[i, j] + u[i - 1, j]) * dy
                    A[k, k + ny] = -mu * dy / dx - (-rho * 0.5 * (u[i, j] + u[i + 1, j]) * dy)
                    A[k, k] = -A[k, k + 1] - A[k, k - ny] - A[k, k + ny] + rho * dx * dy / dt + 2 * mu * dx / dy
                    b[k] = (p[i - 1, j] - p[i, j]) * dy + rho * dx * dy / dt * u0[i, j]

    def fill_Av(self):  # karman_taichi.py:251-294
        nx, ny, dx, dy, dt, rho, mu = self.nx, self.ny, self.dx, self.dy, self.dt, self.rho, self.mu
        ct, u, v, p, v0 = self.ct, self.u, self.v, self.p, self.v0
        A, M, b = self.Av, self.Mv, self.bv
        for i in range(1, nx + 1):
            for j in range(1, ny + 2):
                k = (i - 1) * (ny + 1) + (j - 1)
                if (ct[i, j] + ct[i, j - 1]) == 0 or (ct[i, j] + ct[i, j - 1]) == 2:
                    A[k, k] = 1.0; b[k] = v[i, j]
                elif (ct[i, j] + ct[i - 1, j]) == 0:
                    A[k, k - 1] = -mu * dx / dy - (-rho * 0.5 * (v[i, j - 1] + v[i, j]) * dx)
                    A[k, k + 1] = -mu * dx / dy - (rho * 0.5 * (v[i, j + 1] + v[i, j]) * dx)
                    A[k, k + ny + 1] = -mu * dy / dx - (-rho * 0.5 * (u[i + 1, j - 1] + u[i + 1, j]) * dy)
                    A[k, k] = -A[k, k - 1] - A[k, k + 1] - A[k, k + ny + 1] + rho * dx * dy / dt + 2 * mu * dy / dx
                    b[k] = (p[i, j] - p[i, j - 1]) * dx + rho * dx * dy / dt * v0[i, j]
                elif (ct[i, j] + ct[i + 1, j]) == 0:
                    A[k, k - 1] = -mu * dx / dy - (-rho * 0.5 * (v[i, j - 1] + v[i, j]) * dx)
                    A[k, k + 1] = -mu * dx / dy - (rho * 0.5 * (v[i, j + 1] + v[i, j]) * dx)
                    A[k, k - ny - 1] = -mu * dy / dx - (rho * 0.5 * (u[i, j] + u[i, j - 1]) * dy)
                    A[k, k] = -A[k, k - 1] - A[k, k + 1] - A[k, k - ny - 1] + rho * dx * dy / dt + 2 * mu * dy / dx
                    b[k] = (p[i, j] - p[i, j - 1]) * dx + rho * dx * dy / dt * v0[i, j]
                else:
                    A[k, k - 1] = -mu * dx / dy - (-rho * 0.5 * (v[i, j - 1] + v[i, j]) * dx)
                    A[k, k + 1] = -mu * dx / dy - (rho * 0.5 * (v[i, j + 1] + v[i, j]) * dx)
                    A[k, k - ny - 1] = -mu * dy / dx - (rho * 0.5 * (u[i, j] + u[i, j - 1]) * dy)
                    A[k, k + ny + 1] = -mu * dy / dx - (-rho * 0.5 * (u[i + 1, j - 1] + u[i + 1, j]) * dy)
                    A[k, k] = (-A[k, k - 1] - A[k, k + 1] - A[k, k - ny - 1] - A[k, k + ny + 1]
                               + rho * dx * dy / dt)
                    b[k] = (p[i, j] - p[i, j - 1]) * dx + rho * dx * dy / dt * v0[i, j]
        for i in range(1, nx + 1):
            for j in range(1, ny + 2):
                k = (i - 1) * (ny + 1) + (j - 1)
                M[k, k] = A[k, k]

    def fill_Ap(self):  # karman_taichi.py:297-339
        nx, ny, dx, dy, rho = self.nx, self.ny, self.dx, self.dy, self.rho
        ct, u, v = self.ct, self.u, self.v
        A, M, b, Au, Av = self.Ap, self.Mp, self.bp, self.Au, self.Av
        n = nx * ny
        with np.errstate(divide="ignore"):
            for i in range(1, nx + 1):
                for j in range(1, ny + 1):
                    k = (i - 1) * ny + (j - 1)
                    b[k] = rho * (u[i, j] - u[i + 1, j]) * dy + rho * (v[i, j + 1] - v[i, j]) * dx
                    vk = (i - 1) * (ny + 1) + (j - 1)
                    A[k, k - 1] = -rho * dx * dx / np.float64(Av[vk, vk])
                    A[k, k + 1] = -rho * dx * dx / np.float64(Av[vk + 1, vk + 1])
                    uk = k
                    A[k, k - ny] = -rho * dy * dy / np.float64(Au[uk, uk])
                    A[k, k + ny] = -rho * dy * dy / np.float64(Au[uk + ny, uk + ny])
                    if (ct[i, j] + ct[i, j - 1]) == 0:
                        A[k, k - 1] = 0
                    if (ct[i, j] + ct[i, j + 1]) == 0:
                        A[k, k + 1] = 0
                    if (ct[i, j] + ct[i - 1, j]) == 0:
                        A[k, k - ny] = 0
                    if (ct[i, j] + ct[i + 1, j]) == 0:
                        A[k, k + ny] = 0
                    A[k, k] = -A[k, k - 1] - A[k, k + 1] - A[k, k - ny] - A[k, k + ny]
                    M[k, k] = A[k, k]
        # second loop: inlet rows pinned with off-diagonals cleared; the outlet
        # pins rows n-ny+1 .. n-1 (row n is out of range) and keeps their links
        for i in range(ny):
            for key in [kk for kk in A.e if kk[0] == i and kk[1] != i]:
                A.e[key] = 0.0
            A[i, i] = 1.0; M[i, i] = 1.0; b[i] = 0.0
            A[n - i, n - i] = 1.0; M[n - i, n - i] = 1.0
            if n - i < n:
                b[n - i] = 0.0

    def solve(self, A, M, b, x, eps):  # karman_taichi.py:342-456
        n = b.size
        S = self.ny if n in (self.nu, self.np_) else self.ny + 1
        planes = A.planes(S)
        diag = np.array([M[k, k] for k in range(n)])
        res = bicgstab(planes, b, S, eps=eps, max_iter=100 * n, x0=x, M=diag,
                       omega_break=True, order="karman")
        x[...] = res.x
        return res

    def solve_momentum_bicgstab(self, eps=1e-8, max_iterations=1):  # :482-494
        for _ in range(max_iterations):
            self.fill_Au(); self.fill_Av()
            ru = self.solve(self.Au, self.Mu, self.bu, self.xu, eps)
            rv = self.solve(self.Av, self.Mv, self.bv, self.xv, eps)
            self.xu_back(); self.xv_back()
        return ru, rv

    def xu_back(self):  # :459-464
        nx, ny, a = self.nx, self.ny, self.velo_rel
        xu = self.xu.reshape(nx + 1, ny)
        self.u[1:nx + 2, 1:ny + 1] = self.u[1:nx + 2, 1:ny + 1] + a * (xu - self.u[1:nx + 2, 1:ny + 1])

    def xv_back(self):  # :467-472
        nx, ny, a = self.nx, self.ny, self.velo_rel
        xv = self.xv.reshape(nx, ny + 1)
        self.v[1:nx + 1, 1:ny + 2] = self.v[1:nx + 1, 1:ny + 2] + a * (xv - self.v[1:nx + 1, 1:ny + 2])

    def xp_back(self):  # :475-478
        self.pcor[1:self.nx + 1, 1:self.ny + 1] = self.xp.reshape(self.nx, self.ny)

    def solve_pcorrection_bicgstab(self, eps=1e-8):  # :497-504
        self.fill_Ap()
        res = self.solve(self.Ap, self.Mp, self.bp, self.xp, eps)
        self.xp_back()
        return res

    def puv_correction(self):  # :507-542
        nx, ny, dx, dy = self.nx, self.ny, self.dx, self.dy
        ct, pc = self.ct, self.pcor
        for i in range(1, nx + 2):
            for j in range(1, ny + 1):
                k = (i - 1) * ny + (j - 1)
                s = ct[i - 1, j] + ct[i, j]
                if s != 0 and s != 2:
                    self.u[i, j] = self.u[i, j] + (pc[i - 1, j] - pc[i, j]) * dy / self.Au[k, k]
        for i in range(1, nx + 1):
            for j in range(1, ny + 2):
                k = (i - 1) * (ny + 1) + (j - 1)
                s = ct[i, j] + ct[i, j - 1]
                if s != 0 and s != 2:
                    self.v[i, j] = self.v[i, j] + (pc[i, j] - pc[i, j - 1]) * dx / self.Av[k, k]
        fl = ct != 1
        self.p[fl] = self.p[fl] + self.p_rel * pc[fl]
        return float(np.abs(pc).max())

    def correct_conserv(self):  # :586-614
        nx, ny, dx, dy = self.nx, self.ny, self.dx, self.dy
        J = slice(1, ny + 1)
        coef = float(np.sum(self.u[1, J])) / float(np.sum(self.u[nx + 1, J]))
        self.u[nx + 1, J] = coef * self.u[nx + 1, J]
        I = slice(1, nx + 1)
        self.udiv[I, J] = (self.u[I, J] - self.u[2:nx + 2, J]) * dy + (self.v[I, 2:ny + 2] - self.v[I, J]) * dx

    def time_forward(self):  # :617-622
        self.u0 = self.u.copy(); self.v0 = self.v.copy()

    def substep(self):
        """One SIMPLE sub-iteration of the __main__ loop (karman_taichi.py:636-651)."""
        ru, rv = self.solve_momentum_bicgstab(1e-8, 1)
        self.correct_conserv()
        rp = self.solve_pcorrection_bicgstab(1e-8)
        pmax = self.puv_correction()
        return dict(it_u=ru.iters, it_v=rv.iters, it_p=rp.iters, pcor_max=pmax,
                    st=(ru.status, rv.status, rp.status))


# ----------------------------------------------------------------------------
# Aggregation multigrid V-cycle (restatement of the GB300 preconditioner, FP32)
# ----------------------------------------------------------------------------
class MultigridOracle:
    """2x2 Galerkin aggregation in Laplacian form (rows without off-diagonal
    links are isolated: solved pointwise, never aggregated, links into them
    folded into the row sum), red-black
    Gauss-Seidel smoothing weighted by omega[l] (nu_pre / nu_post sweeps on
    level 0, nu_coarse on every level below), coarse corrections scaled by
    alpha[l]; on the coarsest level Jacobi sweeps (<= 1024 cells) or, with
    coarsest_sweeps = 0, the exact solve by a dense FP32 inverse (<= 128 cells)."""

    COARSEST = 1024          # coarsest level of the Jacobi variant (cells)
    COARSEST_DIRECT = 128    # coarsest level of the direct variant (coarsest_sweeps = 0)

    def __init__(self, coef, NX, NY, nu_pre=1, nu_post=1, coarsest_sweeps=0, omega=(1.0, 1.5), alpha=(1.9, 2.0),
                 max_levels=16, lap=False, nu_coarse=2):
        f32 = np.float32
        om = list(omega) if hasattr(omega, "__len__") else [omega] * 16
        al = list(alpha) if hasattr(alpha, "__len__") else [alpha] * 16
        self.omega = [f32(om[min(l, len(om) - 1)]) for l in range(16)]
        self.alpha = [f32(al[min(l, len(al) - 1)]) for l in range(16)]
        self.nu_pre, self.nu_post, self.sweeps = nu_pre, nu_post, coarsest_sweeps
        self.nu_coarse = max(1, nu_coarse)
        c = np.asarray(coef, dtype=f32).reshape(5, NX, NY)
        self.levels = [self._level(c, NX, NY, self.omega[0], lap)]
        target = self.COARSEST_DIRECT if coarsest_sweeps == 0 else self.COARSEST
        while len(self.levels) < max_levels and NX * NY > target:
            NXc, NYc = (NX + 1) // 2, (NY + 1) // 2
            c = self._coarsen(c, self.levels[-1]["iso"], NX, NY, NXc, NYc, self.levels[-1]["lap"])
            NX, NY = NXc, NYc
            self.levels.append(self._level(c, NX, NY, self.omega[min(len(self.levels), 15)], True))
        self.inv = self._coarse_inverse(self.levels[-1]) if coarsest_sweeps == 0 else None

    @staticmethod
    def _coarse_inverse(L):
        """Dense FP32 inverse of the coarsest operator by in-place Gauss-Jordan
        without pivoting (k_mg_coarse_inverse); None when a pivot is not positive."""
        f = np.float32
        c, NX, NY = L["c"], L["NX"], L["NY"]
        n = NX * NY
        cf = c.reshape(5, -1)
        A = np.zeros((n, n), dtype=f)
        for k in range(n):
            w, e, no, so = cf[1, k], cf[2, k], cf[3, k], cf[4, k]
            d = f(cf[0, k] - f(f(f(w + e) + no) + so)) if L["lap"] else cf[0, k]
            if w == 0 and e == 0 and no == 0 and so == 0 and d == 0:
                d = f(1)
            A[k, k] = d
            j = k % NY
            if k >= NY: A[k, k - NY] = w
            if k + NY < n: A[k, k + NY] = e
            if j + 1 < NY: A[k, k + 1] = no
            if j >= 1: A[k, k - 1] = so
        for p in range(n):
            piv = A[p, p]
            if not (piv > 0) or not np.isfinite(piv):
                return None
            ip = f(1) / piv
            col = A[:, p].copy()
            A[p, :] = A[p, :] * ip
            A[p, p] = ip
            rows = np.arange(n) != p
            A[rows, :] = (A[rows, :] - np.outer(col[rows], A[p, :])).astype(f)
            A[rows, p] = (-col[rows] * ip).astype(f)
        return A

    @staticmethod
    def _level(c, NX, NY, omega, lap):
        linked = (c[1] != 0) | (c[2] != 0) | (c[3] != 0) | (c[4] != 0)
        d = (c[0] - (c[1] + c[2] + c[3] + c[4])).astype(np.float32) if lap else c[0]
        with np.errstate(divide="ignore"):
            winv = np.where(d == 0, np.float32(0), np.where(linked, omega / d, np.float32(1) / d))
        return dict(c=c, NX=NX, NY=NY, iso=~linked, winv=winv.astype(np.float32), lap=lap)

    @staticmethod
    def _coarsen(c, iso, NXf, NYf, NXc, NYc, lapf):
        """Galerkin coarse operator in Laplacian form [rs, aW, aE, aN, aS].

        The four children of an aggregate are visited in the order
        (0,0), (0,1), (1,0), (1,1) and each child's links in the order W, E,
        N, S, every sum rounded to FP32 as it is formed (the order of
        k_mg_coarsen); absent or isolated children contribute exact zeros."""
        f = np.float32
        # fine arrays padded to (2 NXc, 2 NYc); padded cells count as isolated
        cp = np.zeros((5, 2 * NXc, 2 * NYc), dtype=f)
        cp[:, :NXf, :NYf] = c
        isop = np.ones((2 * NXc + 2, 2 * NYc + 2), dtype=bool)   # one-cell isolated frame
        isop[1:NXf + 1, 1:NYf + 1] = iso
        rs, aW, aE, aN, aS = (np.zeros((NXc, NYc), dtype=f) for _ in range(5))
        for di in (0, 1):
            for dj in (0, 1):
                sl = (slice(di, 2 * NXc, 2), slice(dj, 2 * NYc, 2))
                w, e, n, s_ = (cp[q][sl] for q in (1, 2, 3, 4))
                me = ~isop[1 + di:2 * NXc + 1:2, 1 + dj:2 * NYc + 1:2]
                isoW = isop[di:2 * NXc:2, 1 + dj:2 * NYc + 1:2]
                isoE = isop[2 + di:2 * NXc + 2:2, 1 + dj:2 * NYc + 1:2]
                isoN = isop[1 + di:2 * NXc + 1:2, 2 + dj:2 * NYc + 2:2]
                isoS = isop[1 + di:2 * NXc + 1:2, dj:2 * NYc:2]
                r = cp[0][sl].copy() if lapf else (cp[0][sl] + (((w + e) + n) + s_)).astype(f)
                z = f(0)
                r = (r - np.where(isoW, w, z)).astype(f)
                r = (r - np.where(isoE, e, z)).astype(f)
                r = (r - np.where(isoN, n, z)).astype(f)
                r = (r - np.where(isoS, s_, z)).astype(f)
                if di == 0:
                    aW = (aW + np.where(me & ~isoW, w, z)).astype(f)
                else:
                    aE = (aE + np.where(me & ~isoE, e, z)).astype(f)
                if dj == 1:
                    aN = (aN + np.where(me & ~isoN, n, z)).astype(f)
                else:
                    aS = (aS + np.where(me & ~isoS, s_, z)).astype(f)
                rs = (rs + np.where(me, r, z)).astype(f)
        return np.stack([rs, aW, aE, aN, aS]).astype(f)

    @staticmethod
    def _Ax(L, x):
        c = L["c"]
        xw = np.zeros_like(x); xe = np.zeros_like(x); xn = np.zeros_like(x); xs = np.zeros_like(x)
        xw[1:, :] = x[:-1, :]; xe[:-1, :] = x[1:, :]; xn[:, :-1] = x[:, 1:]; xs[:, 1:] = x[:, :-1]
        if L["lap"]:
            return c[0] * x + c[1] * (xw - x) + c[2] * (xe - x) + c[3] * (xn - x) + c[4] * (xs - x)
        return c[0] * x + c[1] * xw + c[2] * xe + c[3] * xn + c[4] * xs

    def _rb(self, L, b, x, color):
        ii, jj = np.meshgrid(np.arange(L["NX"]), np.arange(L["NY"]), indexing="ij")
        m = ((ii + jj) & 1) == color
        r = b - self._Ax(L, x)
        x[m] = (x + L["winv"] * r)[m]

    def apply(self, r):
        r = np.asarray(r, dtype=np.float32)
        L0 = self.levels[0]
        bs = [r.reshape(L0["NX"], L0["NY"])]
        xs = []
        nlev = len(self.levels)
        for l, L in enumerate(self.levels):
            b = bs[l]
            if l == nlev - 1:
                if self.sweeps == 0 and self.inv is not None:
                    x = (self.inv @ b.reshape(-1)).astype(np.float32).reshape(b.shape)
                else:
                    x = L["winv"] * b
                    for _ in range(self.sweeps if self.sweeps > 0 else 64):
                        x = x + L["winv"] * (b - self._Ax(L, x))
                xs.append(x)
                break
            ii, jj = np.meshgrid(np.arange(L["NX"]), np.arange(L["NY"]), indexing="ij")
            x = np.where(((ii + jj) & 1) == 0, L["winv"] * b, np.float32(0)).astype(np.float32)
            self._rb(L, b, x, 1)
            for _ in range(1, self.nu_pre if l == 0 else self.nu_coarse):
                self._rb(L, b, x, 0); self._rb(L, b, x, 1)
            xs.append(x)
            res = np.where(L["iso"], np.float32(0), b - self._Ax(L, x))
            Lc = self.levels[l + 1]
            pad = np.zeros((2 * Lc["NX"], 2 * Lc["NY"]), dtype=np.float32)
            pad[:L["NX"], :L["NY"]] = res
            bs.append(pad.reshape(Lc["NX"], 2, Lc["NY"], 2).sum(axis=(1, 3)).astype(np.float32))
        for l in range(nlev - 2, -1, -1):
            L = self.levels[l]
            xc = xs[l + 1]
            up = np.repeat(np.repeat(xc, 2, axis=0), 2, axis=1)[:L["NX"], :L["NY"]]
            xs[l] = np.where(L["iso"], xs[l], xs[l] + self.alpha[min(l, 15)] * up).astype(np.float32)
            for _ in range(self.nu_post if l == 0 else self.nu_coarse):
                self._rb(L, bs[l], xs[l], 1); self._rb(L, bs[l], xs[l], 0)
        return xs[0].reshape(-1)


def post_process_field(u, v, p, pcor, udiv, dx, dy):
    """post_process_field, karman_taichi.py:545-583, and scale_field, :573-583
    (whose min / max start from 1e9 / 0).  Returns u_post, v_post, udiv (interior
    updated, rest as given), minmax [5][2] for (u_post, v_post, p, pcor, udiv)
    and the five 3x-upsampled canvases scaled to [0, 1]."""
    u, v, p, pcor = (np.asarray(a, dtype=np.float64) for a in (u, v, p, pcor))
    udiv = np.array(udiv, dtype=np.float64, copy=True)
    NX, NY = p.shape
    nx, ny = NX - 2, NY - 2
    u_post = 0.5 * (u[:NX, :] + u[1:NX + 1, :])
    v_post = 0.5 * (v[:, :NY] + v[:, 1:NY + 1])
    udiv[1:nx + 1, 1:ny + 1] = ((u[1:nx + 1, 1:ny + 1] - u[2:nx + 2, 1:ny + 1]) * dy
                                + (v[1:nx + 1, 2:ny + 2] - v[1:nx + 1, 1:ny + 1]) * dx)
    fields = (u_post, v_post, p, pcor, udiv)
    minmax = np.array([[min(1.0e9, f.min()), max(0.0, f.max())] for f in fields])
    disp = np.stack([np.repeat(np.repeat((f - lo) / (hi - lo + 1.0e-9), 3, axis=0), 3, axis=1)
                     for f, (lo, hi) in zip(fields, minmax)])
    return u_post, v_post, udiv, minmax, disp


def pcorr_random_system(N=1024, seed=0, blocked=0.05):
    """A seeded standalone pressure-correction system on an N x N grid (padded
    [N+2][N+2], standard form, FP64): face coefficients 1/aP_face with aP_face
    log-uniform in [1, 10]; square blocked blobs (side 4-16) covering about
    `blocked` of the cells, whose rows are identities and whose links are
    removed; p' pinned to zero at the first fluid cell as bicgsimp.py:146-151
    pins (1, 1); right-hand side the divergence of a seeded Gaussian face
    velocity smoothed by a 5 x 5 box filter, mean removed over the fluid.
    Returns (coef [5][N+2][N+2], b [N+2][N+2])."""
    rng = np.random.default_rng(seed)
    NX = NY = N + 2
    solid = np.zeros((NX, NY), dtype=bool)
    target = blocked * N * N
    while solid[1:-1, 1:-1].sum() < target:
        s = int(rng.integers(4, 17))
        i0, j0 = int(rng.integers(1, N - s + 2)), int(rng.integers(1, N - s + 2))
        solid[i0:i0 + s, j0:j0 + s] = True
    fluid = np.zeros((NX, NY), dtype=bool)
    fluid[1:-1, 1:-1] = ~solid[1:-1, 1:-1]
    ae = np.zeros((NX, NY))    # link between (i, j) and (i+1, j)
    an = np.zeros((NX, NY))    # link between (i, j) and (i, j+1)
    ae[1:N, 1:N + 1] = 1.0 / np.exp(rng.uniform(0.0, np.log(10.0), (N - 1, N)))
    an[1:N + 1, 1:N] = 1.0 / np.exp(rng.uniform(0.0, np.log(10.0), (N, N - 1)))
    ae[:-1] *= fluid[:-1] & fluid[1:]
    an[:, :-1] *= fluid[:, :-1] & fluid[:, 1:]
    pin = tuple(np.argwhere(fluid)[0])
    c = np.zeros((5, NX, NY))
    c[2, :-1] = -ae[:-1]            # aE of (i, j)
    c[1, 1:] = -ae[:-1]             # aW of (i+1, j)
    c[3, :, :-1] = -an[:, :-1]      # aN of (i, j)
    c[4, :, 1:] = -an[:, :-1]       # aS of (i, j+1)
    c[0] = -(c[1] + c[2] + c[3] + c[4])
    for q in range(1, 5):
        c[q][~fluid] = 0.0
    c[0][~fluid] = 0.0
    c[0][solid] = 1.0
    c[:, pin[0], pin[1]] = 0.0
    c[0, pin[0], pin[1]] = 1.0

    def box5(a):
        p = np.pad(a, 2, mode="edge")
        out = np.zeros_like(a)
        for di in range(5):
            for dj in range(5):
                out += p[di:di + a.shape[0], dj:dj + a.shape[1]]
        return out / 25.0
    u = box5(rng.standard_normal((NX + 1, NY)))
    v = box5(rng.standard_normal((NX, NY + 1)))
    b = (u[:-1] - u[1:]) + (v[:, :-1] - v[:, 1:])
    b[~fluid] = 0.0
    b[pin] = 0.0
    m = fluid.copy()
    m[pin] = False
    b[m] -= b[m].mean()
    return c, b


def lex_sweep(coef, b, x, box, omega=1.0, relax=True, x_mid=None):
    """One in-place lexicographic relaxation sweep over the box (i0, i1, j0, j1),
    i outer and j inner, as jacosimp.py:210-238 runs it in Python scope: each
    cell reads its west and south neighbours already updated.  The cells of an
    anti-diagonal i + j = d depend only on diagonal d - 1, so the sweep is
    evaluated diagonal by diagonal with NumPy, each cell in the reference's
    operation order.  coef: [5][NX][NY]."""
    i0, i1, j0, j1 = box
    ni, nj = i1 - i0, j1 - j0
    for d in range(ni + nj - 1):
        a = np.arange(max(0, d - nj + 1), min(ni - 1, d) + 1)
        i, j = i0 + a, j0 + (d - a)
        xm = ((((-coef[1, i, j] * x[i - 1, j]) - coef[2, i, j] * x[i + 1, j]) - coef[3, i, j] * x[i, j + 1])
              - coef[4, i, j] * x[i, j - 1] + b[i, j]) / coef[0, i, j]
        if relax:
            if x_mid is not None:
                x_mid[i, j] = xm
            x[i, j] = (1.0 - omega) * x[i, j] + omega * xm
        else:
            x[i, j] = xm
    return x


class JacoSimpleOracle(SimpleOracle):
    """Restatement of jacosimp.py:9-272: simple.py's assembly (jacosimp.py's
    compute_coef_u/v/p and set_bc are simple.py's), lexicographic relaxation
    sweeps instead of solves, constants of jacosimp.py:18-25."""

    def __init__(self, lx, ly, nx, ny):
        super().__init__(lx, ly, nx, ny)
        self.dt = 100000.0
        self.alpha_p = 0.01
        self.alpha_u = 0.01
        self.alpha = 0.1

    def jaco_momentum(self):  # jacosimp.py:210-228
        nx, ny = self.nx, self.ny
        self.compute_coef_u(); self.compute_coef_v(); self.set_bc()
        lex_sweep(self.coef_u, self.b_u, self.u, (2, nx + 1, 1, ny + 1), self.alpha_u, True, self.u_mid)
        lex_sweep(self.coef_v, self.b_v, self.v, (1, nx + 1, 2, ny + 1), self.alpha_u, True, self.v_mid)

    def jaco_pcorrection(self):  # jacosimp.py:230-238
        self.compute_coef_p()
        lex_sweep(self.coef_p, self.mdiv, self.pcor, (1, self.nx + 1, 1, self.ny + 1), 1.0, False)

    def update_pressure(self):  # jacosimp.py:194-198
        nx, ny = self.nx, self.ny
        self.p[1:nx + 1, 1:ny + 1] += self.alpha_p * self.pcor[1:nx + 1, 1:ny + 1]

    def jaco_update_velocity(self):  # jacosimp.py:200-208
        nx, ny, dx, dy = self.nx, self.ny, self.dx, self.dy
        pc = self.pcor
        I, J = slice(2, nx + 1), slice(1, ny + 1)
        self.u[I, J] += self.alpha * (pc[1:nx, J] - pc[I, J]) * dy / self.coef_u[0, I, J]
        I, J = slice(1, nx + 1), slice(2, ny + 1)
        self.v[I, J] += self.alpha * (pc[I, 1:ny] - pc[I, J]) * dx / self.coef_v[0, I, J]

    def jaco_step(self):  # one step of jacosimp.py:253-268
        self.jaco_momentum()
        self.jaco_pcorrection()
        self.update_pressure()
        self.jaco_update_velocity()
        self.compute_mdiv()


def jacobi_sweep(coef, b, x, S, omega=1.0, region=None):
    """One Jacobi sweep as kc_jacobi defines it (pressure_valid.py:192-233,
    debug/20210828_karman_taihi.py:375-393 with every cell reading the previous
    iterate): flat 5-point neighbours k -+ S, k -+ 1 (zero outside [0, n)).
    Returns (y, max |x_mid - x| over the region)."""
    c = np.asarray(coef, dtype=np.float64).reshape(5, -1)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    x = np.asarray(x, dtype=np.float64).reshape(-1)
    n = x.size
    NX = n // S
    i0, i1, j0, j1 = region if region is not None else (0, NX, 0, S)
    xw = np.zeros(n); xw[S:] = x[:-S]
    xe = np.zeros(n); xe[:-S] = x[S:]
    xn = np.zeros(n); xn[:-1] = x[1:]
    xs = np.zeros(n); xs[1:] = x[:-1]
    r = (((b - c[1] * xw) - c[2] * xe) - c[3] * xn) - c[4] * xs
    ii, jj = np.divmod(np.arange(n), S)
    inside = (ii >= i0) & (ii < i1) & (jj >= j0) & (jj < j1) & (c[0] != 0)
    xm = np.where(inside, r / np.where(c[0] != 0, c[0], 1.0), x)
    y = np.where(inside, (1.0 - omega) * x + omega * xm, x)
    d = np.abs(xm - x)[inside]
    return y, (float(d.max()) if d.size else 0.0)

def rbgs_sweeps(coef, b, x, sweeps, S):
    """Red-black Gauss-Seidel sweeps on the flat 5-point stencil (the
    Gauss-Seidel counterpart of pressure_valid.py:192-233's Jacobi solves):
    colour = parity of i + j of the [n/S][S] view; each sweep updates the red
    cells from the previous black values, then the black cells from the new
    red ones; rows with a zero diagonal keep their x.  coef: [5, n] standard
    form, b, x: [n] (float64).  Returns x and the residual norms of the
    iterate each sweep started from."""
    coef = np.asarray(coef, dtype=np.float64).reshape(5, -1)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    x = np.array(x, dtype=np.float64).reshape(-1)
    n = b.size
    k = np.arange(n)
    red = ((k // S + k % S) % 2) == 0
    d = coef[0]
    winv = np.where(d != 0.0, 1.0 / np.where(d != 0.0, d, 1.0), 0.0)

    def ax(x):   # links k -+ S (west, east) and k +- 1 (north, south); out of range: 0
        xs = np.concatenate(([0.0] * S, x, [0.0] * S))
        y = coef[0] * x + coef[1] * xs[0:n] + coef[2] * xs[2 * S:2 * S + n]
        xf = np.concatenate(([0.0], x, [0.0]))
        y = y + coef[3] * xf[2:n + 2] + coef[4] * xf[0:n]
        return y

    norms = []
    for _ in range(sweeps):
        r = b - ax(x)
        norms.append(float(np.sqrt((r * r).sum())))
        x = np.where(red, x + winv * r, x)
        r = b - ax(x)
        x = np.where(~red, x + winv * r, x)
    return x, norms
