"""Drop-in for the reference's ``simple.SIMPLESolver`` (simple.py:9-285).

Same constructor ``SIMPLESolver(lx, ly, nx, ny)``, constants (simple.py:16-25),
``bc`` dict (simple.py:39) and per-stage methods, with CUDA float64 tensors
for the fields.  Coefficients are SoA planes ``coef_*[5, NX, NY]`` (component
order aP, aW, aE, aN, aS as the reference's ``coef[i, j, 0..4]``).

The assembly kernel computes the coefficients with set_bc's boundary folding
fused in, so ``compute_coef_u`` / ``compute_coef_v`` assemble both systems
(including the folding), and ``set_bc`` writes the boundary velocities
(simple.py:181, 186, 192, 196).  Called in the reference's order
(compute_coef_u, compute_coef_v, set_bc) the resulting state is the same.

``bicgsimp=True`` selects the bicgsimp.py variant: east-wall fix
(bicgsimp.py:196), p' pinned at (1, 1) (bicgsimp.py:146-151), persistent
solvers (bicgsimp.py:260-262) and the max-residual returns of
compute_mdiv / update_velocity (bicgsimp.py:114-122, 212-225).
"""
from __future__ import annotations

import ctypes as C
import os

import torch

from . import _lib as L
from .bicgsolver import BICGSolver
from .cgsolver import CGSolver
from .linalg import ptr, stream_handle


class SIMPLESolver:
    def __init__(self, lx, ly, nx, ny, device="cuda", bicgsimp=False):
        self.lx, self.ly, self.nx, self.ny = lx, ly, nx, ny
        self.dx, self.dy = lx / nx, ly / ny
        self.rho, self.mu, self.dt = 1.00, 0.01, 10000
        self.real = torch.float64
        self.alpha_p = self.alpha_u = self.alpha_m = 0.001
        self.bicgsimp = bicgsimp
        if bicgsimp:
            self.dt, self.alpha_p, self.alpha_u, self.alpha_m = 1e12, 0.1, 0.8, 0.05
        self.device = torch.device(device)
        L.load()
        f = dict(dtype=torch.float64, device=self.device)
        z = torch.zeros
        self.u, self.v = z((nx + 3, ny + 2), **f), z((nx + 2, ny + 3), **f)
        self.u_mid, self.v_mid = z((nx + 3, ny + 2), **f), z((nx + 2, ny + 3), **f)
        self.u0, self.v0 = z((nx + 3, ny + 2), **f), z((nx + 2, ny + 3), **f)
        self.p, self.pcor, self.mdiv = z((nx + 2, ny + 2), **f), z((nx + 2, ny + 2), **f), z((nx + 2, ny + 2), **f)
        self.bc = {"w": [0.0, 0.0], "e": [0.0, 0.0], "n": [0.0, 0.0], "s": [0.0, 0.0]}
        self.ct = z((nx + 2, ny + 2), **f)   # unused by the reference as well (simple.py:40)
        self.coef_u, self.b_u = z((5, nx + 3, ny + 2), **f), z((nx + 3, ny + 2), **f)
        self.coef_v, self.b_v = z((5, nx + 2, ny + 3), **f), z((nx + 2, ny + 3), **f)
        self.coef_p, self.b_p = z((5, nx + 2, ny + 2), **f), z((nx + 2, ny + 2), **f)
        self._mass = z(2, **f)
        self._diff = z(1, **f)
        self._rws = torch.zeros(L.load().kc_reduce_ws_bytes(), dtype=torch.uint8, device=self.device)
        self._assembled = False
        self.u_momentum_solver = self.v_momentum_solver = self.p_correction_solver = None
        self.log = []

    # ---- helpers ------------------------------------------------------------
    def _phys(self):
        ph = L.KcPhys()
        ph.nx, ph.ny = self.nx, self.ny
        ph.mode = L.MODE_BICGSIMP if self.bicgsimp else L.MODE_SIMPLE
        ph.dx, ph.dy, ph.rho, ph.mu, ph.dt, ph.U = self.dx, self.dy, self.rho, self.mu, float(self.dt), 0.0
        for q, key in enumerate(("w", "e", "n", "s")):
            ph.bc[q][0], ph.bc[q][1] = float(self.bc[key][0]), float(self.bc[key][1])
        ph.alpha_m, ph.alpha_u, ph.alpha_p = self.alpha_m, self.alpha_u, self.alpha_p
        return ph

    def _s(self):
        return stream_handle(self.device)

    # ---- assembly (simple.py:77-110, 172-216) --------------------------------
    def _assemble(self):
        L.check(L.load().kc_assemble_momentum(C.byref(self._phys()), ptr(self.u), ptr(self.v), ptr(self.p),
                                              ptr(self.u0), ptr(self.v0), None, ptr(self.coef_u), ptr(self.b_u),
                                              ptr(self.coef_v), ptr(self.b_v), None, None, None, None, self._s()),
                "kc_assemble_momentum")
        self._assembled = True

    def compute_coef_u(self):
        self._assemble()

    def compute_coef_v(self):
        if not self._assembled:
            self._assemble()

    def set_bc(self):
        L.check(L.load().kc_apply_bc_values(C.byref(self._phys()), ptr(self.u), ptr(self.v), self._s()),
                "kc_apply_bc_values")
        self._assembled = False

    def compute_mdiv(self):
        """simple.py:137-141; returns max|mdiv| as bicgsimp.py:114-122 does."""
        L.check(L.load().kc_mass_residual(C.byref(self._phys()), ptr(self.u), ptr(self.v), None, ptr(self.mdiv),
                                          ptr(self._mass), ptr(self._rws), self._s()), "kc_mass_residual")
        return float(self._mass[0].item())

    def compute_coef_p(self):
        """simple.py:143-170 (bicgsimp.py:124-151 pins (1, 1))."""
        L.check(L.load().kc_assemble_pcorr(C.byref(self._phys()), ptr(self.u), ptr(self.v), ptr(self.coef_u),
                                           ptr(self.coef_v), None, ptr(self.coef_p), ptr(self.b_p), None, None,
                                           ptr(self.mdiv), ptr(self._mass), ptr(self._rws), self._s()),
                "kc_assemble_pcorr")

    # ---- corrections (simple.py:218-238) -------------------------------------
    def _correct(self, alpha_u, alpha_p):
        ph = self._phys()
        ph.alpha_u, ph.alpha_p = alpha_u, alpha_p
        L.check(L.load().kc_correct(C.byref(ph), ptr(self.pcor), ptr(self.coef_u), ptr(self.coef_v), None,
                                    ptr(self.u), ptr(self.v), ptr(self.p), None, ptr(self._rws), self._s()),
                "kc_correct")

    def correct_pressure(self):
        self._correct(0.0, self.alpha_p)

    def correct_velocity(self):
        self._correct(self.alpha_u, 0.0)

    def update_velocity(self):
        """u = alpha_m u_mid + (1 - alpha_m) u; returns the bicgsimp.py:225 residual."""
        L.check(L.load().kc_relax_velocity(C.byref(self._phys()), None, ptr(self.u_mid), ptr(self.v_mid),
                                           ptr(self.u), ptr(self.v), ptr(self._diff), ptr(self._rws), self._s()),
                "kc_relax_velocity")
        return float(self._diff[0].item())

    # ---- stages (simple.py:241-285) -------------------------------------------
    def solve_momentum_eqn(self, n_iter, eps=None):
        res = 0.0
        for _ in range(n_iter):
            self.compute_coef_u()
            self.compute_coef_v()
            self.set_bc()
            if self.bicgsimp:
                if self.u_momentum_solver is None:
                    self.u_momentum_solver = BICGSolver(self.coef_u, self.b_u, self.u_mid)
                    self.v_momentum_solver = BICGSolver(self.coef_v, self.b_v, self.v_mid)
                iu = self.u_momentum_solver.solve(eps=1e-4 if eps is None else eps, quiet=True)
                iv = self.v_momentum_solver.solve(eps=1e-4 if eps is None else eps, quiet=True)
            else:
                iu = BICGSolver(self.coef_u, self.b_u, self.u_mid).solve(eps=1e-1 if eps is None else eps)
                iv = BICGSolver(self.coef_v, self.b_v, self.v_mid).solve(eps=1e-1 if eps is None else eps)
            res = self.update_velocity()
            self.log.append(("momentum", iu.iters, iv.iters))
        return res

    bicg_solve_momentum_eqn = solve_momentum_eqn

    def solve_pcorrection_eqn(self, eps=None):
        self.compute_coef_p()
        if self.bicgsimp:
            if self.p_correction_solver is None:
                self.p_correction_solver = CGSolver(self.coef_p, self.b_p, self.pcor)
            info = self.p_correction_solver.solve(1e-8 if eps is None else eps, quiet=True)
        else:
            info = CGSolver(self.coef_p, self.b_p, self.pcor).solve(eps=1e-2 if eps is None else eps)
        self.log.append(("pcorr", info.iters))
        return info

    def bicg_solve_pcorrection_eqn(self, eps):
        return self.solve_pcorrection_eqn(eps)

    # ---- Jacobi paths (pressure_valid.py:192-233) ----------------------------------
    def jacobian_solve_u(self) -> float:
        """One under-relaxed Jacobi sweep of the u equations on i in [2, nx], j in [1, ny]
        (pressure_valid.py:192-206); returns max |u_mid - u|."""
        from .linalg import Stencil, jacobi
        nx, ny = self.nx, self.ny
        if getattr(self, "_jac_u", None) is None:
            self._jac_u = torch.empty_like(self.u)
        d = jacobi(Stencil(self.coef_u), self.b_u, self.u, self._jac_u, omega=self.alpha_u,
                   region=(2, nx + 1, 1, ny + 1))
        self.u.copy_(self._jac_u)
        return float(d.item())

    def jacob_solve_momentum_eqn(self, n_iter):
        """pressure_valid.py:208-214."""
        self.compute_coef_u()
        self.compute_coef_v()
        self.set_bc()
        return [self.jacobian_solve_u() for _ in range(n_iter)]

    def jacobian_solve_p(self) -> float:
        """One Jacobi sweep of the p' equations (right-hand side mdiv) on i in [1, nx], j in
        [1, ny] (pressure_valid.py:221-233); returns max |pcor_mid - pcor|."""
        from .linalg import Stencil, jacobi
        nx, ny = self.nx, self.ny
        if getattr(self, "_jac_p", None) is None:
            self._jac_p = torch.empty_like(self.pcor)
        d = jacobi(Stencil(self.coef_p), self.mdiv, self.pcor, self._jac_p, omega=1.0,
                   region=(1, nx + 1, 1, ny + 1))
        self.pcor.copy_(self._jac_p)
        return float(d.item())

    def jacob_solve_pcorrection_eqn(self, eps, max_iter=100000):
        """pressure_valid.py:235-239, with an iteration cap."""
        res, k = 1.0, 0
        while res > eps and k < max_iter:
            res = self.jacobian_solve_p()
            k += 1
        return res, k

    def dump_matrix(self, step, msg, directory="log"):
        """simple.py:51-54: u, v, p, mdiv, pcor to {directory}/{step:06}-{name}-{msg}.csv."""
        from .fields import savetxt
        os.makedirs(directory, exist_ok=True)
        for name, val in {"u": self.u, "v": self.v, "p": self.p, "mdiv": self.mdiv, "pcor": self.pcor}.items():
            savetxt(os.path.join(directory, f"{step:06}-{name}-{msg}.csv"), val)

    def dump_coef(self, step, msg, directory="log"):
        """simple.py:56-75: the five coefficient planes and b of u, v, p (file names as the reference's,
        including the space in 'bu -', 'bv -', 'bp -')."""
        from .fields import savetxt
        os.makedirs(directory, exist_ok=True)
        for tag, coef, b in (("u", self.coef_u, self.b_u), ("v", self.coef_v, self.b_v), ("p", self.coef_p, self.b_p)):
            for k, comp in enumerate(("ap", "aw", "ae", "an", "as")):
                savetxt(os.path.join(directory, f"{step:06}-{comp}{tag}-{msg}.csv"), coef[k])
            savetxt(os.path.join(directory, f"{step:06}-b{tag} -{msg}.csv"), b)

    def init(self):
        """simple.py:257-264 (bicgsimp.py:246-256 also zeroes u0, v0, pcor)."""
        self.u.zero_(); self.v.zero_(); self.p.zero_()
        if self.bicgsimp:
            self.u0.zero_(); self.v0.zero_(); self.pcor.zero_()

    def solve(self, n_steps=2000, callback=None):
        """simple.py:266-285 without the CSV/PNG dumps; bicgsimp.py:311-328
        adds the momentum < 1e-2 and continuity < 1e-6 stop."""
        self.init()
        for step in range(n_steps):
            mres = self.solve_momentum_eqn(1)
            self.compute_mdiv()
            self.solve_pcorrection_eqn()
            self.correct_pressure()
            self.correct_velocity()
            cres = self.compute_mdiv()
            if callback:
                callback(step, mres, cres)
            if self.bicgsimp and mres < 1e-2 and cres < 1e-6:
                break
        return self
