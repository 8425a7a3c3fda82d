"""Drop-in for the reference's ``jacosimp.SIMPLESolver`` (jacosimp.py:9-272).

The lid-driven cavity SIMPLE variant that relaxes the equations instead of
solving them: each step makes one in-place lexicographic sweep of the u and
v momentum equations (under-relaxed by alpha_u, jacosimp.py:210-228) and one
of the pressure correction (right-hand side mdiv, jacosimp.py:230-238), then
corrects p (alpha_p) and u, v (alpha), jacosimp.py:194-208.  The sweeps run
on the GPU as anti-diagonal wavefronts (``kc_lex_sweep``), which give the
serial sweep's values exactly; assembly, boundary folding, the mass source
and the corrections are the kernels of ``simple.SIMPLESolver`` (jacosimp.py's
compute_coef_u/v/p, set_bc and compute_mdiv are simple.py's).  Constants as
jacosimp.py:18-25: dt = 100000, alpha_p = alpha_u = 0.01, alpha = 0.1.
"""
from __future__ import annotations

from . import _lib as L
from . import simple
from .linalg import ptr


class SIMPLESolver(simple.SIMPLESolver):
    def __init__(self, lx, ly, nx, ny, device="cuda"):
        super().__init__(lx, ly, nx, ny, device=device)
        self.dt = 100000
        self.alpha_p = 0.01
        self.alpha_u = 0.01
        self.alpha = 0.1

    def _sweep(self, coef, b, x, x_mid, box, omega, relax):
        NX, NY = x.shape
        i0, i1, j0, j1 = box
        L.check(L.load().kc_lex_sweep(ptr(coef), NX * NY, 1, NX, NY, i0, i1, j0, j1, ptr(b), ptr(x), ptr(x_mid),
                                      float(omega), int(relax), self._s()), "kc_lex_sweep")

    def solve_momentum_eqn(self):
        """jacosimp.py:210-228: coefficients, boundary folding, then one under-relaxed
        lexicographic sweep of u over i in [2, nx], j in [1, ny] and of v over i in [1, nx],
        j in [2, ny]."""
        nx, ny = self.nx, self.ny
        self.compute_coef_u()
        self.compute_coef_v()
        self.set_bc()
        self._sweep(self.coef_u, self.b_u, self.u, self.u_mid, (2, nx + 1, 1, ny + 1), self.alpha_u, True)
        self._sweep(self.coef_v, self.b_v, self.v, self.v_mid, (1, nx + 1, 2, ny + 1), self.alpha_u, True)

    def solve_pcorrection_eqn(self):
        """jacosimp.py:230-238: p' coefficients and mdiv, then one lexicographic sweep of
        p' (right-hand side mdiv) over i in [1, nx], j in [1, ny]."""
        self.compute_coef_p()
        self._sweep(self.coef_p, self.mdiv, self.pcor, None, (1, self.nx + 1, 1, self.ny + 1), 1.0, False)

    def update_pressure(self):
        """jacosimp.py:194-198: p += alpha_p p'."""
        self._correct(0.0, self.alpha_p)

    def update_velocity(self):
        """jacosimp.py:200-208: u += alpha (p'_W - p') dy / aP, v likewise."""
        self._correct(self.alpha, 0.0)

    def solve(self, n_steps=60000, callback=None):
        """jacosimp.py:249-272 without the every-100-steps PNG/CSV output."""
        self.init()
        for step in range(n_steps):
            self.solve_momentum_eqn()
            self.solve_pcorrection_eqn()
            self.update_pressure()
            self.update_velocity()
            self.compute_mdiv()
            if callback:
                callback(step)
        return self
