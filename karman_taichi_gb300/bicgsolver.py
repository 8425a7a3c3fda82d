"""Drop-in for the reference's ``bicgsolver.BICGSolver`` (bicgsolver.py:5-135).

BiCGSTAB with ``M = I`` and a cold start (x = 0, r = r~ = b), stopping when
sqrt(rTr / r0Tr) < eps or rho == 0, capped at NX*NY iterations, exactly as
bicgsolver.py:88-135 -- but fused into three device passes per iteration
with the scalars kept on the GPU.  ``solve`` writes ``x`` in place and
returns a ``SolveInfo``.
"""
from __future__ import annotations

from .cgsolver import CGSolver
from .linalg import bicgstab


class BICGSolver(CGSolver):
    def solve(self, eps=1e-8, quiet=True, history_len=4096):
        hist = self._history_buf(history_len)
        info = bicgstab(self._A(), self.b, self.x, eps=eps, max_iter=self.steps, ws=self.ws, history=hist)
        self._record(info)
        if not quiet:
            print(f">>> BICG: {info.status_name} after {info.iters} iterations, relative residual {info.rel_res:e}")
        return info
