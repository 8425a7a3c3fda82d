"""Drop-in for the reference's ``cgsolver.CGSolver`` (cgsolver.py:4-131).

Same constructor, attributes and methods, with ``torch.Tensor`` (CUDA,
float64 or float32) in place of ``ti.field``.  ``coef`` may be the
reference's ``[NX, NY, 5]`` array-of-structs (read in place, like the
reference holds a reference to the caller's field) or SoA planes
``[5, NX, NY]``.  ``solve`` writes ``x`` in place and, unlike the reference
(which returns None), returns a ``SolveInfo``.  The iteration runs on the
device; the residual history (cgsolver.py:88, 111) is recorded on the device
and copied back once per solve.
"""
from __future__ import annotations

import math

import torch

from . import _lib as L
from .linalg import Stencil, Workspace, cg, dot, spmv


class CGSolver:
    def __init__(self, coef: torch.Tensor, b: torch.Tensor, x: torch.Tensor):
        self.coef, self.b, self.x = coef, b, x
        self._layout = "aos" if (coef.dim() == 3 and coef.shape[-1] == 5 and coef.shape[0] != 5) else "soa"
        if self._layout == "aos":
            self.NX, self.NY = coef.shape[0], coef.shape[1]
        else:
            self.NX, self.NY = coef.shape[1], coef.shape[2]
        self.real = coef.dtype
        self.N_ext = 0
        self.steps = self.NX * self.NY          # cgsolver.py:14
        self.history = []                       # convergence history (cgsolver.py:15)
        self.ws = Workspace(coef.device)
        self._hist = None
        dev, dt = coef.device, coef.dtype
        self.Ap = torch.zeros((self.NX, self.NY), dtype=dt, device=dev)
        self.Ax = torch.zeros((self.NX, self.NY), dtype=dt, device=dev)
        self.r = torch.zeros((self.NX, self.NY), dtype=dt, device=dev)
        self.p = torch.zeros((self.NX, self.NY), dtype=dt, device=dev)

    # cgsolver.py:41-47 copies the given fields into the solver's own
    def update_coef(self, coef, b, x):
        self.coef.copy_(coef)
        self.b.copy_(b)
        self.x.copy_(x)

    def _A(self) -> Stencil:
        return Stencil(self.coef, layout=self._layout)

    def reduce(self, p, q) -> float:
        """FP64 sum of p*q over the whole field (cgsolver.py:49-54)."""
        return dot(p, q)

    def compute_Ap(self):
        spmv(self._A(), self.p, self.Ap)

    def compute_Ax(self):
        spmv(self._A(), self.x, self.Ax)

    def compute_residual(self):
        """r = b - A x (cgsolver.py:121-126)."""
        self.compute_Ax()
        torch.sub(self.b, self.Ax, out=self.r)

    def check_solution(self) -> float:
        self.compute_residual()
        return math.sqrt(self.reduce(self.r, self.r))

    def _history_buf(self, n):
        if self._hist is None or self._hist.numel() < n:
            self._hist = torch.zeros(n, dtype=torch.float64, device=self.coef.device)
        return self._hist

    def _record(self, info):
        h = self._hist[: info.iters + 1].cpu().tolist() if self._hist is not None else []
        self.history = [f"{v:e}\n" for v in h]

    def solve(self, eps=1e-8, quiet=True, history_len=4096):
        hist = self._history_buf(history_len)
        info = cg(self._A(), self.b, self.x, eps=eps, max_iter=self.steps, ws=self.ws, history=hist)
        self._record(info)
        if not quiet:
            print(f">>> CG: {info.status_name} after {info.iters} iterations, relative residual {info.rel_res:e}")
        return info

    def save_history(self, path="convergence.txt"):
        with open(path, "w") as f:
            for line in self.history:
                f.write(line)
