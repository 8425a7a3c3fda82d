"""Torch-facing wrappers around the stencil solvers of libkarman_gb300.

Tensors stay on the GPU; every call passes raw device pointers and the
current torch stream through the C ABI.  Nothing here computes on the host:
if the library is missing, ``KcLibraryMissing`` is raised.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from . import _lib as L


@dataclass
class SolveInfo:
    """Outcome of a solve (the reference returns None and prints instead)."""
    status: int
    iters: int
    rel_res: float
    r0: float
    refinements: int = 0

    @property
    def ok(self) -> bool:
        return self.status == L.OK

    @property
    def status_name(self) -> str:
        return L.status_name(self.status)


def ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def stream_handle(device=None):
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def dtype_code(t: torch.Tensor) -> int:
    if t.dtype == torch.float64:
        return L.F64
    if t.dtype == torch.float32:
        return L.F32
    raise TypeError(f"unsupported dtype {t.dtype}: expected float64 or float32")


def require_cuda(*ts):
    for t in ts:
        if t is None:
            continue
        if not t.is_cuda:
            raise ValueError("karman_taichi_gb300 operates on CUDA tensors only (no CPU fallback)")
        if not t.is_contiguous():
            raise ValueError("tensor must be contiguous")


class Stencil:
    """5-point stencil operator ``A`` on ``n`` unknowns with far stride ``S``.

    ``coef`` is either SoA planes ``[5, NX, NY]`` / ``[5, n]`` or the
    reference's array-of-structs ``[NX, NY, 5]`` (simple.py:42-47), read in
    place without conversion (component stride 1, element stride 5).
    Component order: aP, aW (k-S), aE (k+S), aN (k+1), aS (k-1).
    """

    def __init__(self, coef: torch.Tensor, stride: int | None = None, layout: str | None = None,
                 form: int = L.FORM_STANDARD):
        require_cuda(coef)
        self.form = int(form)
        if layout is None:
            layout = "aos" if (coef.dim() == 3 and coef.shape[-1] == 5 and coef.shape[0] != 5) else "soa"
        self.coef, self.layout = coef, layout
        if layout == "aos":
            NX, NY = coef.shape[0], coef.shape[1]
            self.n, self.cs, self.es = NX * NY, 1, 5
            self.stride = NY if stride is None else stride
            self.shape = (NX, NY)
        else:
            if coef.shape[0] != 5:
                raise ValueError("SoA coefficients must have 5 leading planes")
            self.n = coef[0].numel()
            self.cs, self.es = self.n, 1
            if stride is None:
                if coef.dim() != 3:
                    raise ValueError("stride required for flat [5, n] coefficients")
                stride = coef.shape[2]
            self.stride = stride
            self.shape = tuple(coef.shape[1:])
        self.dtype = dtype_code(coef)
        self._sys = L.KcSystem(self.n, self.cs, self.es, coef.data_ptr(), int(self.stride), self.dtype, self.form)

    @property
    def system(self) -> L.KcSystem:
        return self._sys

    @property
    def device(self):
        return self.coef.device


class Workspace:
    """Grow-only device scratch buffer (zero-filled on allocation)."""

    def __init__(self, device=None):
        self.device = device
        self.buf = None

    def get(self, nbytes: int) -> torch.Tensor:
        if self.buf is None or self.buf.numel() < nbytes:
            self.buf = torch.zeros(max(int(nbytes), 256), dtype=torch.uint8, device=self.device)
        return self.buf


def spmv(A: Stencil, x: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """y = A x (bicgsolver.py:65-76)."""
    require_cuda(x)
    if out is None:
        out = torch.empty_like(x)
    L.check(L.load().kc_spmv(C.byref(A.system), ptr(x), ptr(out), stream_handle(x.device)), "kc_spmv")
    return out


_jac_ws = {}


def jacobi(A: Stencil, b: torch.Tensor, x: torch.Tensor, y: torch.Tensor, *, omega=1.0, region=None,
           max_diff: torch.Tensor | None = None) -> torch.Tensor:
    """One Jacobi sweep y = (1 - omega) x + omega (b - sum_nb a_nb x_nb) / aP on
    region = (i0, i1, j0, j1) of the [n/stride][stride] view (pressure_valid.py:
    192-233, debug/20210828_karman_taihi.py:375-393); returns max |x_mid - x|
    as a 1-element device tensor."""
    require_cuda(b, x, y)
    dev = b.device
    lib = L.load()
    ws = _jac_ws.get(dev)
    if ws is None:
        ws = _jac_ws[dev] = torch.zeros(lib.kc_jacobi_ws_bytes(), dtype=torch.uint8, device=dev)
    out = max_diff if max_diff is not None else torch.empty(1, dtype=torch.float64, device=dev)
    i0, i1, j0, j1 = region if region is not None else (0, A.n // A.stride, 0, A.stride)
    L.check(lib.kc_jacobi(C.byref(A.system), ptr(b), ptr(x), ptr(y), float(omega), int(i0), int(i1), int(j0),
                          int(j1), ptr(out), ptr(ws), ws.numel(), stream_handle(dev)), "kc_jacobi")
    return out


_dot_ws = {}


def dot_device(p: torch.Tensor, q: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """FP64 sum(p*q) into a 1-element device tensor (no host sync)."""
    require_cuda(p, q)
    if p.numel() != q.numel() or p.dtype != q.dtype:
        raise ValueError("dot: shape/dtype mismatch")
    dev = p.device
    lib = L.load()
    ws = _dot_ws.get(dev)
    if ws is None:
        ws = torch.zeros(lib.kc_dot_ws_bytes(p.numel()), dtype=torch.uint8, device=dev)
        _dot_ws[dev] = ws
    if out is None:
        out = torch.empty(1, dtype=torch.float64, device=dev)
    L.check(lib.kc_dot(dtype_code(p), p.numel(), ptr(p), ptr(q), ptr(out), ptr(ws), ws.numel(),
                       stream_handle(dev)), "kc_dot")
    return out


def dot(p: torch.Tensor, q: torch.Tensor) -> float:
    """CGSolver.reduce (cgsolver.py:49-54): returns a Python float (host sync)."""
    return float(dot_device(p, q).item())


def _opts(eps, max_iter, x0, precond, omega_break, rel_to, check_every=0, use_graph=True,
          history=None, persistent=True):
    o = L.KcSolveOpts()
    o.eps, o.max_iter, o.x0, o.precond = float(eps), int(max_iter), int(x0), int(precond)
    o.omega_break, o.rel_to, o.check_every, o.use_graph = int(omega_break), int(rel_to), int(check_every), int(use_graph)
    o.persistent = int(persistent)
    if history is not None:
        o.history, o.history_len = history.data_ptr(), history.numel()
    else:
        o.history, o.history_len = None, 0
    return o


def bicgstab(A: Stencil, b: torch.Tensor, x: torch.Tensor, *, eps=1e-8, max_iter=None, warm=False,
             M: torch.Tensor | None = None, omega_break=False, rel_to_b=False, ws: Workspace | None = None,
             history: torch.Tensor | None = None, check_every=0, use_graph=True, persistent=True) -> SolveInfo:
    """BiCGSTAB on the device (bicgsolver.py:88-135; karman_taichi.py:342-456).

    ``persistent=True`` runs the whole solve as one cooperative launch;
    otherwise each iteration is three launches (optionally graph-captured)."""
    require_cuda(b, x, M)
    if b.numel() != A.n or x.numel() != A.n:
        raise ValueError(f"b/x have {b.numel()}/{x.numel()} elements, operator has {A.n}")
    if b.dtype != A.coef.dtype or x.dtype != A.coef.dtype:
        raise TypeError("b, x and the coefficients must share a dtype")
    lib = L.load()
    nbytes = lib.kc_bicgstab_ws_bytes(A.n, A.stride, A.dtype)
    buf = (ws or Workspace(b.device)).get(nbytes)
    o = _opts(eps, A.n if max_iter is None else max_iter, L.X0_WARM if warm else L.X0_ZERO,
              L.PRECOND_JACOBI if M is not None else L.PRECOND_NONE, omega_break,
              L.REL_B if rel_to_b else L.REL_R0, check_every, use_graph, history, persistent)
    info = L.KcSolveInfo()
    rc = lib.kc_bicgstab(C.byref(A.system), ptr(b), ptr(x), ptr(M), ptr(buf), buf.numel(), C.byref(o),
                         C.byref(info), stream_handle(b.device))
    L.check(rc, "kc_bicgstab")
    return SolveInfo(info.status, info.iters, info.rel_res, info.r0)


def cg(A: Stencil, b: torch.Tensor, x: torch.Tensor, *, eps=1e-8, max_iter=None, ws: Workspace | None = None,
       history: torch.Tensor | None = None, check_every=0, use_graph=True, persistent=True) -> SolveInfo:
    """Conjugate gradients on the device (cgsolver.py:83-114)."""
    require_cuda(b, x)
    if b.numel() != A.n or x.numel() != A.n:
        raise ValueError("b/x size does not match the operator")
    lib = L.load()
    nbytes = lib.kc_cg_ws_bytes(A.n, A.stride, A.dtype)
    buf = (ws or Workspace(b.device)).get(nbytes)
    o = _opts(eps, A.n if max_iter is None else max_iter, L.X0_ZERO, L.PRECOND_NONE, 0, L.REL_R0,
              check_every, use_graph, history, persistent)
    info = L.KcSolveInfo()
    rc = lib.kc_cg(C.byref(A.system), ptr(b), ptr(x), ptr(buf), buf.numel(), C.byref(o), C.byref(info),
                   stream_handle(b.device))
    L.check(rc, "kc_cg")
    return SolveInfo(info.status, info.iters, info.rel_res, info.r0)


def rbgs(A: Stencil, b: torch.Tensor, x: torch.Tensor, *, eps=1e-8, max_iter=200, warm=True, rel_to_b=True,
         ws: Workspace | None = None, history: torch.Tensor | None = None, check_every=0,
         use_graph=True) -> SolveInfo:
    """Red-black Gauss-Seidel solve of an FP64 system until ||b - A x|| < eps
    times ||b|| (``rel_to_b``) or ||b - A x0||; the Gauss-Seidel counterpart of
    the reference's Jacobi solves (pressure_valid.py:192-233).  ``max_iter``
    counts sweeps; ``warm`` starts from the given x."""
    require_cuda(b, x)
    if A.dtype != L.F64 or b.dtype != torch.float64 or x.dtype != torch.float64:
        raise TypeError("rbgs solves FP64 systems")
    if b.numel() != A.n or x.numel() != A.n:
        raise ValueError(f"b/x have {b.numel()}/{x.numel()} elements, operator has {A.n}")
    lib = L.load()
    buf = (ws or Workspace(b.device)).get(lib.kc_rbgs_ws_bytes(A.n, A.stride))
    o = _opts(eps, max_iter, L.X0_WARM if warm else L.X0_ZERO, L.PRECOND_NONE, 0,
              L.REL_B if rel_to_b else L.REL_R0, check_every, use_graph, history, False)
    info = L.KcSolveInfo()
    rc = lib.kc_rbgs(C.byref(A.system), ptr(b), ptr(x), ptr(buf), buf.numel(), C.byref(o), C.byref(info),
                     stream_handle(b.device))
    L.check(rc, "kc_rbgs")
    return SolveInfo(info.status, info.iters, info.rel_res, info.r0)


def bicgstab_refined(A64: Stencil, A32: Stencil, b: torch.Tensor, x: torch.Tensor, *, eps=1e-8,
                     eps_inner=1e-3, max_refine=30, max_iter=None, ws: Workspace | None = None,
                     use_graph=True, persistent=True, warm=False) -> SolveInfo:
    """FP64-residual iterative refinement around an FP32 BiCGSTAB with FP64
    inner products; stops when ||b - A64 x|| / ||b|| < eps.  ``warm`` starts
    from the given x instead of zero."""
    require_cuda(b, x)
    if A64.dtype != L.F64 or A32.dtype != L.F32:
        raise TypeError("bicgstab_refined needs an FP64 and an FP32 operator")
    lib = L.load()
    nbytes = lib.kc_refined_ws_bytes(A64.n, A64.stride)
    buf = (ws or Workspace(b.device)).get(nbytes)
    o = _opts(eps, 50 * A64.n if max_iter is None else max_iter, L.X0_WARM if warm else L.X0_ZERO,
              L.PRECOND_NONE, 0, L.REL_R0, 0, use_graph, None, persistent)
    info = L.KcSolveInfo()
    rc = lib.kc_bicgstab_refined(C.byref(A64.system), C.byref(A32.system), ptr(b), ptr(x), ptr(buf),
                                 buf.numel(), C.byref(o), float(eps_inner), int(max_refine), C.byref(info),
                                 stream_handle(b.device))
    L.check(rc, "kc_bicgstab_refined")
    return SolveInfo(info.status, info.iters, info.rel_res, info.r0, info.refinements)


def rbgs_refined(A64: Stencil, A32: Stencil, b: torch.Tensor, x: torch.Tensor, *, eps=1e-8,
                 eps_inner=1e-5, max_refine=30, max_iter=None, ws: Workspace | None = None,
                 use_graph=True, warm=False) -> SolveInfo:
    """FP64-residual iterative refinement around FP32 red-black Gauss-Seidel
    sweeps (``iters`` counts sweeps); stops when ||b - A64 x|| / ||b|| < eps.
    For diagonally dominant systems (the momentum rows).  Systems whose rows
    never link across their ends get 12 sweeps per refinement pass, two per
    launch; others one sweep per launch to ``eps_inner``."""
    require_cuda(b, x)
    if A64.dtype != L.F64 or A32.dtype != L.F32:
        raise TypeError("rbgs_refined needs an FP64 and an FP32 operator")
    lib = L.load()
    nbytes = lib.kc_refined_ws_bytes(A64.n, A64.stride)
    buf = (ws or Workspace(b.device)).get(nbytes)
    o = _opts(eps, 50 * A64.n if max_iter is None else max_iter, L.X0_WARM if warm else L.X0_ZERO,
              L.PRECOND_NONE, 0, L.REL_R0, 0, use_graph, None, False)
    info = L.KcSolveInfo()
    rc = lib.kc_rbgs_refined(C.byref(A64.system), C.byref(A32.system), ptr(b), ptr(x), ptr(buf), buf.numel(),
                             C.byref(o), float(eps_inner), int(max_refine), C.byref(info), stream_handle(b.device))
    L.check(rc, "kc_rbgs_refined")
    return SolveInfo(info.status, info.iters, info.rel_res, info.r0, info.refinements)


TAIL_CELLS = 1536   # default: levels of at most this many cells run in the multigrid tail block


class Multigrid:
    """Aggregation multigrid V-cycle (FP32) for a 2-D 5-point operator; the
    preconditioner of the mixed-precision pressure-correction solve.
    ``nu_pre`` / ``nu_post`` are the red-black sweeps on level 0, ``nu_coarse``
    those on every level below (1..3 in the fused two-launch cycle);
    ``omega`` / ``alpha`` are per-level smoother weights and coarse-correction
    scales (scalars broadcast to all levels; the last entry repeats);
    ``coarsest_sweeps=0`` solves the coarsest level (<= 128 cells) exactly.
    ``tail`` runs the levels of at most that many cells (True: 1536) in one
    single-block launch, ``big_cells`` picks the large tiles for the levels of
    at least that many cells; neither changes the result (the launch shapes
    the autotuner chooses between)."""

    def __init__(self, A32: Stencil, nu_pre=1, nu_post=1, coarsest_sweeps=0, omega=(1.0, 1.5), alpha=(1.9, 2.0),
                 max_levels=16, tail=True, big_cells=200000, nu_coarse=2):
        if A32.dtype != L.F32:
            raise TypeError("multigrid runs on FP32 coefficients")
        self.A = A32
        o = L.KcMgOpts()
        o.nu_pre, o.nu_post, o.coarsest_sweeps, o.max_levels = nu_pre, nu_post, coarsest_sweeps, max_levels
        o.nu_coarse = int(nu_coarse)
        o.tail = TAIL_CELLS if tail is True else int(tail)
        o.big_cells = int(big_cells)
        om = list(omega) if hasattr(omega, "__len__") else [omega] * 16
        al = list(alpha) if hasattr(alpha, "__len__") else [alpha] * 16
        for l in range(16):
            o.omega[l] = float(om[min(l, len(om) - 1)])
            o.alpha[l] = float(al[min(l, len(al) - 1)])
        self.opts = o
        lib = L.load()
        self.ws = torch.zeros(lib.kc_mg_ws_bytes(A32.n, A32.stride, C.byref(o)), dtype=torch.uint8,
                              device=A32.device)

    def setup(self):
        """(Re)build the coarse operators from the current fine coefficients."""
        L.check(L.load().kc_mg_setup(C.byref(self.A.system), ptr(self.ws), self.ws.numel(), C.byref(self.opts),
                                     stream_handle(self.A.device)), "kc_mg_setup")
        return self

    def apply(self, r: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        require_cuda(r)
        out = torch.empty_like(r) if out is None else out
        L.check(L.load().kc_mg_apply(C.byref(self.A.system), ptr(self.ws), C.byref(self.opts), ptr(r), ptr(out),
                                     stream_handle(r.device)), "kc_mg_apply")
        return out


def _mg_refined(fn, A64, A32, b, x, mg, eps, eps_inner, max_refine, max_iter, x0, ws, use_graph, check_every):
    require_cuda(b, x, x0)
    lib = L.load()
    buf = (ws or Workspace(b.device)).get(lib.kc_pbicgstab_ws_bytes(A64.n, A64.stride))
    o = _opts(eps, 50 * A64.n if max_iter is None else max_iter, L.X0_ZERO, L.PRECOND_NONE, 0, L.REL_B,
              check_every, use_graph, None, False)
    info = L.KcSolveInfo()
    rc = getattr(lib, fn)(C.byref(A64.system), C.byref(A32.system), ptr(b), ptr(x), ptr(x0), ptr(mg.ws),
                          C.byref(mg.opts), ptr(buf), buf.numel(), C.byref(o), float(eps_inner),
                          int(max_refine), C.byref(info), stream_handle(b.device))
    L.check(rc, fn)
    return SolveInfo(info.status, info.iters, info.rel_res, info.r0, info.refinements)


def pbicgstab_refined(A64: Stencil, A32: Stencil, b: torch.Tensor, x: torch.Tensor, mg: Multigrid, *, eps=1e-8,
                      eps_inner=1e-4, max_refine=30, max_iter=None, x0: torch.Tensor | None = None,
                      ws: Workspace | None = None, use_graph=True, check_every=4) -> SolveInfo:
    """Multigrid-preconditioned FP32 BiCGSTAB (FP64 iterate and inner products)
    inside FP64 iterative refinement; stops when ||b - A64 x|| / ||b|| < eps.
    ``x0`` is an optional FP64 initial guess (e.g. the learned network's
    prediction)."""
    return _mg_refined("kc_pbicgstab_refined", A64, A32, b, x, mg, eps, eps_inner, max_refine, max_iter, x0, ws,
                       use_graph, check_every)


def pcg_refined(A64: Stencil, A32: Stencil, b: torch.Tensor, x: torch.Tensor, mg: Multigrid, *, eps=1e-8,
                eps_inner=1e-4, max_refine=30, max_iter=None, x0: torch.Tensor | None = None,
                ws: Workspace | None = None, use_graph=True, check_every=4) -> SolveInfo:
    """Multigrid-preconditioned FP32 CG (symmetric systems) inside FP64
    iterative refinement; same contract as :func:`pbicgstab_refined`."""
    return _mg_refined("kc_pcg_refined", A64, A32, b, x, mg, eps, eps_inner, max_refine, max_iter, x0, ws,
                       use_graph, check_every)


def pcg_flexible(A64: Stencil, A32: Stencil, b: torch.Tensor, x: torch.Tensor, mg: Multigrid, *, net=None,
                 eps=1e-8, eps_inner=1e-4, max_outer=30, max_iter=None, warm=False, ws: Workspace | None = None,
                 inner_ws: Workspace | None = None, use_graph=True, check_every=4):
    """Flexible CG (FP64 outer vectors) whose first preconditioner application
    is the trained network's prediction (``net``: a ``kc_unet_net`` structure,
    see ``learned.UNet.native_net``; None for none) and every later one a
    multigrid-preconditioned FP32 CG pass (kc_pcg_flexible).  Returns
    (SolveInfo, KcFlexInfo); KC_STALL when two outer iterations in a row cut
    the residual by less than 10 %."""
    require_cuda(b, x)
    lib = L.load()
    buf = (ws or Workspace(b.device)).get(lib.kc_pcg_flexible_ws_bytes(A64.n))
    ibuf = (inner_ws or Workspace(b.device)).get(lib.kc_pbicgstab_ws_bytes(A64.n, A64.stride))
    o = _opts(eps, 50 * A64.n if max_iter is None else max_iter, L.X0_WARM if warm else L.X0_ZERO, L.PRECOND_NONE, 0,
              L.REL_B, check_every, use_graph, None, False)
    info, fi = L.KcSolveInfo(), L.KcFlexInfo()
    rc = lib.kc_pcg_flexible(C.byref(A64.system), C.byref(A32.system), ptr(b), ptr(x),
                             C.byref(net) if net is not None else None, ptr(mg.ws), C.byref(mg.opts), ptr(ibuf),
                             ibuf.numel(), ptr(buf), buf.numel(), C.byref(o), float(eps_inner), int(max_outer),
                             C.byref(info), C.byref(fi), stream_handle(b.device))
    L.check(rc, "kc_pcg_flexible")
    return SolveInfo(info.status, info.iters, info.rel_res, info.r0, info.refinements), fi
