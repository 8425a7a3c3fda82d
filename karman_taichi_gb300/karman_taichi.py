"""Drop-in for the reference's ``karman_taichi.py`` driver (karman_taichi.py:1-683).

The reference keeps its fields in module globals; here they live in a
``KarmanState`` passed to functions of the same names.  The assembled sparse
matrices (pointer SNodes, karman_taichi.py:53-55, 82-84, 112-114) become flat
5-point planes with identical per-row values (see csrc/kc_karman.cu), and
``bicgstab`` is the device BiCGSTAB with right Jacobi, warm start and the
omega == 0 break (karman_taichi.py:342-456).
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np
import torch

from . import _lib as L
from . import geometry
from .config import KarmanConfig
from .linalg import Stencil, Workspace, bicgstab as _bicgstab, ptr, stream_handle


class KarmanState:
    def __init__(self, cfg: KarmanConfig = KarmanConfig(), device="cuda"):
        self.cfg = cfg
        self.device = torch.device(device)
        L.load()
        nx, ny = cfg.nx, cfg.ny
        f = dict(dtype=torch.float64, device=self.device)
        z = torch.zeros
        self.p, self.pcor, self.udiv = z((nx + 2, ny + 2), **f), z((nx + 2, ny + 2), **f), z((nx + 2, ny + 2), **f)
        self.u, self.u0 = z((nx + 3, ny + 2), **f), z((nx + 3, ny + 2), **f)
        self.v, self.v0 = z((nx + 2, ny + 3), **f), z((nx + 2, ny + 3), **f)
        self.ct = torch.zeros((nx + 2, ny + 2), dtype=torch.int32, device=self.device)
        self.nu, self.nv, self.np_ = (nx + 1) * ny, nx * (ny + 1), nx * ny
        self.Au, self.bu, self.xu, self.Mu = z((5, self.nu), **f), z(self.nu, **f), z(self.nu, **f), z(self.nu, **f)
        self.Av, self.bv, self.xv, self.Mv = z((5, self.nv), **f), z(self.nv, **f), z(self.nv, **f), z(self.nv, **f)
        self.Ap, self.bp, self.xp, self.Mp = z((5, self.np_), **f), z(self.np_, **f), z(self.np_, **f), z(self.np_, **f)
        self.ws = {k: Workspace(self.device) for k in "uvp"}
        self.rws = torch.zeros(L.load().kc_reduce_ws_bytes(), dtype=torch.uint8, device=self.device)
        self.pmax = z(1, **f)
        k = L.KcKarman()
        k.nx, k.ny, k.dx, k.dy = nx, ny, cfg.dx, cfg.dy
        k.rho, k.mu, k.dt, k.velo_rel, k.p_rel = cfg.rho, cfg.mu, cfg.dt, cfg.velo_rel, cfg.p_rel
        self.K = k
        self.solves = []

    def s(self):
        return stream_handle(self.device)


def init(st: KarmanState):
    """karman_taichi.py:130-154 (cell types built on the host, bit-exact)."""
    cfg = st.cfg
    st.p.copy_(torch.from_numpy(geometry.karman_initial_pressure(cfg.nx, cfg.ny)))
    st.u.zero_(); st.u0.zero_(); st.v.zero_(); st.v0.zero_()
    st.ct.copy_(torch.from_numpy(geometry.karman_cell_types(cfg.nx, cfg.ny, cfg.circle)))
    for t in (st.xu, st.xv, st.xp, st.pcor):
        t.zero_()


def fill_Au(st: KarmanState):
    L.check(L.load().kc_karman_fill_u(C.byref(st.K), ptr(st.ct), ptr(st.u), ptr(st.v), ptr(st.p), ptr(st.u0),
                                      ptr(st.Au), ptr(st.bu), ptr(st.Mu), st.s()), "kc_karman_fill_u")


def fill_Av(st: KarmanState):
    L.check(L.load().kc_karman_fill_v(C.byref(st.K), ptr(st.ct), ptr(st.u), ptr(st.v), ptr(st.p), ptr(st.v0),
                                      ptr(st.Av), ptr(st.bv), ptr(st.Mv), st.s()), "kc_karman_fill_v")


def fill_Ap(st: KarmanState):
    L.check(L.load().kc_karman_fill_p(C.byref(st.K), ptr(st.ct), ptr(st.u), ptr(st.v), ptr(st.Au), ptr(st.Av),
                                      ptr(st.Ap), ptr(st.bp), ptr(st.Mp), st.s()), "kc_karman_fill_p")


def bicgstab(st: KarmanState, which: str, eps=1e-8, output=0):
    """karman_taichi.py:342-456 on system ``which`` in {'u', 'v', 'p'}: right
    Jacobi, warm start from the previous solution, cap 100 n."""
    A, b, x, M = {"u": (st.Au, st.bu, st.xu, st.Mu), "v": (st.Av, st.bv, st.xv, st.Mv),
                  "p": (st.Ap, st.bp, st.xp, st.Mp)}[which]
    S = st.cfg.ny + 1 if which == "v" else st.cfg.ny
    info = _bicgstab(Stencil(A, stride=S), b, x, eps=eps, max_iter=100 * b.numel(), warm=True, M=M,
                     omega_break=True, ws=st.ws[which])
    st.solves.append((which, info))
    if output:
        print(f"        >> {which}: {info.status_name} after {info.iters} iterations, rel res {info.rel_res:e}")
    return info


def xu_back(st):
    L.check(L.load().kc_karman_back(C.byref(st.K), 0, ptr(st.xu), ptr(st.u), st.s()), "kc_karman_back")


def xv_back(st):
    L.check(L.load().kc_karman_back(C.byref(st.K), 1, ptr(st.xv), ptr(st.v), st.s()), "kc_karman_back")


def xp_back(st):
    L.check(L.load().kc_karman_back(C.byref(st.K), 2, ptr(st.xp), ptr(st.pcor), st.s()), "kc_karman_back")


def solve_momentum_bicgstab(st, eps=1e-8, max_iterations=1, solve_output=0, linalg_output=0):
    """karman_taichi.py:482-494."""
    out = None
    for steps in range(max_iterations):
        if solve_output:
            print(f"    [ {steps} / {max_iterations} ] Iteratively solving momentum equation using BiCGSTAB...")
        fill_Au(st)
        fill_Av(st)
        iu = bicgstab(st, "u", eps, linalg_output)
        iv = bicgstab(st, "v", eps, linalg_output)
        xu_back(st)
        xv_back(st)
        out = (iu, iv)
    return out


def solve_pcorrection_bicgstab(st, eps=1e-8, linalg_output=0):
    """karman_taichi.py:497-504."""
    fill_Ap(st)
    info = bicgstab(st, "p", eps, linalg_output)
    xp_back(st)
    return info


def puv_correction(st) -> float:
    """karman_taichi.py:507-542; returns max |pcor| over all cells."""
    L.check(L.load().kc_karman_puv_correction(C.byref(st.K), ptr(st.ct), ptr(st.pcor), ptr(st.Au), ptr(st.Av),
                                              ptr(st.u), ptr(st.v), ptr(st.p), ptr(st.pmax), ptr(st.rws), st.s()),
            "kc_karman_puv_correction")
    return float(st.pmax[0].item())


def correct_conserv(st):
    """karman_taichi.py:586-614 (outlet mass-flow rescale and udiv)."""
    L.check(L.load().kc_karman_correct_conserv(C.byref(st.K), ptr(st.u), ptr(st.v), ptr(st.udiv), st.s()),
            "kc_karman_correct_conserv")


def post_process_field(st, canvases=True):
    """karman_taichi.py:545-583: cell-centre velocities, udiv, display canvases (device arrays)."""
    from .fields import PostProcessor
    if getattr(st, "_post", None) is None:
        st._post = PostProcessor(st.cfg.nx, st.cfg.ny, st.device)
    return st._post(st.u, st.v, st.p, st.pcor, st.udiv, st.cfg.dx, st.cfg.dy, canvases)


def write_matrix(mat, name):
    """karman_taichi.py:157-159."""
    from .fields import write_matrix as wm
    wm(mat, name)


def time_forward(st):
    """karman_taichi.py:617-622."""
    lib = L.load()
    L.check(lib.kc_copy(ptr(st.u0), ptr(st.u), st.u.numel() * 8, st.s()), "kc_copy")
    L.check(lib.kc_copy(ptr(st.v0), ptr(st.v), st.v.numel() * 8, st.s()), "kc_copy")


def substep(st):
    """One SIMPLE sub-iteration of karman_taichi.py:636-651."""
    solve_momentum_bicgstab(st, st.cfg.eps, 1, 0, 0)
    correct_conserv(st)
    solve_pcorrection_bicgstab(st, st.cfg.eps, 0)
    return puv_correction(st)


def run(st, n_steps=1, max_sub=None, verbose=False):
    """The __main__ loop of karman_taichi.py:625-659 without the PNG/CSV output."""
    cfg = st.cfg
    max_sub = cfg.max_sub if max_sub is None else max_sub
    log = []
    for time_step in range(n_steps):
        pcor_max = 0.0
        subs = 0
        for sub in range(max_sub):
            pcor_current = 10000.0
            t0 = time.perf_counter()
            if sub == 0:
                pcor_max = substep(st)
            else:
                pcor_current = substep(st)
            subs += 1
            if verbose:
                print(f"    >> [ time = {time_step * cfg.dt: .4f} ] sub {sub}: pcor {pcor_current:.3e} / {pcor_max:.3e} "
                      f"({time.perf_counter() - t0:.3f} s)")
            if pcor_current < cfg.pcor_ratio * pcor_max:
                break
        time_forward(st)
        log.append(dict(step=time_step, subs=subs, pcor_max=pcor_max))
    return log
