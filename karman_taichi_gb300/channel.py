"""Channel SIMPLE driver on the GPU (blocked-cell cylinder in a channel).

One time step is the SIMPLE outer loop of karman_taichi.py:633-659 /
simple.py:270-281 with the discretisation of simple.py (mid-point convection,
set_bc-style wall and Dirichlet folding) and the outlet treatment of
karman_taichi.py (zero-gradient row + mass-flow rescale):

    assemble u, v momentum   (kc_assemble_momentum)
    solve u*, v*             (BiCGSTAB, cold start, rel tol eps)
    relax + outlet           (kc_relax_velocity, kc_outlet_conserve)
    assemble p'              (kc_assemble_pcorr; its max|mdiv| is the mass residual)
    solve p'                 (BiCGSTAB)
    correct u, v, p          (kc_correct)
    stop when mass residual <= mass_tol or after max_outer iterations
    u0 <- u, v0 <- v         (time_forward, karman_taichi.py:617-622)

``precision='fp64'`` is the plain method.  ``precision='mixed'`` assembles an
FP32 copy of every system and solves with FP32 BiCGSTAB (FP64 inner products)
inside an FP64 iterative refinement; its pressure correction (symmetric) is
solved by CG preconditioned with the aggregation multigrid V-cycle
(``pcorr_precond='mg'``, the multigrid step the reference names as missing,
README.md:31), and an
optional ``learned`` object supplies the trained network, applied as the
first preconditioner application of a flexible CG for p'
(karman_taichi_gb300.learned, kc_pcg_flexible).
"""
from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np
import torch

from . import _lib as L
from . import geometry
from .config import ChannelConfig
from .linalg import (Multigrid, Stencil, Workspace, bicgstab, bicgstab_refined, pcg_flexible, pcg_refined, ptr,
                     rbgs, rbgs_refined, stream_handle)


# sweeps the Gauss-Seidel momentum solve may take before the refined BiCGSTAB takes over
MOMENTUM_SWEEPS = 200
# inner tolerance of the one-sweep Gauss-Seidel path of the momentum refinement (systems whose rows
# link across their ends; the channel's padded systems take 12 sweeps per pass without an inner test)
EPS_INNER_GS = 1e-5


class ChannelSolver:
    def __init__(self, cfg: ChannelConfig, device="cuda", precision="fp64", use_graph=True,
                 eps_inner=1e-3, learned=None, pcorr_precond="mg", mg_opts=None, eps_inner_p=1e-4, native=True,
                 momentum="rbgs_refined", recycle=4):
        """``momentum`` (mixed precision): "rbgs_refined" (default), FP32
        red-black Gauss-Seidel sweeps in FP64 refinement (several sweeps per
        launch; 12.95 against 11.53 time steps/s at 2048 x 512 on GB300);
        "bicgstab", FP32 BiCGSTAB in FP64 refinement; or "rbgs", FP64 red-black
        Gauss-Seidel (on GB300 an FP64
        sweep is bound by the FP64 pipe, ~56 us at 2048 x 512, and 9-13 sweeps
        from the warm start cost more than the refined BiCGSTAB).  Both
        Gauss-Seidel variants hand over to the refined BiCGSTAB, from where
        they stopped, if they miss the tolerance.  The FP64 path always uses
        the reference's BiCGSTAB.  ``recycle`` (mixed precision without a
        network): every p' solve starts from the Galerkin projection onto the
        last ``recycle`` p' solutions (kc_recycle_guess; 0: from zero)."""
        if precision not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        if momentum not in ("rbgs", "rbgs_refined", "bicgstab"):
            raise ValueError("momentum must be 'rbgs', 'rbgs_refined' or 'bicgstab'")
        self.cfg, self.precision, self.use_graph = cfg, precision, use_graph
        self.momentum = momentum if precision == "mixed" else "bicgstab"
        self.eps_inner, self.eps_inner_p = eps_inner, eps_inner_p
        self.learned = learned
        self.device = torch.device(device)
        L.load()
        nx, ny = cfg.nx, cfg.ny
        f64 = dict(dtype=torch.float64, device=self.device)
        f32 = dict(dtype=torch.float32, device=self.device)
        z = torch.zeros
        self.solid_np = geometry.solid_mask(nx, ny, cfg.obstacles)
        self.solid = torch.from_numpy(self.solid_np).to(self.device)
        self.u, self.v, self.p = z((nx + 3, ny + 2), **f64), z((nx + 2, ny + 3), **f64), z((nx + 2, ny + 2), **f64)
        self.u0, self.v0 = z_like(self.u), z_like(self.v)
        self.pcor = z_like(self.p)
        self.u_mid, self.v_mid = z_like(self.u), z_like(self.v)
        self.coef_u, self.b_u = z((5, nx + 3, ny + 2), **f64), z_like(self.u)
        self.coef_v, self.b_v = z((5, nx + 2, ny + 3), **f64), z_like(self.v)
        self.coef_p, self.b_p = z((5, nx + 2, ny + 2), **f64), z_like(self.p)
        if precision == "mixed":
            self.coef_u32, self.b_u32 = z((5, nx + 3, ny + 2), **f32), z((nx + 3, ny + 2), **f32)
            self.coef_v32, self.b_v32 = z((5, nx + 2, ny + 3), **f32), z((nx + 2, ny + 3), **f32)
            self.coef_p32, self.b_p32 = z((5, nx + 2, ny + 2), **f32), z((nx + 2, ny + 2), **f32)
        else:
            self.coef_u32 = self.b_u32 = self.coef_v32 = self.b_v32 = self.coef_p32 = self.b_p32 = None
        self.mass = z(2, **f64)
        self.pmax = z(1, **f64)
        self.rws = torch.zeros(L.load().kc_reduce_ws_bytes(), dtype=torch.uint8, device=self.device)
        self.ws_u, self.ws_v, self.ws_p = Workspace(self.device), Workspace(self.device), Workspace(self.device)
        self.A_u, self.A_v, self.A_p = Stencil(self.coef_u), Stencil(self.coef_v), Stencil(self.coef_p)
        self.mg = None
        self.pcorr_precond = pcorr_precond if precision == "mixed" else "none"
        if precision == "mixed":
            self.A_u32, self.A_v32 = Stencil(self.coef_u32), Stencil(self.coef_v32)
            # the FP32 pressure system comes out of the assembly in Laplacian form
            self.A_p32 = Stencil(self.coef_p32, form=L.FORM_LAPLACIAN)
            if self.pcorr_precond == "mg":
                self.mg = Multigrid(self.A_p32, **(mg_opts or {}))
        self.x0_p = None     # optional initial guess for p'
        self.learned_stats = [0, 0]   # p' solves that applied / rejected the network's prediction
        self._flex_ws = None
        self._side = None   # the stream the p' hierarchy is built on while the recycled guess forms
        self.recycle = int(recycle) if (precision == "mixed" and learned is None and self.mg is not None) else 0
        self._rstate = L.KcRecycleState()
        self._rc_buf = None
        if self.recycle:
            self._side = torch.cuda.Stream(device=self.device)
            n = (nx + 2) * (ny + 2)
            nbytes = L.load().kc_channel_recycle_ws_bytes(n, self.recycle)
            self._rc_raw = torch.zeros(nbytes + 256, dtype=torch.uint8, device=self.device)
            off = (-self._rc_raw.data_ptr()) % 256
            a256 = lambda b: (b + 255) // 256 * 256
            R = self.recycle
            # the native step's layout: R ring slots, the guess, the projection's scratch
            self._rc_buf = self._rc_raw[off:off + nbytes]
            self._rc_ring = self._rc_buf[:R * n * 8].view(torch.float64).view(R, n)
            self._rc_x0 = self._rc_buf[a256(R * n * 8):a256(R * n * 8) + n * 8].view(torch.float64)
            self._rc_ws = self._rc_buf[a256(R * n * 8) + a256(n * 8):]
        self.fallbacks = 0   # accelerated solves that fell back (p': plain BiCGSTAB; Gauss-Seidel momentum: refined BiCGSTAB)
        self.last_accel = None  # SolveInfo of the last accelerated p' solve
        ph = L.KcPhys()
        ph.nx, ph.ny, ph.mode = nx, ny, L.MODE_CHANNEL
        ph.dx, ph.dy, ph.rho, ph.mu, ph.dt, ph.U = cfg.dx, cfg.dy, cfg.rho, cfg.mu, cfg.dt, cfg.U
        ph.alpha_m, ph.alpha_u, ph.alpha_p = cfg.alpha_m, cfg.alpha_u, cfg.alpha_p
        self.phys = ph
        self.history = []        # per time step: list of per-outer-iteration records
        # the native step (kc_channel_step) runs the whole outer loop in the library (with the
        # network, when one is attached); the Python loop below it is kept for stage-by-stage use
        self.native = bool(native) and (precision == "fp64" or self.mg is not None)
        self.persistent = True   # BiCGSTAB solves as one cooperative launch (native step)
        self.check_every_p = 4   # CG iterations per graph chunk between the host's convergence checks
        self._chan = None
        self.reset()

    # ---- state ------------------------------------------------------------------
    def reset(self, seed=None):
        cfg = self.cfg
        u, v, p = geometry.channel_initial_fields(cfg.nx, cfg.ny, self.solid_np, cfg.U, cfg.noise,
                                                  cfg.seed if seed is None else seed)
        self.set_state(u, v, p)

    def set_state(self, u, v, p, u0=None, v0=None):
        self._rstate.count = self._rstate.head = 0   # new fields: the ring of p' solutions starts empty
        def put(dst, src):
            src = torch.as_tensor(src, dtype=torch.float64)
            dst.copy_(src.to(self.device, non_blocking=True))
        put(self.u, u); put(self.v, v); put(self.p, p)
        put(self.u0, u if u0 is None else u0); put(self.v0, v if v0 is None else v0)
        self.pcor.zero_()

    def state_numpy(self):
        return {k: getattr(self, k).cpu().numpy() for k in ("u", "v", "p", "u0", "v0", "pcor")}

    # ---- stages -----------------------------------------------------------------
    def _s(self):
        return stream_handle(self.device)

    def assemble_momentum(self):
        lib = L.load()
        L.check(lib.kc_assemble_momentum(C.byref(self.phys), ptr(self.u), ptr(self.v), ptr(self.p), ptr(self.u0),
                                         ptr(self.v0), ptr(self.solid), ptr(self.coef_u), ptr(self.b_u),
                                         ptr(self.coef_v), ptr(self.b_v), ptr(self.coef_u32), ptr(self.b_u32),
                                         ptr(self.coef_v32), ptr(self.b_v32), self._s()), "kc_assemble_momentum")

    def _solve(self, A, A32, b, x, ws):
        cfg = self.cfg
        if self.precision == "fp64":
            return bicgstab(A, b, x, eps=cfg.eps, max_iter=A.n, ws=ws, use_graph=self.use_graph,
                            persistent=self.persistent)
        # warm start from the previous outer iteration's u*, v* (karman_taichi.py:362-371 warm-starts too);
        # the stopping test is ||b - A x|| / ||b|| < eps, the reference's test for a cold start
        before = 0
        if self.momentum == "rbgs_refined":
            info = rbgs_refined(A, A32, b, x, eps=cfg.eps, eps_inner=EPS_INNER_GS, max_iter=MOMENTUM_SWEEPS, ws=ws,
                                use_graph=self.use_graph, warm=True)
            if info.ok:
                return info
            self.fallbacks += 1   # the refined BiCGSTAB takes over from where Gauss-Seidel stopped
            before = info.iters
        elif self.momentum == "rbgs":
            info = rbgs(A, b, x, eps=cfg.eps, max_iter=MOMENTUM_SWEEPS, warm=True, rel_to_b=True, ws=ws,
                        use_graph=self.use_graph)
            if info.ok:
                return info
            self.fallbacks += 1   # the refined BiCGSTAB takes over from where Gauss-Seidel stopped
            before = info.iters
        info = bicgstab_refined(A, A32, b, x, eps=cfg.eps, eps_inner=self.eps_inner, ws=ws,
                                use_graph=self.use_graph, persistent=self.persistent, warm=True)
        info.iters += before
        return info

    def solve_momentum(self):
        iu = self._solve(self.A_u, getattr(self, "A_u32", None), self.b_u, self.u_mid, self.ws_u)
        iv = self._solve(self.A_v, getattr(self, "A_v32", None), self.b_v, self.v_mid, self.ws_v)
        return iu, iv

    def relax(self):
        lib = L.load()
        L.check(lib.kc_relax_velocity(C.byref(self.phys), ptr(self.solid), ptr(self.u_mid), ptr(self.v_mid),
                                      ptr(self.u), ptr(self.v), None, ptr(self.rws), self._s()), "kc_relax_velocity")
        L.check(lib.kc_outlet_conserve(C.byref(self.phys), ptr(self.u), self._s()), "kc_outlet_conserve")

    def assemble_p(self):
        lib = L.load()
        L.check(lib.kc_assemble_pcorr(C.byref(self.phys), ptr(self.u), ptr(self.v), ptr(self.coef_u),
                                      ptr(self.coef_v), ptr(self.solid), ptr(self.coef_p), ptr(self.b_p),
                                      ptr(self.coef_p32), ptr(self.b_p32), None, ptr(self.mass), ptr(self.rws),
                                      self._s()), "kc_assemble_pcorr")

    def solve_p(self):
        if self.learned is not None and self.mg is not None:
            # the network as the first preconditioner application of a flexible CG
            self.mg.setup()
            NX, NY = self.b_p.shape
            info, fi = pcg_flexible(self.A_p, self.A_p32, self.b_p, self.pcor, self.mg,
                                    net=self.learned.native(NX, NY), eps=self.cfg.eps, eps_inner=self.eps_inner_p,
                                    ws=self._ws_flex(), inner_ws=self.ws_p, use_graph=self.use_graph,
                                    check_every=self.check_every_p)
            self.last_accel = info
            self.learned_stats[0] += fi.learned_used
            self.learned_stats[1] += fi.learned_rejected
            if info.ok:
                return info
            self.fallbacks += 1
            plain = bicgstab(self.A_p, self.b_p, self.pcor, eps=self.cfg.eps, max_iter=self.A_p.n, ws=self.ws_p,
                             use_graph=self.use_graph, persistent=self.persistent)
            plain.iters += info.iters
            return plain
        if self.mg is not None:
            x0 = self.x0_p
            if self.recycle and x0 is None and self._rstate.count > 0:
                # the hierarchy on a side stream while the guess forms on this one (as the native step)
                main = torch.cuda.current_stream(self.device)
                side = self._side
                side.wait_stream(main)
                with torch.cuda.stream(side):
                    self.mg.setup()
                x0 = self._recycle_guess()
                main.wait_stream(side)
            else:
                self.mg.setup()
            # the pressure correction is symmetric: multigrid-preconditioned CG
            info = pcg_refined(self.A_p, self.A_p32, self.b_p, self.pcor, self.mg, eps=self.cfg.eps,
                               eps_inner=self.eps_inner_p, x0=x0, ws=self.ws_p, use_graph=self.use_graph,
                               check_every=self.check_every_p)
            if self.recycle:
                self._recycle_push()
            self.last_accel = info
            if info.ok:
                return info
            # accelerated solve stalled: plain BiCGSTAB is the fallback
            self.fallbacks += 1
            plain = bicgstab(self.A_p, self.b_p, self.pcor, eps=self.cfg.eps, max_iter=self.A_p.n, ws=self.ws_p,
                             use_graph=self.use_graph, persistent=self.persistent)
            plain.iters += info.iters
            if self.recycle:   # the ring keeps the solution the step goes on with
                self._rstate.head = (self._rstate.head - 1) % self.recycle
                self._rstate.count -= 1
                self._recycle_push()
            return plain
        return self._solve(self.A_p, getattr(self, "A_p32", None), self.b_p, self.pcor, self.ws_p)

    # ---- recycling: the ring of p' solutions in one buffer laid out as the native step's ------------
    def _recycle_guess(self):
        """x0 from the projection onto the stored solutions, newest first (None when the ring is empty)."""
        m, R = self._rstate.count, self.recycle
        if m == 0:
            return None
        Z = (C.c_void_p * m)(*[self._rc_ring[(self._rstate.head - 1 - i) % R].data_ptr() for i in range(m)])
        L.check(L.load().kc_recycle_guess(C.byref(self.A_p.system), ptr(self.b_p), Z, m, ptr(self._rc_x0),
                                          ptr(self._rc_ws), self._rc_ws.numel(), None, self._s()),
                "kc_recycle_guess")
        return self._rc_x0

    def _recycle_push(self):
        self._rc_ring[self._rstate.head].copy_(self.pcor.view(-1))
        self._rstate.head = (self._rstate.head + 1) % self.recycle
        self._rstate.count = min(self._rstate.count + 1, self.recycle)

    def _ws_flex(self):
        if self._flex_ws is None:
            self._flex_ws = Workspace(self.device)
        return self._flex_ws

    def correct(self):
        lib = L.load()
        L.check(lib.kc_correct(C.byref(self.phys), ptr(self.pcor), ptr(self.coef_u), ptr(self.coef_v),
                               ptr(self.solid), ptr(self.u), ptr(self.v), ptr(self.p), ptr(self.pmax),
                               ptr(self.rws), self._s()), "kc_correct")

    def time_forward(self):
        lib = L.load()
        L.check(lib.kc_copy(ptr(self.u0), ptr(self.u), self.u.numel() * 8, self._s()), "kc_copy")
        L.check(lib.kc_copy(ptr(self.v0), ptr(self.v), self.v.numel() * 8, self._s()), "kc_copy")

    def outer_iteration(self):
        self.assemble_momentum()
        iu, iv = self.solve_momentum()
        self.relax()
        self.assemble_p()
        ip = self.solve_p()
        self.correct()
        mass = float(self.mass[0].item())
        return dict(mass=mass, it_u=iu.iters, it_v=iv.iters, it_p=ip.iters,
                    st=(iu.status, iv.status, ip.status), ref=(iu.refinements, iv.refinements, ip.refinements))

    # ---- native step ------------------------------------------------------------------
    def native_struct(self):
        """The kc_channel descriptor of this solver (buffers preallocated to the sizes the
        native step needs)."""
        if self._chan is not None:
            return self._chan
        lib = L.load()
        c = L.KcChannel()
        c.phys = self.phys
        c.precision = L.F64 if self.precision == "fp64" else L.F32
        c.max_outer, c.use_graph, c.persistent = self.cfg.max_outer, int(self.use_graph), int(self.persistent)
        c.momentum = {"rbgs": L.MOMENTUM_RBGS, "rbgs_refined": L.MOMENTUM_RBGS_REFINED}.get(self.momentum,
                                                                                       L.MOMENTUM_BICGSTAB)
        c.check_every_p = int(self.check_every_p)
        c.mass_tol, c.eps, c.eps_inner, c.eps_inner_p = self.cfg.mass_tol, self.cfg.eps, self.eps_inner, self.eps_inner_p
        for k in ("u", "v", "p", "u0", "v0", "pcor", "u_mid", "v_mid", "solid", "coef_u", "b_u", "coef_v", "b_v",
                  "coef_p", "b_p", "coef_u32", "b_u32", "coef_v32", "b_v32", "coef_p32", "b_p32", "mass", "pmax",
                  "rws"):
            t = getattr(self, k)
            setattr(c, k, None if t is None else t.data_ptr())
        sizes = {}
        for k, A in (("u", self.A_u), ("v", self.A_v), ("p", self.A_p)):
            plain = lib.kc_bicgstab_ws_bytes(A.n, A.stride, L.F64)
            if self.precision == "fp64":
                sizes[k] = plain
            elif k == "p":
                sizes[k] = max(plain, lib.kc_pbicgstab_ws_bytes(A.n, A.stride))
            else:
                sizes[k] = max(lib.kc_refined_ws_bytes(A.n, A.stride), lib.kc_rbgs_ws_bytes(A.n, A.stride))
        for k, ws in (("u", self.ws_u), ("v", self.ws_v), ("p", self.ws_p)):
            buf = ws.get(sizes[k])
            setattr(c, "ws_" + k, buf.data_ptr())
            setattr(c, "ws_" + k + "_bytes", buf.numel())
        if self.mg is not None:
            c.mg_ws, c.mg_ws_bytes, c.mg_opts = self.mg.ws.data_ptr(), self.mg.ws.numel(), self.mg.opts
        if self.recycle:
            c.recycle = self.recycle
            c.ws_recycle, c.ws_recycle_bytes = self._rc_buf.data_ptr(), self._rc_buf.numel()
            c.rstate = C.addressof(self._rstate)
        if self.learned is not None and self.mg is not None:
            NX, NY = self.b_p.shape
            self._net = self.learned.native(NX, NY)          # kept alive with the descriptor
            buf = self._ws_flex().get(lib.kc_pcg_flexible_ws_bytes(self.A_p.n))
            c.learned = C.addressof(self._net)
            c.ws_flex, c.ws_flex_bytes = buf.data_ptr(), buf.numel()
        self._chan = c
        return c

    def _step_native(self):
        st = L.KcChannelStats()
        L.check(L.load().kc_channel_step(C.byref(self.native_struct()), C.byref(st), self._s()), "kc_channel_step")
        self.fallbacks += st.fallbacks
        self.learned_stats[0] += st.learned
        self.learned_stats[1] += st.learned_rejected
        rec = [dict(mass=st.mass, it_u=st.it_u, it_v=st.it_v, it_p=st.it_p, outer=st.outer, status=st.status)]
        self.history.append(rec)
        return rec

    def step(self):
        """One time step; returns the per-outer-iteration records (native: one record
        with the step's totals and its outer-iteration count)."""
        if self.native:
            return self._step_native()
        rec = []
        for _ in range(self.cfg.max_outer):
            s = self.outer_iteration()
            rec.append(s)
            # a NaN or Inf ends the step (as kc_channel_step does): the outer loop would only repeat it
            if L.NONFINITE in s["st"] or not np.isfinite(s["mass"]):
                s["status"] = L.NONFINITE
                break
            if s["mass"] <= self.cfg.mass_tol:
                break
        self.time_forward()
        self.history.append(rec)
        return rec

    def run(self, n_steps=None, callback=None):
        n = self.cfg.n_steps if n_steps is None else n_steps
        for k in range(n):
            t = time.perf_counter()
            rec = self.step()
            if callback:
                callback(k, rec, time.perf_counter() - t)
        return self.history

    def post_process(self, canvases=True):
        """post_process_field (karman_taichi.py:545-583) of the current fields: device arrays
        u_post, v_post, udiv, minmax and (canvases) u/v/p/pcor/udiv_disp."""
        from .fields import PostProcessor
        if getattr(self, "_post", None) is None:
            self._post = PostProcessor(self.cfg.nx, self.cfg.ny, self.device)
            self.udiv = torch.zeros_like(self.p)
        return self._post(self.u, self.v, self.p, self.pcor, self.udiv, self.cfg.dx, self.cfg.dy, canvases)

    def write_fields(self, step, directory=".", images=False):
        """The every-10-steps dump of karman_taichi.py:677-683 (CSV), optionally the five canvases as PGM."""
        from . import fields
        out = self.post_process(canvases=images)
        paths = fields.write_timestep(step, {"pcor": self.pcor, "p": self.p, "u": self.u, "v": self.v,
                                             "udiv": self.udiv}, directory)
        if images:
            for name in fields.CANVASES:
                paths.append(fields.write_pgm(out[name + "_disp"], os.path.join(directory,
                                                                                f"timestep{step:06}_{name}.pgm")))
        return paths

    def mass_residual(self) -> float:
        """max |mdiv| of the current (corrected) field."""
        lib = L.load()
        out = torch.zeros(2, dtype=torch.float64, device=self.device)
        L.check(lib.kc_mass_residual(C.byref(self.phys), ptr(self.u), ptr(self.v), ptr(self.solid), None,
                                     ptr(out), ptr(self.rws), self._s()), "kc_mass_residual")
        return float(out[0].item())


def z_like(t):
    return torch.zeros_like(t)
