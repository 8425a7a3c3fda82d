"""Learned initial guess for the pressure-correction solve.

The reference has no learned component (its p' solve is plain or Jacobi
BiCGSTAB from zero, bicgsolver.py:88-135, karman_taichi.py:342-456).  The
accelerated path can start the p' solve from a network's prediction instead
of zero: a 4-level U-Net (16/32/48/64 channels, 3x3 convolutions + ReLU, 2x2
average pooling, nearest upsampling with skip concatenation, 1x1 head,
226,721 parameters) evaluated and trained on the GPU by the kernels of
``csrc/kc_unet.cu`` (BF16 activations and weights on the tensor cores, FP32
accumulation, FP32 master weights and Adam).

Inputs (per cell of the p' grid, zero outside the fluid; assembled at full
resolution by kc_unet_features, then 2x2-averaged: the network runs at half
resolution and its output is bilinearly upsampled, kc_unet_guess_up2):
  0  b / s_b                the mass imbalance, s_b its RMS over fluid cells
  1  fluid indicator        (a row with links)
  2  d / mean(d)            d = sum |a_nb|, the diagonal of the p' operator
  3  P1(i) / s_p            the 1-D channel solution of the column-summed
                            system: flux F(i) = sum_{i' <= i} sum_j b, and
                            P1(i) = sum_{i' >= i} F(i') / sum_j |aE(i', j)|
                            (Neumann inlet, Dirichlet outlet), s_p its RMS.
Output: p' / s_p.  The network sees the global, smooth part of p' through P1
(its receptive field is ~100 cells, the channel 2048) and learns the 2-D
corrections around the obstacle and the walls.

Every step -- features, convolutions, pooling, upsampling, loss, optimiser
-- is a kc_unet_* kernel.
"""
from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np
import torch

from . import _lib as L
from .linalg import ptr, stream_handle

CH = (16, 32, 48, 64)
CIN = 16          # input channels (4 features, zero padded)
NFEAT = 4
WEIGHTS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights")


def layer_specs():
    """(name, cin, cout) of every 3x3 convolution in forward order."""
    c0, c1, c2, c3 = CH
    return [("e0a", CIN, c0), ("e0b", c0, c0), ("e1a", c0, c1), ("e1b", c1, c1),
            ("e2a", c1, c2), ("e2b", c2, c2), ("b3a", c2, c3), ("b3b", c3, c3),
            ("d2a", c3 + c2, c2), ("d2b", c2, c2), ("d1a", c2 + c1, c1), ("d1b", c1, c1),
            ("d0a", c1 + c0, c0), ("d0b", c0, c0)]


def init_params(seed=0):
    """He-normal 3x3 weights [9][cout][cin] (padded input channels zero), zero
    biases, small head; the same draw as the CPU restatement's init_params."""
    rng = np.random.default_rng(seed)
    P = {}
    for name, cin, cout in layer_specs():
        fan_in = 9 * (NFEAT if name == "e0a" else cin)
        w = rng.standard_normal((9, cout, cin)).astype(np.float32) * np.float32(np.sqrt(2.0 / fan_in))
        if name == "e0a":
            w[:, :, NFEAT:] = 0.0
        P[name + ".w"] = w
        P[name + ".b"] = np.zeros(cout, dtype=np.float32)
    P["head.w"] = (rng.standard_normal(CH[0]) * 0.1).astype(np.float32)
    P["head.b"] = np.zeros(1, dtype=np.float32)
    return P


def _check(rc, what):
    return L.check(rc, what)


def _split(c):
    """Channel groups the convolution kernel accepts (16/32/48/64 each)."""
    out, o = [], 0
    while o < c:
        g = min(64, c - o)
        g = 48 if g not in (16, 32, 48, 64) and g > 48 else g
        g = 32 if g not in (16, 32, 48, 64) and g > 32 else g
        g = 16 if g not in (16, 32, 48, 64) else g
        out.append((o, g))
        o += g
    return out


class UNet:
    """Device U-Net: FP32 master parameters in one flat buffer, BF16 copies
    for the kernels, activations for one (H, W) kept for the backward pass."""

    def __init__(self, device="cuda", params=None, seed=0):
        self.device = torch.device(device)
        L.load()
        P = params if params is not None else init_params(seed)
        names = []
        for name, _, _ in layer_specs():
            names += [name + ".w", name + ".b"]
        names += ["head.w", "head.b"]
        self.names = names
        self.shapes = {k: tuple(np.shape(P[k])) for k in names}
        sizes = [int(np.prod(self.shapes[k])) for k in names]
        self.offsets = dict(zip(names, np.cumsum([0] + sizes[:-1]).tolist()))
        self.n_params = int(sum(sizes))
        flat = np.concatenate([np.asarray(P[k], dtype=np.float32).reshape(-1) for k in names])
        f32 = dict(dtype=torch.float32, device=self.device)
        self.p = torch.from_numpy(flat).to(self.device)
        self.p16 = torch.empty(self.n_params, dtype=torch.bfloat16, device=self.device)
        self.g = torch.zeros(self.n_params, **f32)
        self.m = torch.zeros(self.n_params, **f32)
        self.v = torch.zeros(self.n_params, **f32)
        self.step_count = 0
        self.flipped = {}
        for name, cin, cout in layer_specs():
            self.flipped[name] = torch.empty(9 * cin * cout, dtype=torch.bfloat16, device=self.device)
        self._sync_bf16()
        self.acts = {}
        self.shape = None

    # ---- parameter views --------------------------------------------------------------
    def _view(self, t, k):
        o = self.offsets[k]
        n = int(np.prod(self.shapes[k]))
        return t[o:o + n]

    def params_numpy(self):
        h = self.p.cpu().numpy()
        return {k: h[self.offsets[k]:self.offsets[k] + int(np.prod(self.shapes[k]))].reshape(self.shapes[k]).copy()
                for k in self.names}

    def grads_numpy(self):
        h = self.g.cpu().numpy()
        return {k: h[self.offsets[k]:self.offsets[k] + int(np.prod(self.shapes[k]))].reshape(self.shapes[k]).copy()
                for k in self.names}

    def _sync_bf16(self):
        _check(L.load().kc_unet_to_bf16(ptr(self.p), ptr(self.p16), self.n_params, stream_handle(self.device)),
               "kc_unet_to_bf16")

    # ---- buffers ----------------------------------------------------------------------
    def _alloc(self, H, W):
        if self.shape == (H, W):
            return
        if H % 8 or W % 8:
            raise ValueError("U-Net grid must be a multiple of 8 in both directions")
        bf = dict(dtype=torch.bfloat16, device=self.device)
        c0, c1, c2, c3 = CH
        dims = [(H, W), (H // 2, W // 2), (H // 4, W // 4), (H // 8, W // 8)]
        A = {}
        (h0, w0), (h1, w1), (h2, w2), (h3, w3) = dims
        for name, (h, w), c in [("in", dims[0], CIN), ("e0a", dims[0], c0), ("s0", dims[0], c0), ("x1", dims[1], c0),
                                ("e1a", dims[1], c1), ("s1", dims[1], c1), ("x2", dims[2], c1),
                                ("e2a", dims[2], c2), ("s2", dims[2], c2), ("x3", dims[3], c2),
                                ("b3a", dims[3], c3), ("y3", dims[3], c3), ("c2", dims[2], c3 + c2),
                                ("d2a", dims[2], c2), ("y2", dims[2], c2), ("c1", dims[1], c2 + c1),
                                ("d1a", dims[1], c1), ("y1", dims[1], c1), ("c0", dims[0], c1 + c0),
                                ("d0a", dims[0], c0), ("y0", dims[0], c0)]:
            A[name] = torch.zeros((h, w, c), **bf)
        A["out"] = torch.zeros((H, W), dtype=torch.float32, device=self.device)
        # gradient buffers: gA[l] grad of the level's output, gB[l] grad of its
        # first convolution's output, gS[l] grad of the skip s_l, gC[l] grad of
        # the concatenation c_l, gX[l] grad of the pooled input x_l
        z = lambda lvl, c: torch.zeros((dims[lvl][0], dims[lvl][1], c), **bf)
        self.gA = [z(l, CH[l]) for l in range(4)]
        self.gB = [z(l, CH[l]) for l in range(4)]
        self.gS = [z(l, CH[l]) for l in range(3)]
        self.gC = [z(l, CH[l + 1] + CH[l]) for l in range(3)]
        self.gX = [None] + [z(l, CH[l - 1]) for l in range(1, 4)]
        self.dout = torch.zeros((H, W), dtype=torch.float32, device=self.device)
        self.acts = A
        self.dims = dims
        self.shape = (H, W)

    # ---- building blocks --------------------------------------------------------------
    def _conv(self, x, name, cin, cout, y, relu=True):
        H, W = x.shape[:2]
        lib = L.load()
        w = self._view(self.p16, name + ".w")
        b = self._view(self.p, name + ".b")
        _check(lib.kc_unet_conv3x3(ptr(x), H, W, cin, ptr(w), 0, ptr(b), cout, 1 if relu else 0, None, ptr(y), 0,
                                   stream_handle(self.device)), "kc_unet_conv3x3")

    def _conv_data_grad(self, dy, name, cin, cout, dx, mask):
        """dx[H][W][cin] = conv(dy, flipped W), zeroed where mask <= 0 (mask nullable)."""
        H, W = dy.shape[:2]
        lib = L.load()
        wt = self.flipped[name]
        s = stream_handle(self.device)
        for o, g in _split(cin):
            _check(lib.kc_unet_conv3x3(ptr(dy), H, W, cout, C.c_void_p(wt.data_ptr() + 2 * o * cout),
                                       cin * cout, None, g, 0,
                                       None if mask is None else C.c_void_p(mask.data_ptr() + 2 * o),
                                       C.c_void_p(dx.data_ptr() + 2 * o), cin, s), "kc_unet_conv3x3 (data grad)")

    def _wgrad(self, x, dy, name, cin, cout):
        H, W = x.shape[:2]
        _check(L.load().kc_unet_conv3x3_wgrad(ptr(x), ptr(dy), H, W, cin, cout, ptr(self._view(self.g, name + ".w")),
                                              ptr(self._view(self.g, name + ".b")), stream_handle(self.device)),
               "kc_unet_conv3x3_wgrad")

    def _pool(self, x, y):
        H, W, Cc = x.shape
        _check(L.load().kc_unet_pool2(ptr(x), H, W, Cc, ptr(y), stream_handle(self.device)), "kc_unet_pool2")

    def _upcat(self, u, s, y):
        H, W, cs = s.shape
        _check(L.load().kc_unet_up2_concat(ptr(u), u.shape[2], ptr(s), cs, H, W, ptr(y), stream_handle(self.device)),
               "kc_unet_up2_concat")

    # ---- forward / backward -----------------------------------------------------------
    def forward(self, feat):
        """feat: bf16 [H][W][16] -> FP32 [H][W] (a view of an internal buffer)."""
        H, W = feat.shape[:2]
        self._alloc(H, W)
        A = self.acts
        A["in"].copy_(feat)
        c0, c1, c2, c3 = CH
        self._conv(A["in"], "e0a", CIN, c0, A["e0a"]); self._conv(A["e0a"], "e0b", c0, c0, A["s0"])
        self._pool(A["s0"], A["x1"])
        self._conv(A["x1"], "e1a", c0, c1, A["e1a"]); self._conv(A["e1a"], "e1b", c1, c1, A["s1"])
        self._pool(A["s1"], A["x2"])
        self._conv(A["x2"], "e2a", c1, c2, A["e2a"]); self._conv(A["e2a"], "e2b", c2, c2, A["s2"])
        self._pool(A["s2"], A["x3"])
        self._conv(A["x3"], "b3a", c2, c3, A["b3a"]); self._conv(A["b3a"], "b3b", c3, c3, A["y3"])
        self._upcat(A["y3"], A["s2"], A["c2"])
        self._conv(A["c2"], "d2a", c3 + c2, c2, A["d2a"]); self._conv(A["d2a"], "d2b", c2, c2, A["y2"])
        self._upcat(A["y2"], A["s1"], A["c1"])
        self._conv(A["c1"], "d1a", c2 + c1, c1, A["d1a"]); self._conv(A["d1a"], "d1b", c1, c1, A["y1"])
        self._upcat(A["y1"], A["s0"], A["c0"])
        self._conv(A["c0"], "d0a", c1 + c0, c0, A["d0a"]); self._conv(A["d0a"], "d0b", c0, c0, A["y0"])
        _check(L.load().kc_unet_head(ptr(A["y0"]), c0, H * W, ptr(self._view(self.p, "head.w")),
                                     ptr(self._view(self.p, "head.b")), ptr(A["out"]), stream_handle(self.device)),
               "kc_unet_head")
        return A["out"]

    def backward(self, dout):
        """Accumulates d loss / d params into self.g for d loss / d out = dout (FP32 [H][W])."""
        lib = L.load()
        s = stream_handle(self.device)
        A = self.acts
        H, W = self.shape
        c0, c1, c2, c3 = CH
        for name, cin, cout in layer_specs():
            _check(lib.kc_unet_flip_weights(ptr(self._view(self.p16, name + ".w")), cout, cin, cin,
                                            ptr(self.flipped[name]), s), "kc_unet_flip_weights")
        gA, gB, gS, gC, gX = self.gA, self.gB, self.gS, self.gC, self.gX
        _check(lib.kc_unet_head_bwd(ptr(A["y0"]), c0, H * W, ptr(self._view(self.p, "head.w")), ptr(dout),
                                    ptr(gA[0]), ptr(self._view(self.g, "head.w")), ptr(self._view(self.g, "head.b")),
                                    s), "kc_unet_head_bwd")
        _check(lib.kc_unet_relu_bwd(ptr(gA[0]), ptr(A["y0"]), gA[0].numel(), s), "kc_unet_relu_bwd")

        def block(lvl, a_name, b_name, in_name, cin, d_out, d_in, in_mask):
            """out = b(a(in)); d_out = grad of out (ReLU derivative applied): weight
            grads of a and b, gB[lvl] = grad of a's output, d_in = grad of in
            (masked by in_mask > 0 when in is a ReLU output; skipped when None)."""
            cout = CH[lvl]
            self._wgrad(A[a_name], d_out, b_name, cout, cout)
            self._conv_data_grad(d_out, b_name, cout, cout, gB[lvl], A[a_name])
            self._wgrad(A[in_name], gB[lvl], a_name, cin, cout)
            if d_in is not None:
                self._conv_data_grad(gB[lvl], a_name, cin, cout, d_in, in_mask)

        def split_cat(lvl):
            """gC[lvl] -> gA[lvl + 1] (upsampled input) and gS[lvl] (skip)."""
            Hl, Wl = self.dims[lvl]
            _check(lib.kc_unet_up2_concat_bwd(ptr(gC[lvl]), CH[lvl + 1], CH[lvl], Hl, Wl, ptr(gA[lvl + 1]),
                                              ptr(gS[lvl]), 0, s), "kc_unet_up2_concat_bwd")

        def pool_back(lvl, s_name):
            """gS[lvl] += pool gradient of gX[lvl + 1]; ReLU derivative of s_lvl."""
            Hl, Wl = self.dims[lvl]
            _check(lib.kc_unet_pool2_bwd(ptr(gX[lvl + 1]), Hl, Wl, CH[lvl], ptr(gS[lvl]), 1, s), "kc_unet_pool2_bwd")
            _check(lib.kc_unet_relu_bwd(ptr(gS[lvl]), ptr(A[s_name]), gS[lvl].numel(), s), "kc_unet_relu_bwd")

        # decoder: y_l = d_lb(d_la(c_l)), c_l = [up(y_{l+1}), s_l] (both ReLU outputs: c_l masks)
        block(0, "d0a", "d0b", "c0", c1 + c0, gA[0], gC[0], A["c0"]); split_cat(0)
        block(1, "d1a", "d1b", "c1", c2 + c1, gA[1], gC[1], A["c1"]); split_cat(1)
        block(2, "d2a", "d2b", "c2", c3 + c2, gA[2], gC[2], A["c2"]); split_cat(2)
        # bottleneck y3 = b3b(b3a(x3)); x3 = pool(s2) is not a ReLU output
        block(3, "b3a", "b3b", "x3", c2, gA[3], gX[3], None)
        # encoder: s_l = e_lb(e_la(x_l)), x_l = pool(s_{l-1}), x_0 = the features
        pool_back(2, "s2"); block(2, "e2a", "e2b", "x2", c1, gS[2], gX[2], None)
        pool_back(1, "s1"); block(1, "e1a", "e1b", "x1", c0, gS[1], gX[1], None)
        pool_back(0, "s0"); block(0, "e0a", "e0b", "in", CIN, gS[0], None, None)

    def zero_grad(self):
        self.g.zero_()

    def adam_step(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        _check(L.load().kc_unet_adam(ptr(self.p), ptr(self.g), ptr(self.m), ptr(self.v), self.n_params, lr, b1, b2,
                                     eps, self.step_count, ptr(self.p16), stream_handle(self.device)), "kc_unet_adam")

    def mse(self, out, target, weight, count):
        loss = torch.zeros(1, dtype=torch.float32, device=self.device)
        dout = self.dout
        _check(L.load().kc_unet_mse(ptr(out), ptr(target), ptr(weight), out.numel(), 1.0 / max(count, 1e-30), ptr(dout),
                                    ptr(loss), stream_handle(self.device)), "kc_unet_mse")
        return loss, dout

    # ---- native use ---------------------------------------------------------------------
    def native_net(self, NX, NY):
        """A ``kc_unet_net`` for the p' grid [NX][NY]: this network's FP32 and
        BF16 parameters and a device workspace, for kc_unet_predict and the
        flexible solve of the native SIMPLE step (no Python in the loop)."""
        lib = L.load()
        if lib.kc_unet_param_count() != self.n_params:
            raise ValueError("parameter layout differs from the library's U-Net")
        key = (NX, NY)
        if getattr(self, "_native", None) is None or self._native[0] != key:
            nbytes = lib.kc_unet_predict_ws_bytes(NX, NY)
            ws = torch.zeros(nbytes + 256, dtype=torch.uint8, device=self.device)
            off = (-ws.data_ptr()) % 256
            n = L.KcUnetNet()
            n.NX, n.NY = NX, NY
            n.params, n.params16 = self.p.data_ptr(), self.p16.data_ptr()
            n.ws, n.ws_bytes = ws.data_ptr() + off, nbytes
            self._native = (key, n, ws)
        return self._native[1]

    # ---- persistence --------------------------------------------------------------------
    def save(self, path):
        os.makedirs(os.path.dirname(path), exist_ok=True)
        np.savez_compressed(path, **{k.replace(".", "__"): v for k, v in self.params_numpy().items()})

    @classmethod
    def load(cls, path, device="cuda"):
        with np.load(path) as z:
            P = {k.replace("__", "."): z[k] for k in z.files}
        return cls(device=device, params=P)


# ---- features -------------------------------------------------------------------------------
def padded_shape(NX, NY):
    """Full-resolution feature grid: multiples of 16, so the half-resolution
    grid the network runs on divides by 8 (three poolings)."""
    return (NX + 15) // 16 * 16, (NY + 15) // 16 * 16


class Featurizer:
    """Device buffers of the feature pipeline of one p' grid [NX][NY]:
    kc_unet_features (full resolution, bf16 [H][W][16]) -> kc_unet_pool2 ->
    half resolution [H/2][W/2][16], the network's input."""

    def __init__(self, NX, NY, device):
        self.NX, self.NY = NX, NY
        self.H, self.W = padded_shape(NX, NY)
        self.Hh, self.Wh = self.H // 2, self.W // 2
        self.device = torch.device(device)
        bf = dict(dtype=torch.bfloat16, device=self.device)
        self.full = torch.zeros((self.H, self.W, CIN), **bf)
        self.fluid = torch.zeros((NX, NY), dtype=torch.float32, device=self.device)
        self.scales = torch.zeros(4, dtype=torch.float64, device=self.device)
        lib = L.load()
        self.ws = torch.zeros(lib.kc_unet_features_ws_bytes(NX), dtype=torch.uint8, device=self.device)

    def __call__(self, b, coef32, out=None):
        """Half-resolution features of A x = b (coef32: FP32 Laplacian planes)."""
        lib = L.load()
        s = stream_handle(self.device)
        _check(lib.kc_unet_features(ptr(b), ptr(coef32), self.NX, self.NY, self.H, self.W, ptr(self.full),
                                    ptr(self.fluid), ptr(self.scales), ptr(self.ws), self.ws.numel(), s),
               "kc_unet_features")
        half = out if out is not None else torch.empty((self.Hh, self.Wh, CIN), dtype=torch.bfloat16,
                                                       device=self.device)
        _check(lib.kc_unet_pool2(ptr(self.full), self.H, self.W, CIN, ptr(half), s), "kc_unet_pool2")
        return half

    def target(self, p, coef32):
        """Half-resolution training target of the solution p (after __call__ on the same system)."""
        tgt = torch.empty((self.Hh, self.Wh), dtype=torch.float32, device=self.device)
        wgt = torch.empty_like(tgt)
        _check(L.load().kc_unet_target_down2(ptr(p), ptr(coef32), self.NX, self.NY, ptr(self.scales), self.Hh,
                                             self.Wh, ptr(tgt), ptr(wgt), stream_handle(self.device)),
               "kc_unet_target_down2")
        return tgt, wgt

    def guess(self, out, coef32, x0):
        """x0 (FP64 [NX][NY]) from the network output (FP32 [H/2][W/2])."""
        _check(L.load().kc_unet_guess_up2(ptr(out), self.Hh, self.Wh, ptr(coef32), self.NX, self.NY,
                                          ptr(self.scales), ptr(x0), stream_handle(self.device)),
               "kc_unet_guess_up2")
        return x0


class LearnedGuess:
    """ChannelSolver hook.  The accelerated solver applies the network through
    ``native(NX, NY)`` as the first preconditioner application of a flexible
    CG (kc_pcg_flexible, inside the native step); ``predict(solver)`` is the
    same prediction driven from Python (training, tests, the initial-guess
    use)."""

    def __init__(self, net: UNet):
        self.net = net
        self.fz = None
        self.x0 = None
        self.calls = 0

    def native(self, NX, NY):
        return self.net.native_net(NX, NY)

    def predict(self, solver):
        NX, NY = solver.b_p.shape
        if self.fz is None or (self.fz.NX, self.fz.NY) != (NX, NY):
            self.fz = Featurizer(NX, NY, solver.device)
            self.half = torch.zeros((self.fz.Hh, self.fz.Wh, CIN), dtype=torch.bfloat16, device=solver.device)
            self.x0 = torch.zeros((NX, NY), dtype=torch.float64, device=solver.device)
        feat = self.fz(solver.b_p, solver.coef_p32, self.half)
        out = self.net.forward(feat)
        self.fz.guess(out, solver.coef_p32, self.x0)
        self.calls += 1
        return self.x0


# ---- training data and training -----------------------------------------------------------------
def collect_pairs(solver, n_steps, every=1, max_pairs=None):
    """Runs the solver's SIMPLE steps and records (features, target, weight,
    fluid count) of the p' systems of every `every`-th outer iteration, at the
    network's half resolution; the target is the converged p' / s_p (solved to
    rel. tol 1e-8)."""
    NX, NY = solver.b_p.shape
    fz = Featurizer(NX, NY, solver.device)
    pairs = []
    k = 0
    for _ in range(n_steps):
        for _ in range(solver.cfg.max_outer):
            solver.assemble_momentum()
            solver.solve_momentum()
            solver.relax()
            solver.assemble_p()
            take = k % every == 0 and (max_pairs is None or len(pairs) < max_pairs)
            if take:
                feat = fz(solver.b_p, solver.coef_p32)
                scales = fz.scales.clone()
            solver.solve_p()
            if take:
                fz.scales.copy_(scales)
                tgt, wgt = fz.target(solver.pcor, solver.coef_p32)
                pairs.append((feat, tgt, wgt, float(wgt.sum().item())))
            k += 1
            solver.correct()
            if float(solver.mass[0].item()) <= solver.cfg.mass_tol:
                break
        solver.time_forward()
    return pairs


class PairStore:
    """Training pairs kept on the device in compact form, for the large training
    sets (about 3 MB a pair at the 2048 x 512 channel's half resolution, against
    11 MB for the network's 16-channel bf16 input): the NFEAT real feature
    channels (bf16), the target (bf16; it is normalised to unit RMS, and
    8 mantissa bits are far below the prediction's error) and the fluid weight
    (uint8 quarters: a 2 x 2 average of a 0/1 mask).  Indexing gives the
    (features, target, weight, count) tuples `train` and `mean_loss` take,
    through one reusable set of full-size buffers."""

    def __init__(self, capacity, Hh, Wh, device):
        dev = torch.device(device)
        self.capacity, self.Hh, self.Wh = int(capacity), Hh, Wh
        self.feat = torch.empty((self.capacity, Hh, Wh, NFEAT), dtype=torch.bfloat16, device=dev)
        self.tgt = torch.empty((self.capacity, Hh, Wh), dtype=torch.bfloat16, device=dev)
        self.wq = torch.empty((self.capacity, Hh, Wh), dtype=torch.uint8, device=dev)
        self.count = []
        self._feat = torch.zeros((Hh, Wh, CIN), dtype=torch.bfloat16, device=dev)
        self._tgt = torch.empty((Hh, Wh), dtype=torch.float32, device=dev)
        self._wgt = torch.empty((Hh, Wh), dtype=torch.float32, device=dev)

    def __len__(self):
        return len(self.count)

    def full(self):
        return len(self.count) >= self.capacity

    def add(self, feat, tgt, wgt):
        k = len(self.count)
        self.feat[k].copy_(feat[..., :NFEAT])
        self.tgt[k].copy_(tgt)
        self.wq[k].copy_(torch.round(wgt * 4).to(torch.uint8))
        self.count.append(float(wgt.sum().item()))

    def __getitem__(self, k):
        self._feat[..., :NFEAT].copy_(self.feat[k])
        self._tgt.copy_(self.tgt[k])
        self._wgt.copy_(self.wq[k].to(torch.float32) * 0.25)
        return self._feat, self._tgt, self._wgt, self.count[k]


def collect_runs(cfgs, n_steps, store, every=1, device="cuda"):
    """Fills `store` with pairs from the SIMPLE runs of `cfgs` (one after the
    other, `n_steps` time steps each, every `every`-th outer iteration),
    stopping when it is full; returns the pairs taken per run."""
    from .channel import ChannelSolver
    taken = []
    for cfg in cfgs:
        if store.full():
            break
        solver = ChannelSolver(cfg, device=device, precision="mixed")
        NX, NY = solver.b_p.shape
        fz = Featurizer(NX, NY, solver.device)
        assert (fz.Hh, fz.Wh) == (store.Hh, store.Wh), "every run must have the store's grid"
        k = before = len(store)
        for _ in range(n_steps):
            for _ in range(solver.cfg.max_outer):
                solver.assemble_momentum()
                solver.solve_momentum()
                solver.relax()
                solver.assemble_p()
                take = k % every == 0 and not store.full()
                if take:
                    feat = fz(solver.b_p, solver.coef_p32)
                    scales = fz.scales.clone()
                solver.solve_p()
                if take:
                    fz.scales.copy_(scales)
                    tgt, wgt = fz.target(solver.pcor, solver.coef_p32)
                    store.add(feat, tgt, wgt)
                k += 1
                solver.correct()
                if float(solver.mass[0].item()) <= solver.cfg.mass_tol:
                    break
            solver.time_forward()
            if store.full():
                break
        taken.append(len(store) - before)
        del solver, fz
        torch.cuda.empty_cache()
    return taken


def training_configs(base, n, seed=0):
    """Channels of the 2048 x 512 kind for the training set: the base grid and
    inlet, the cylinder's diameter (24-40 cells), centre (x 300-500, y 256 +- 26)
    and Re (100-200) drawn per run, per-run initial noise (seeds from 100:
    the benchmark's seed 0 and the default training seed 7 are not among them)."""
    rng = np.random.default_rng(seed)
    out = []
    for r in range(n):
        D = int(rng.integers(24, 41))
        ci = int(rng.integers(300, 501))
        cj = int(256 + rng.integers(-26, 27))
        Re = float(rng.uniform(100.0, 200.0))
        out.append(base.with_(name=base.name, D=D, obstacles=(("circle", ci, cj, D),), Re=Re, seed=100 + r))
    return out


def train(net, pairs, steps, lr=1e-3, batch=4, seed=0, log_every=0):
    """Adam on the mean squared error over fluid cells: `batch` pairs per step
    (gradients accumulated), learning rate on a cosine schedule."""
    rng = np.random.default_rng(seed)
    hist = []
    for it in range(steps):
        net.zero_grad()
        loss_sum = None
        for _ in range(batch):
            feat, tgt, wgt, count = pairs[int(rng.integers(len(pairs)))]
            out = net.forward(feat)
            loss, dout = net.mse(out, tgt, wgt, count * batch)
            net.backward(dout)
            loss_sum = loss if loss_sum is None else loss_sum + loss
        net.adam_step(lr * 0.5 * (1.0 + np.cos(np.pi * it / max(steps, 1))))
        if log_every and (it % log_every == 0 or it == steps - 1):
            hist.append((it, float(loss_sum.item())))
    return hist


def mean_loss(net, pairs):
    """Mean squared error of the prediction over the pairs' fluid cells."""
    tot = 0.0
    for feat, tgt, wgt, count in pairs:
        out = net.forward(feat)
        loss, _ = net.mse(out, tgt, wgt, count)
        tot += float(loss.item())
    return tot / max(len(pairs), 1)


def weights_path(config_name):
    return os.path.join(WEIGHTS_DIR, f"unet_{config_name}.npz")


def available(config_name="channel_2048x512"):
    return os.path.exists(weights_path(config_name))


def make_channel_solver(cfg, device):
    """The accelerated channel solver with the trained initial guess."""
    from .channel import ChannelSolver
    net = UNet.load(weights_path(cfg.name), device=device)
    return ChannelSolver(cfg, device=device, precision="mixed", learned=LearnedGuess(net))


def main(argv=None):
    """python -m karman_taichi_gb300.learned --config channel_2048x512 --steps-sim 20 --train-steps 1500
    python -m karman_taichi_gb300.learned --pairs 20000 --runs 24 --steps-sim 150 --train-steps 5000"""
    import argparse
    from .channel import ChannelSolver
    from .config import get
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="channel_2048x512")
    ap.add_argument("--steps-sim", type=int, default=20, help="SIMPLE time steps that generate training pairs")
    ap.add_argument("--train-steps", type=int, default=1500)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=7,
                    help="seed of the initial-state noise of the training run (the benchmark runs seed 0)")
    ap.add_argument("--out", default=None)
    ap.add_argument("--pairs", type=int, default=0,
                    help="collect this many pairs from --runs varied channels of the config's grid into an "
                         "on-device store (0: the pairs of one run of --steps-sim steps)")
    ap.add_argument("--runs", type=int, default=24)
    a = ap.parse_args(argv)
    cfg = get(a.config).with_(seed=a.seed)
    dev = torch.device("cuda", 0)
    t0 = time.time()
    if a.pairs > 0:
        probe = Featurizer(cfg.nx + 2, cfg.ny + 2, dev)
        pairs = PairStore(a.pairs, probe.Hh, probe.Wh, dev)
        del probe
        taken = collect_runs(training_configs(get(a.config), a.runs), a.steps_sim, pairs, device=dev)
        torch.cuda.synchronize()
        print(f"{len(pairs)} pairs from {len(taken)} runs of up to {a.steps_sim} time steps {taken} in "
              f"{time.time() - t0:.1f} s", flush=True)
        held = [pairs[int(k)] for k in np.linspace(0, len(pairs) - 1, 8).astype(int)]
        sample = lambda: [(f.clone(), t.clone(), w.clone(), c) for f, t, w, c in held]
    else:
        solver = ChannelSolver(cfg, device=dev, precision="mixed")
        pairs = collect_pairs(solver, a.steps_sim)
        torch.cuda.synchronize()
        print(f"{len(pairs)} pairs from {a.steps_sim} time steps (seed {a.seed}) in {time.time() - t0:.1f} s",
              flush=True)
        sample = lambda: pairs
    net = UNet(dev, seed=0)
    before = mean_loss(net, sample())
    t0 = time.time()
    hist = train(net, pairs, a.train_steps, lr=a.lr, log_every=max(1, a.train_steps // 10))
    torch.cuda.synchronize()
    print(f"trained {a.train_steps} steps in {time.time() - t0:.1f} s: mean loss {before:.4g} -> "
          f"{mean_loss(net, sample()):.4g} (on {len(sample())} pairs); {hist}", flush=True)
    path = a.out or weights_path(cfg.name)
    net.save(path)
    print("saved", path, flush=True)


if __name__ == "__main__":
    main()
