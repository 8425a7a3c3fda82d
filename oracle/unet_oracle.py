"""CPU restatement of the learned initial guess's U-Net (test infrastructure).

Only tests import this module: it is the checker of the GPU U-Net kernels
(karman_taichi_gb300/csrc/kc_unet.cu) and of karman_taichi_gb300/learned.py,
never a product path.  The reference has no learned component, so there is
no reference file to cite; the network is the one the accelerated path
specifies (4 levels, 16/32/48/64 channels, 3x3 convolutions, ReLU, 2x2
average pooling, nearest upsampling with skip concatenation, 1x1 head).

With ``bf16=True`` every stored activation, gradient of an activation and
convolution weight is rounded to bfloat16 (round to nearest even) at the
points where the GPU stores it, products and sums are FP32 -- so GPU and
oracle differ only in summation order.  With ``bf16=False`` and float64
arrays it is plain differentiable arithmetic, which the finite-difference
test pins.
"""
from __future__ import annotations

import numpy as np

CH = (16, 32, 48, 64)
CIN = 16   # padded input features


def to_bf16(a):
    """Round float32 values to bfloat16 precision (nearest even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32).copy()
    out[np.isnan(a)] = np.nan
    return out


def layer_specs():
    """(name, cin_padded, cin_real, cout) of every 3x3 convolution, in order."""
    c0, c1, c2, c3 = CH
    return [("e0a", CIN, CIN, c0), ("e0b", c0, c0, c0),
            ("e1a", c0, c0, c1), ("e1b", c1, c1, c1),
            ("e2a", c1, c1, c2), ("e2b", c2, c2, c2),
            ("b3a", c2, c2, c3), ("b3b", c3, c3, c3),
            ("d2a", c3 + c2, c3 + c2, c2), ("d2b", c2, c2, c2),
            ("d1a", c2 + c1, c2 + c1, c1), ("d1b", c1, c1, c1),
            ("d0a", c1 + c0, c1 + c0, c0), ("d0b", c0, c0, c0)]


def init_params(seed=0, n_features=4):
    """He-normal 3x3 weights [9][cout][cin], zero biases, a small 1x1 head."""
    rng = np.random.default_rng(seed)
    P = {}
    for name, cin, cin_real, cout in layer_specs():
        fan_in = 9 * (n_features if name == "e0a" else cin_real)
        w = rng.standard_normal((9, cout, cin)).astype(np.float32) * np.float32(np.sqrt(2.0 / fan_in))
        if name == "e0a":
            w[:, :, n_features:] = 0.0
        P[name + ".w"] = w
        P[name + ".b"] = np.zeros(cout, dtype=np.float32)
    P["head.w"] = (rng.standard_normal(CH[0]) * 0.1).astype(np.float32)
    P["head.b"] = np.zeros(1, dtype=np.float32)
    return P


class UNetOracle:
    def __init__(self, params, bf16=True, dtype=np.float32):
        self.bf16 = bf16
        self.dt = dtype
        self.P = {k: np.asarray(v, dtype=dtype) for k, v in params.items()}

    def _r(self, a):
        return to_bf16(a) if self.bf16 else np.asarray(a, dtype=self.dt)

    def _w(self, name):
        w = self.P[name + ".w"]
        return to_bf16(w) if self.bf16 else w

    @staticmethod
    def _shift(x, dy, dx):
        """x shifted so out[i, j] = x[i + dy, j + dx] (zero outside)."""
        H, W = x.shape[:2]
        out = np.zeros_like(x)
        i0, i1 = max(0, -dy), min(H, H - dy)
        j0, j1 = max(0, -dx), min(W, W - dx)
        out[i0:i1, j0:j1] = x[i0 + dy:i1 + dy, j0 + dx:j1 + dx]
        return out

    def conv(self, x, w, b=None, relu=False, mask=None):
        """y[i,j,co] = sum_tap,ci x[i+ky-1, j+kx-1, ci] w[tap, co, ci] (+ b), rounded like the GPU."""
        H, W, _ = x.shape
        y = np.zeros((H, W, w.shape[1]), dtype=self.dt)
        for tap in range(9):
            ky, kx = divmod(tap, 3)
            y += self._shift(x, ky - 1, kx - 1) @ w[tap].T
        if b is not None:
            y = y + b
        if relu:
            y = np.maximum(y, 0)
        if mask is not None:
            y = np.where(mask > 0, y, 0)
        return self._r(y)

    @staticmethod
    def flip(w):
        """Data-gradient weights: wt[tap'][ci][co] = w[8 - tap'][co][ci]."""
        return np.ascontiguousarray(w[::-1].transpose(0, 2, 1))

    def pool(self, x):
        H, W, C = x.shape
        return self._r(x.reshape(H // 2, 2, W // 2, 2, C).sum(axis=(1, 3)) * 0.25)

    def up_concat(self, u, s):
        up = np.repeat(np.repeat(u, 2, axis=0), 2, axis=1)
        return np.concatenate([up, s], axis=2)

    def forward(self, feat):
        """feat [H][W][16] (H, W multiples of 8) -> out [H][W] (FP32) and the activation cache."""
        A = {"in": self._r(feat)}
        c = lambda name, x: self.conv(x, self._w(name), self.P[name + ".b"], relu=True)
        A["e0a"] = c("e0a", A["in"]); A["s0"] = c("e0b", A["e0a"]); A["x1"] = self.pool(A["s0"])
        A["e1a"] = c("e1a", A["x1"]); A["s1"] = c("e1b", A["e1a"]); A["x2"] = self.pool(A["s1"])
        A["e2a"] = c("e2a", A["x2"]); A["s2"] = c("e2b", A["e2a"]); A["x3"] = self.pool(A["s2"])
        A["b3a"] = c("b3a", A["x3"]); A["y3"] = c("b3b", A["b3a"])
        A["c2"] = self.up_concat(A["y3"], A["s2"])
        A["d2a"] = c("d2a", A["c2"]); A["y2"] = c("d2b", A["d2a"])
        A["c1"] = self.up_concat(A["y2"], A["s1"])
        A["d1a"] = c("d1a", A["c1"]); A["y1"] = c("d1b", A["d1a"])
        A["c0"] = self.up_concat(A["y1"], A["s0"])
        A["d0a"] = c("d0a", A["c0"]); A["y0"] = c("d0b", A["d0a"])
        out = A["y0"] @ self.P["head.w"] + self.P["head.b"][0]
        return out.astype(self.dt), A

    @staticmethod
    def mse(out, target, weight):
        n = float(np.count_nonzero(weight))
        d = (out - target) * weight
        return float((d * d).sum() / n), (2.0 * d * weight / n).astype(out.dtype)

    def _wgrad(self, x, dy):
        dw = np.zeros((9, dy.shape[2], x.shape[2]), dtype=self.dt)
        for tap in range(9):
            ky, kx = divmod(tap, 3)
            xs = self._shift(x, ky - 1, kx - 1)
            dw[tap] = dy.reshape(-1, dy.shape[2]).T @ xs.reshape(-1, x.shape[2])
        return dw, dy.reshape(-1, dy.shape[2]).sum(axis=0)

    def backward(self, A, dout):
        """Gradients of all parameters for d loss / d out = dout."""
        G = {}
        G["head.w"] = (A["y0"].reshape(-1, CH[0]) * dout.reshape(-1, 1)).sum(axis=0)
        G["head.b"] = np.array([dout.sum()], dtype=self.dt)
        d = self._r(dout[..., None] * self.P["head.w"])
        d = np.where(A["y0"] > 0, d, 0)

        def conv_back(name, x_in, d_out, mask):
            G[name + ".w"], G[name + ".b"] = self._wgrad(x_in, d_out)
            return self.conv(d_out, self.flip(self._w(name)), mask=mask)

        d = conv_back("d0b", A["d0a"], d, A["d0a"])
        dc0 = conv_back("d0a", A["c0"], d, A["c0"])
        c1n, c0n = CH[1], CH[0]
        dy1 = self._r(dc0[..., :c1n].reshape(dc0.shape[0] // 2, 2, dc0.shape[1] // 2, 2, c1n).sum(axis=(1, 3)))
        ds0 = dc0[..., c1n:]
        d = conv_back("d1b", A["d1a"], dy1, A["d1a"])
        dc1 = conv_back("d1a", A["c1"], d, A["c1"])
        c2n = CH[2]
        dy2 = self._r(dc1[..., :c2n].reshape(dc1.shape[0] // 2, 2, dc1.shape[1] // 2, 2, c2n).sum(axis=(1, 3)))
        ds1 = dc1[..., c2n:]
        d = conv_back("d2b", A["d2a"], dy2, A["d2a"])
        dc2 = conv_back("d2a", A["c2"], d, A["c2"])
        c3n = CH[3]
        dy3 = self._r(dc2[..., :c3n].reshape(dc2.shape[0] // 2, 2, dc2.shape[1] // 2, 2, c3n).sum(axis=(1, 3)))
        ds2 = dc2[..., c3n:]
        d = conv_back("b3b", A["b3a"], dy3, A["b3a"])
        dx3 = conv_back("b3a", A["x3"], d, None)

        def pool_back(dx, ds, s):
            up = self._r(np.repeat(np.repeat(dx, 2, axis=0), 2, axis=1) * 0.25)
            return np.where(s > 0, self._r(up + ds), 0)

        d = pool_back(dx3, ds2, A["s2"])
        d = conv_back("e2b", A["e2a"], d, A["e2a"])
        dx2 = conv_back("e2a", A["x2"], d, None)
        d = pool_back(dx2, ds1, A["s1"])
        d = conv_back("e1b", A["e1a"], d, A["e1a"])
        dx1 = conv_back("e1a", A["x1"], d, None)
        d = pool_back(dx1, ds0, A["s0"])
        d = conv_back("e0b", A["e0a"], d, A["e0a"])
        self._wgrad_only("e0a", A["in"], d, G)
        return G

    def _wgrad_only(self, name, x_in, d_out, G):
        G[name + ".w"], G[name + ".b"] = self._wgrad(x_in, d_out)


# ---- features of the p' system, half-resolution target, upsampled guess --------------------
def features_np(b, coef32, H, W):
    """Restatement of kc_unet_features: returns (feat [H][W][16] float32 before
    bfloat16 rounding, fluid [NX][NY], scales (s_b, mean d, s_p, count))."""
    b = np.asarray(b, dtype=np.float64)
    c = np.asarray(coef32, dtype=np.float32)
    NX, NY = b.shape
    links = c[1:5]
    fluid = (links != 0).any(axis=0)
    fl = fluid.astype(np.float64)
    cnt = fl.sum()
    n = cnt if cnt > 0 else 1.0
    bf = b * fl
    d = -(links[0].astype(np.float64) + links[1] + links[2] + links[3]) * fl
    s_b = np.sqrt((bf * bf).sum() / n)
    d_mean = d.sum() / n
    F = np.cumsum(bf.sum(axis=1))
    A = (-c[2].astype(np.float64) * fl).sum(axis=1)
    step = np.where(A > 0, F / np.where(A > 0, A, 1.0), 0.0)
    P1 = np.cumsum(step[::-1])[::-1]
    s_p = np.sqrt((P1 * P1 * fl.sum(axis=1)).sum() / n)
    feat = np.zeros((H, W, CIN), dtype=np.float32)
    feat[:NX, :NY, 0] = np.where(fluid, b / s_b, 0)
    feat[:NX, :NY, 1] = fluid
    feat[:NX, :NY, 2] = np.where(fluid, d / d_mean, 0)
    feat[:NX, :NY, 3] = np.where(fluid, P1[:, None] / s_p, 0)
    return feat, fluid, np.array([s_b, d_mean, s_p, cnt])


def target_down2_np(p, fluid, s_p, Hh, Wh):
    """Restatement of kc_unet_target_down2."""
    NX, NY = p.shape
    tgt = np.zeros((Hh, Wh), dtype=np.float64)
    wgt = np.zeros((Hh, Wh), dtype=np.float64)
    pp = np.zeros((2 * Hh, 2 * Wh))
    ff = np.zeros((2 * Hh, 2 * Wh))
    pp[:NX, :NY] = np.where(fluid, p, 0)
    ff[:NX, :NY] = fluid
    s = pp.reshape(Hh, 2, Wh, 2).sum(axis=(1, 3))
    m = ff.reshape(Hh, 2, Wh, 2).sum(axis=(1, 3))
    tgt = np.where(m > 0, s / np.where(m > 0, m, 1) / s_p, 0)
    wgt = 0.25 * m
    return tgt, wgt


def guess_up2_np(out, fluid, s_p):
    """Restatement of kc_unet_guess_up2 (bilinear, coarse value of (I, J) at fine (2I + 1/2, 2J + 1/2))."""
    Hh, Wh = out.shape
    NX, NY = fluid.shape
    i = np.arange(NX)[:, None] * 0.5 - 0.25
    j = np.arange(NY)[None, :] * 0.5 - 0.25
    i0 = np.floor(i).astype(int)
    j0 = np.floor(j).astype(int)
    ti, tj = i - i0, j - j0
    cl = lambda a, n: np.clip(a, 0, n - 1)
    i1, j1 = cl(i0 + 1, Hh), cl(j0 + 1, Wh)
    i0, j0 = cl(i0, Hh), cl(j0, Wh)
    v = (1 - ti) * ((1 - tj) * out[i0, j0] + tj * out[i0, j1]) + ti * ((1 - tj) * out[i1, j0] + tj * out[i1, j1])
    return np.where(fluid, s_p * v, 0.0)
