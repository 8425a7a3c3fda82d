"""Initial guesses of the p' solves by projection onto earlier solutions
(kc_recycle_guess, the native step's `recycle` option).

The guess x0 = Z y with (Z^T A Z) y = Z^T b is checked against the same
projection in NumPy (1e-10 relative), dependent vectors are dropped, and on a
channel the accelerated path with recycling reaches the same fields as without
(both solve every p' system to ||b - A x|| / ||b|| < 1e-8: 1e-6 relative)
with fewer CG iterations.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _spd(N, seed):
    rng = np.random.default_rng(seed)
    c = np.zeros((5, N, N))
    w = rng.uniform(0.5, 2.0, (N + 1, N))
    h = rng.uniform(0.5, 2.0, (N, N + 1))
    c[1] = -w[:N]; c[2] = -w[1:]; c[3] = -h[:, 1:]; c[4] = -h[:, :N]
    c[1, 0] = 0; c[2, -1] = 0; c[3, :, -1] = 0; c[4, :, 0] = 0
    c[0] = -c[1:].sum(axis=0) + 0.1
    return c


def _guess(dev, c, b, Z):
    import torch
    from karman_taichi_gb300 import _lib as L, linalg
    lib = L.load()
    N = c.shape[1]
    A = linalg.Stencil(torch.from_numpy(c).to(dev))
    bt = torch.from_numpy(b).to(dev)
    zt = [torch.from_numpy(z).to(dev) for z in Z]
    x0 = torch.zeros_like(bt)
    ws = torch.zeros(lib.kc_recycle_ws_bytes(N * N, len(Z)) + 256, dtype=torch.uint8, device=dev)
    off = (-ws.data_ptr()) % 256
    ptrs = (C.c_void_p * max(len(Z), 1))(*[z.data_ptr() for z in zt])
    used = C.c_int(-1)
    L.check(lib.kc_recycle_guess(C.byref(A.system), bt.data_ptr(), ptrs, len(Z), x0.data_ptr(),
                                 ws.data_ptr() + off, ws.numel() - off, C.byref(used), linalg.stream_handle(dev)),
            "kc_recycle_guess")
    return x0.cpu().numpy(), used.value


def test_recycle_guess_is_the_galerkin_projection(dev):
    from oracle import np_oracle as O
    N = 48
    c = _spd(N, 1)
    rng = np.random.default_rng(2)
    b = rng.standard_normal(N * N)
    Z = [rng.standard_normal(N * N) for _ in range(3)]
    x0, used = _guess(dev, c, b, Z)
    A = O.to_csr(c.reshape(5, -1), N)
    Zm = np.stack(Z, 1)
    y = np.linalg.solve(Zm.T @ (A @ Zm), Zm.T @ b)
    ref = Zm @ y
    assert used == 3
    assert np.abs(x0 - ref).max() <= 1e-10 * np.abs(ref).max()
    # the guess of the exact solution's span is the solution
    xs = np.linalg.solve(A.toarray(), b)
    x1, _ = _guess(dev, c, b, [xs, Z[0]])
    assert np.abs(x1 - xs).max() <= 1e-9 * np.abs(xs).max()


def test_recycle_drops_dependent_vectors(dev):
    N = 32
    c = _spd(N, 3)
    rng = np.random.default_rng(4)
    b = rng.standard_normal(N * N)
    z = rng.standard_normal(N * N)
    x0, used = _guess(dev, c, b, [z, 2.0 * z, rng.standard_normal(N * N)])
    assert used == 1          # the second vector repeats the first: it and the older ones are dropped
    x1, _ = _guess(dev, c, b, [z])
    assert np.abs(x0 - x1).max() <= 1e-12 * np.abs(x1).max()
    x2, used2 = _guess(dev, c, b, [])
    assert used2 == 0 and not x2.any()


def test_recycling_keeps_the_fields_and_saves_iterations(dev):
    from karman_taichi_gb300.channel import ChannelSolver
    from karman_taichi_gb300.config import ChannelConfig
    cfg = ChannelConfig("rc", 256, 64, 1.0 / 64, 8, (("circle", 64, 32, 8),), max_outer=20)
    a = ChannelSolver(cfg, device=dev, precision="mixed", recycle=4)
    b = ChannelSolver(cfg, device=dev, precision="mixed", recycle=0)
    ita = itb = 0
    for _ in range(3):
        ra, rb = a.step(), b.step()
        ita += ra[0]["it_p"]
        itb += rb[0]["it_p"]
        assert abs(ra[0]["outer"] - rb[0]["outer"]) <= 1
    assert a.fallbacks == b.fallbacks == 0
    sa, sb = a.state_numpy(), b.state_numpy()
    for k in ("u", "v", "p"):
        assert np.abs(sa[k] - sb[k]).max() <= 1e-6 * np.abs(sb[k]).max(), k
    assert ita < 0.85 * itb, (ita, itb)
    print(f"CG iterations over 3 steps: {ita} with recycling, {itb} without")
