"""Synthetic inputs of the benchmark configurations that are not a channel.

``pcorr_random_system`` is the isolated pressure-correction system of the
1024 x 1024 configuration: the reference's p' operator (face coefficients
rho dy^2 / aP_face, simple.py:150-156) with aP_face drawn log-uniform in
[1, 10], a random 5 % of the cells blocked in square blobs of side 4-16
(identity rows, links into them removed), p' pinned to zero at the first
fluid cell as bicgsimp.py:146-151 pins (1, 1), and a right-hand side that is
the divergence of a seeded Gaussian face velocity smoothed by a 5 x 5 box
filter, with its mean over the fluid removed.  Host-side NumPy, seeded: the
same arrays on every machine.
"""
from __future__ import annotations

import numpy as np


def pcorr_random_system(N=1024, seed=0, blocked=0.05):
    """Returns (coef [5][N+2][N+2] standard form FP64, b [N+2][N+2] FP64)."""
    rng = np.random.default_rng(seed)
    NX = NY = N + 2
    solid = np.zeros((NX, NY), dtype=bool)
    while solid[1:-1, 1:-1].sum() < blocked * N * N:
        s = int(rng.integers(4, 17))
        i0, j0 = int(rng.integers(1, N - s + 2)), int(rng.integers(1, N - s + 2))
        solid[i0:i0 + s, j0:j0 + s] = True
    fluid = np.zeros((NX, NY), dtype=bool)
    fluid[1:-1, 1:-1] = ~solid[1:-1, 1:-1]
    # face links: east faces between (i, j) and (i+1, j), north faces between (i, j) and (i, j+1)
    east = np.zeros((NX, NY))
    north = np.zeros((NX, NY))
    east[1:N, 1:N + 1] = 1.0 / np.exp(rng.uniform(0.0, np.log(10.0), (N - 1, N)))
    north[1:N + 1, 1:N] = 1.0 / np.exp(rng.uniform(0.0, np.log(10.0), (N, N - 1)))
    east[:-1] *= fluid[:-1] & fluid[1:]
    north[:, :-1] *= fluid[:, :-1] & fluid[:, 1:]
    pin = tuple(np.argwhere(fluid)[0])
    c = np.zeros((5, NX, NY))
    c[2, :-1] = -east[:-1]
    c[1, 1:] = -east[:-1]
    c[3, :, :-1] = -north[:, :-1]
    c[4, :, 1:] = -north[:, :-1]
    c[0] = -(c[1] + c[2] + c[3] + c[4])
    c[:, ~fluid] = 0.0
    c[0][solid] = 1.0
    c[:, pin[0], pin[1]] = 0.0
    c[0, pin[0], pin[1]] = 1.0

    def box5(a):
        p = np.pad(a, 2, mode="edge")
        out = np.zeros_like(a)
        for di in range(5):
            for dj in range(5):
                out += p[di:di + a.shape[0], dj:dj + a.shape[1]]
        return out / 25.0

    u = box5(rng.standard_normal((NX + 1, NY)))
    v = box5(rng.standard_normal((NX, NY + 1)))
    b = (u[:-1] - u[1:]) + (v[:, :-1] - v[:, 1:])
    b[~fluid] = 0.0
    b[pin] = 0.0
    m = fluid.copy()
    m[pin] = False
    b[m] -= b[m].mean()
    return c, b
