"""Host-side geometry: blocked-cell masks, cell types and initial fields.

These are built once on the host (NumPy) and copied to the device; the masks
are compared bit for bit with the oracle's.
"""
from __future__ import annotations

import numpy as np


def solid_mask(nx: int, ny: int, obstacles) -> np.ndarray:
    """uint8 [nx+2, ny+2], 1 for a blocked cell.

    ``('square', ci, cj, D)`` blocks cells ``[c - D//2, c - D//2 + D - 1]`` in
    i and j; ``('circle', ci, cj, D)`` blocks cells with
    ``(i - ci)^2 + (j - cj)^2 < (D/2)^2``, the rule of karman_taichi.py:148-150
    (which is the D = 24 circle at (64, 32)).  Only interior cells
    ``[1, nx] x [1, ny]`` can be blocked.
    """
    m = np.zeros((nx + 2, ny + 2), dtype=np.uint8)
    for shape, ci, cj, D in obstacles:
        if shape == "square":
            i0, j0 = ci - D // 2, cj - D // 2
            i_lo, i_hi = max(i0, 1), min(i0 + D - 1, nx)
            j_lo, j_hi = max(j0, 1), min(j0 + D - 1, ny)
            if i_lo <= i_hi and j_lo <= j_hi:
                m[i_lo:i_hi + 1, j_lo:j_hi + 1] = 1
        elif shape == "circle":
            r2 = D * D / 4.0
            i = np.arange(1, nx + 1)[:, None]
            j = np.arange(1, ny + 1)[None, :]
            m[1:nx + 1, 1:ny + 1] |= (((i - ci) ** 2 + (j - cj) ** 2) < r2).astype(np.uint8)
        else:
            raise ValueError(f"unknown obstacle shape {shape!r}")
    return m


def blocked_faces(solid: np.ndarray):
    """(blocked_u [nx+3, ny+2], blocked_v [nx+2, ny+3]): a face is blocked when
    either neighbouring cell is."""
    s = solid.astype(bool)
    nx, ny = s.shape[0] - 2, s.shape[1] - 2
    bu = np.zeros((nx + 3, ny + 2), dtype=bool)
    bu[1:nx + 2, :] = s[0:nx + 1, :] | s[1:nx + 2, :]
    bv = np.zeros((nx + 2, ny + 3), dtype=bool)
    bv[:, 1:ny + 2] = s[:, 0:ny + 1] | s[:, 1:ny + 2]
    return bu, bv


def channel_initial_fields(nx: int, ny: int, solid: np.ndarray, U: float = 1.0, noise: float = 1e-3,
                           seed: int = 0):
    """u = U on every open u face, v = seeded uniform noise in [-noise, noise]
    on the interior v faces (walls and blocked faces 0), p = 0."""
    bu, bv = blocked_faces(solid)
    u = np.zeros((nx + 3, ny + 2))
    u[1:nx + 2, 1:ny + 1] = U
    u[bu] = 0.0
    v = np.zeros((nx + 2, ny + 3))
    rng = np.random.default_rng(seed)
    v[1:nx + 1, 2:ny + 1] = rng.uniform(-noise, noise, size=(nx, ny - 1))
    v[bv] = 0.0
    p = np.zeros((nx + 2, ny + 2))
    return u, v, p


def karman_cell_types(nx: int, ny: int, circle=(64, 32, 144)) -> np.ndarray:
    """int32 ct [nx+2, ny+2] of karman_taichi.py:143-150: 1 = solid ring and
    circle, -1 = fluid.  The circle test runs over i < nx, j < ny as in the
    reference."""
    ct = np.ones((nx + 2, ny + 2), dtype=np.int32)
    ct[1:nx + 1, 1:ny + 1] = -1
    ci, cj, r2 = circle
    i = np.arange(nx)[:, None]
    j = np.arange(ny)[None, :]
    sel = ((i - ci) ** 2 + (j - cj) ** 2) < r2
    sub = ct[:nx, :ny]
    sub[sel] = 1
    return ct


def karman_initial_pressure(nx: int, ny: int) -> np.ndarray:
    """p = 100 - 4000 i / nx (karman_taichi.py:132-135)."""
    i = np.arange(nx + 2, dtype=np.float64)[:, None] * np.ones((1, ny + 2))
    return 100 - 4000.0 * i / nx
