"""Pins the CPU oracle against the reference's own known-answer tests
(restated with seeded inputs) and against SciPy / NumPy direct solves.

Reference tests restated here:
* debug/ti_bicg_test.py:21-98  random diagonally dominant 5-diagonal matrix
  (offsets +-1, +-3, diag = -sum(off) + 0.1, n = 320) vs np.linalg.solve
* benchmark/cg_to_sparse/validation.py:7-45  BiCGSTAB convergence vs
  scipy.sparse.linalg.bicgstab (the removed ``tol=`` becomes ``rtol=``)
* benchmark/cg_to_sparse/test_cg_sparse.py:10-41 and benchmark/test_2dcg_oop.py
  Laplacian + 0.1 I, RHS sin*sin, CG / BiCGSTAB vs a direct sparse solve
* benchmark/2dcg.py:129-132  np.allclose(A x, b)
"""
import math

import numpy as np
import pytest
import scipy.sparse.linalg as spla

from oracle import np_oracle as O


def _kat_5diag(n=320, seed=0):
    rng = np.random.default_rng(seed)
    S = 3
    A = rng.random((n, n))
    for i in range(n):
        for j in range(n):
            if i == j:
                continue
            if abs(i - j) in (1, 3):
                A[i, j] *= -1
            else:
                A[i, j] = 0.0
    for i in range(n):
        A[i, i] = -(A[i].sum() - A[i, i]) + 0.1
    b = rng.random(n)
    # the same matrix as flat 5-point planes
    c = np.zeros((5, n))
    k = np.arange(n)
    c[0] = np.diag(A)
    for comp, off in ((1, -S), (2, S), (3, 1), (4, -1)):
        ok = (k + off >= 0) & (k + off < n)
        c[comp][ok] = A[k[ok], k[ok] + off]
    return A, b, c, S


def _laplacian(N, offset=0.1):
    c = np.zeros((5, N, N))
    c[0] = 4.0 + offset
    c[1, 1:, :] = -1.0
    c[2, :-1, :] = -1.0
    c[3, :, :-1] = -1.0
    c[4, :, 1:] = -1.0
    return c.reshape(5, -1)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_ti_bicg_kat(seed):
    A, b, c, S = _kat_5diag(seed=seed)
    assert np.allclose(O.to_csr(c, S).toarray(), A)
    xs = np.linalg.solve(A, b)
    assert np.allclose(A @ xs, b)
    r = O.bicgstab(c, b, S, eps=1e-8, max_iter=100 * b.size)
    assert r.status == O.OK
    assert np.allclose(r.x, xs)


def test_spmv_orders_agree_and_match_scipy():
    rng = np.random.default_rng(3)
    n, S = 5000, 70
    c = rng.standard_normal((5, n))
    x = rng.standard_normal(n)
    y1 = O.spmv(c, x, S, "simple")
    y2 = O.spmv(c, x, S, "karman")
    y3 = O.to_csr(c, S) @ x
    assert np.allclose(y1, y3, rtol=1e-13, atol=1e-12)
    assert np.allclose(y2, y3, rtol=1e-13, atol=1e-12)


def test_bicgstab_vs_scipy_validation():
    """validation.py: BICGPoissonSolver(64, 1e-6, offset 0) vs SciPy bicgstab."""
    N = 64
    c = _laplacian(N, 0.0)
    xl = np.arange(N) * 2.0 / N
    b = (np.sin(2 * np.pi * xl)[:, None] * np.sin(2 * np.pi * xl)[None, :]).reshape(-1)
    r = O.bicgstab(c, b, N, eps=1e-6)
    xs, info = spla.bicgstab(O.to_csr(c, N), b, rtol=1e-6)
    assert r.status == O.OK and info == 0
    assert np.linalg.norm(r.x - xs) <= 1e-4 * np.linalg.norm(xs)


@pytest.mark.parametrize("solver", ["cg", "bicgstab"])
def test_poisson_vs_direct(solver):
    """test_cg_sparse.py / test_2dcg_oop.py: Laplacian + 0.1 I vs LU."""
    N = 128
    c = _laplacian(N, 0.1)
    xl = np.arange(N) * 2.0 / N
    b = (np.sin(2 * np.pi * xl)[:, None] * np.sin(2 * np.pi * xl)[None, :]).reshape(-1)
    xs = spla.spsolve(O.to_csr(c, N).tocsc(), b)
    r = (O.cg if solver == "cg" else O.bicgstab)(c, b, N, eps=1e-12)
    assert r.status == O.OK
    assert np.abs(r.x - xs).max() <= 1e-9 * np.abs(xs).max()
    assert np.allclose(O.spmv(c, r.x, N), b)      # 2dcg.py:129-132


def test_cg_history_and_zero_rhs():
    N = 16
    c = _laplacian(N)
    r = O.cg(c, np.zeros(N * N), N)
    assert r.status == O.OK and r.iters == 0
    b = np.ones(N * N)
    r = O.cg(c, b, N, eps=1e-10)
    assert r.history[0] == pytest.approx(math.sqrt(N * N))
    assert len(r.history) == r.iters


def test_refined_emulation_reaches_fp64_tolerance():
    N = 64
    c = _laplacian(N, 0.01)
    b = np.random.default_rng(0).standard_normal(N * N)
    r = O.bicgstab_refined(c, b, N, eps=1e-10, eps_inner=1e-3)
    res = b - O.spmv(c, r.x, N)
    assert np.linalg.norm(res) / np.linalg.norm(b) < 1e-10


def test_channel_oracle_correction_enforces_continuity():
    """After the correction step the mass residual equals the p' solve's
    residual, so it drops far below the predicted field's residual."""
    nx, ny = 48, 16
    solid = O.channel_solid_mask(nx, ny, [("square", 16, 8, 4)])
    P = O.ChannelParams(nx=nx, ny=ny, dx=1 / 16, dy=1 / 16, rho=1.0, mu=4 / 16 / 150, dt=0.5 / 16)
    from karman_taichi_gb300 import geometry
    u, v, p = geometry.channel_initial_fields(nx, ny, solid)
    orc = O.ChannelOracle(P, solid, u, v, p)
    s = orc.outer_iteration()
    assert s["st"] == (O.OK, O.OK, O.OK)
    assert orc.mass_residual() < 1e-6 * s["mass"]
    # inflow = outflow up to the p' solve's residual after the correction
    J = slice(1, ny + 1)
    assert abs(orc.u[1, J].sum() - orc.u[nx + 1, J].sum()) < 1e-6 * orc.u[1, J].sum()


def test_karman_oracle_geometry():
    o = O.KarmanOracle(nx=320, ny=64)
    ct = o.ct
    assert (ct[0, :] == 1).all() and (ct[-1, :] == 1).all() and (ct[:, 0] == 1).all() and (ct[:, -1] == 1).all()
    ii, jj = np.nonzero(ct[1:-1, 1:-1] == 1)
    assert len(ii) == sum(1 for i in range(320) for j in range(64) if (i - 64) ** 2 + (j - 32) ** 2 < 144
                          and 1 <= i <= 320 and 1 <= j <= 64)
    assert o.p[0, 0] == 100.0 and o.p[320, 5] == pytest.approx(100 - 4000.0)
