"""Jacobi sweeps (pressure_valid.py:192-233, debug/20210828_karman_taihi.py:375-393):
kc_jacobi against the NumPy restatement, and Jacobi iterations converging to
the direct solution of a diagonally dominant system."""
import numpy as np
import pytest

from oracle import np_oracle as O


def test_restatement_converges_to_direct_solution():
    import scipy.sparse.linalg as spla
    rng = np.random.default_rng(0)
    NX, S = 20, 12
    c = rng.uniform(-1, 0, (5, NX * S))
    c[0] = -(c[1] + c[2] + c[3] + c[4]) + 0.5     # strictly diagonally dominant
    b = rng.standard_normal(NX * S)
    x = np.zeros(NX * S)
    for _ in range(400):
        x, d = O.jacobi_sweep(c, b, x, S)
    xs = spla.spsolve(O.to_csr(c, S).tocsc(), b)
    assert np.abs(x - xs).max() <= 1e-10 * np.abs(xs).max() and d < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("omega,region", [(1.0, None), (0.7, (2, 17, 1, 11))])
def test_kc_jacobi_matches_restatement(dev, omega, region):
    import torch
    from karman_taichi_gb300 import linalg
    rng = np.random.default_rng(1)
    NX, S = 19, 13
    c = rng.uniform(-1, 0, (5, NX, S))
    c[0] = -(c[1] + c[2] + c[3] + c[4]) + 0.3
    c[0, 5, 5] = 0.0                              # a zero diagonal is skipped
    b = rng.standard_normal((NX, S))
    x = rng.standard_normal((NX, S))
    t = lambda a: torch.from_numpy(a).to(dev)
    y = torch.empty_like(t(x))
    d = linalg.jacobi(linalg.Stencil(t(c)), t(b), t(x), y, omega=omega, region=region)
    yr, dr = O.jacobi_sweep(c, b, x, S, omega, region)
    assert np.abs(y.cpu().numpy().reshape(-1) - yr).max() <= 1e-14 * np.abs(yr).max()
    assert abs(float(d.item()) - dr) <= 1e-14 * dr


@pytest.mark.gpu
def test_simple_jacobi_paths_run(dev):
    from karman_taichi_gb300.simple import SIMPLESolver
    s = SIMPLESolver(1.0, 1.0, 16, 16, device=dev)
    s.init()
    d = s.jacob_solve_momentum_eqn(3)
    assert len(d) == 3 and all(np.isfinite(d))
    s.compute_coef_p()
    res, k = s.jacob_solve_pcorrection_eqn(1e-12, max_iter=50)
    assert k >= 1 and np.isfinite(res)
