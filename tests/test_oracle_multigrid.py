"""The restated multigrid cycle (the oracle the GPU V-cycle is checked against)
is a symmetric positive-definite operator -- what CG needs of its
preconditioner -- for one, two and three red-black sweeps on the levels below
level 0, and its coarse levels follow the 2x2 aggregation sizes."""
import numpy as np
import pytest

from oracle import np_oracle as O


def _poisson(NX, NY):
    """Standard-form 5-point Poisson rows on a padded [NX][NY] grid: empty halo
    rows, Neumann walls, Dirichlet through the east halo (a channel outlet)."""
    c = np.zeros((5, NX, NY))
    inner = np.zeros((NX, NY), dtype=bool)
    inner[1:NX - 1, 1:NY - 1] = True
    ii, jj = np.nonzero(inner)
    for q, (di, dj) in zip((1, 2, 3, 4), ((-1, 0), (1, 0), (0, 1), (0, -1))):
        ni, nj = ii + di, jj + dj
        link = inner[ni, nj] | (ni == NX - 1)
        c[q, ii, jj] = np.where(link, -1.0, 0.0)
    c[0, ii, jj] = -(c[1] + c[2] + c[3] + c[4])[ii, jj]
    return c


@pytest.mark.parametrize("nu_coarse", [1, 2, 3])
def test_cycle_is_symmetric_positive_definite(nu_coarse):
    NX, NY = 42, 26
    c = _poisson(NX, NY)
    c32 = O.to_laplacian32(c.reshape(5, -1))
    mg = O.MultigridOracle(c32, NX, NY, lap=True, nu_coarse=nu_coarse)
    assert mg.inv is not None and len(mg.levels) >= 3
    interior = np.zeros((NX, NY), dtype=bool)
    interior[1:NX - 1, 1:NY - 1] = True
    rng = np.random.default_rng(nu_coarse)
    for _ in range(3):
        r1 = np.where(interior, rng.standard_normal((NX, NY)), 0.0).astype(np.float32).reshape(-1)
        r2 = np.where(interior, rng.standard_normal((NX, NY)), 0.0).astype(np.float32).reshape(-1)
        z1, z2 = mg.apply(r1).astype(np.float64), mg.apply(r2).astype(np.float64)
        a, b = z1 @ r2, r1 @ z2
        assert abs(a - b) <= 2e-5 * (np.linalg.norm(z1) * np.linalg.norm(r2)), (a, b)
        assert z1 @ r1 > 0


def test_more_coarse_sweeps_make_a_stronger_cycle():
    """On the same system a cycle with more sweeps below level 0 leaves less of
    a residual after one application (x = M b, ||b - A x||)."""
    NX, NY = 66, 34
    c = _poisson(NX, NY)
    A = O.to_csr(c.reshape(5, -1), NY)
    c32 = O.to_laplacian32(c.reshape(5, -1))
    interior = np.zeros((NX, NY), dtype=bool)
    interior[1:NX - 1, 1:NY - 1] = True
    b = np.where(interior, np.random.default_rng(0).standard_normal((NX, NY)), 0.0).reshape(-1)
    res = []
    for nu in (1, 2, 3):
        mg = O.MultigridOracle(c32, NX, NY, lap=True, nu_coarse=nu, omega=(1.0, 1.1))
        x = mg.apply(b.astype(np.float32)).astype(np.float64)
        res.append(np.linalg.norm(b - A @ x) / np.linalg.norm(b))
    assert res[2] < res[1] < res[0], res


def test_levels_follow_two_by_two_aggregation():
    mg = O.MultigridOracle(O.to_laplacian32(_poisson(98, 42).reshape(5, -1)), 98, 42, lap=True)
    dims = [(L["NX"], L["NY"]) for L in mg.levels]
    for (a, b), (c, d) in zip(dims, dims[1:]):
        assert (c, d) == ((a + 1) // 2, (b + 1) // 2)
    assert dims[-1][0] * dims[-1][1] <= O.MultigridOracle.COARSEST_DIRECT < dims[-2][0] * dims[-2][1]
