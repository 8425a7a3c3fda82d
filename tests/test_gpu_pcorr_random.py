"""The standalone 1024^2 pressure-correction system (log-uniform face
coefficients, 5% blocked blobs, pinned cell, smoothed-divergence right-hand
side): plain FP64 BiCGSTAB and the mixed-precision multigrid CG agree, and
both meet the FP64 residual tolerance.  Two solves stopped at a relative
residual eps differ by up to cond(A) eps, so both run to 1e-12 here and the
solutions are compared to 1e-6."""
import numpy as np
import pytest

from oracle import np_oracle as O

def test_pcorr_random_system_properties():
    c, b = O.pcorr_random_system(64, seed=1)
    fluid = (c[1:] != 0).any(axis=0)
    assert 0.03 < ((c[0] == 1) & ~fluid).sum() / 64 ** 2 < 0.2
    A = O.to_csr(c.reshape(5, -1), c.shape[2])
    rows = np.flatnonzero(fluid.reshape(-1))
    As = A[rows][:, rows]
    assert abs(As - As.T).max() == 0.0


@pytest.mark.gpu
def test_pcorr_random_1024_fp64_and_mixed_agree(dev):
    import torch
    from karman_taichi_gb300 import _lib as L, linalg
    c, b = O.pcorr_random_system(1024, seed=0)
    NX, NY = c.shape[1:]
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    A64 = linalg.Stencil(t(c))
    A32 = linalg.Stencil(t(O.to_laplacian32(c)), form=L.FORM_LAPLACIAN)
    bt = t(b)
    x1 = torch.zeros_like(bt)
    plain = linalg.bicgstab(A64, bt, x1, eps=1e-12, max_iter=A64.n)
    assert plain.ok, plain
    mg = linalg.Multigrid(A32).setup()
    x2 = torch.zeros_like(bt)
    acc = linalg.pcg_refined(A64, A32, bt, x2, mg, eps=1e-12)
    assert acc.ok, acc
    assert acc.iters * 20 < plain.iters, (acc.iters, plain.iters)
    for x in (x1, x2):
        xx = x.cpu().numpy().reshape(-1)
        res = b.reshape(-1) - O.spmv(c.reshape(5, -1), xx, NY)
        assert np.linalg.norm(res) / np.linalg.norm(b) < 1e-11
    a1, a2 = x1.cpu().numpy(), x2.cpu().numpy()
    assert np.abs(a1 - a2).max() <= 1e-6 * np.abs(a1).max()


def test_workload_generator_is_the_oracle_system():
    """bench.py builds the 1024 x 1024 system with the package's generator; it is the oracle's, array
    for array."""
    from karman_taichi_gb300.workloads import pcorr_random_system
    for N, seed in ((64, 1), (130, 4)):
        c1, b1 = pcorr_random_system(N, seed=seed)
        c2, b2 = O.pcorr_random_system(N, seed=seed)
        assert np.array_equal(c1, c2) and np.array_equal(b1, b2)
