"""GPU parity of the stencil solvers (C ABI via ctypes) against the CPU oracle.

Tolerances: FP64 SpMV <= 1e-13 relative (only FMA contraction differs);
FP64 solves agree with the oracle / direct solves to <= 1e-6 relative, the
field tolerance of the FP64 path; FP32 SpMV <= 1e-5 relative.
"""
import ctypes
import math

import numpy as np
import pytest

from oracle import np_oracle as O

pytestmark = pytest.mark.gpu


def _rand_system(n, S, seed, diag_shift=0.1, dtype=np.float64):
    rng = np.random.default_rng(seed)
    c = np.zeros((5, n))
    k = np.arange(n)
    for comp, off in ((1, -S), (2, S), (3, 1), (4, -1)):
        ok = (k + off >= 0) & (k + off < n)
        c[comp][ok] = -rng.random(n)[ok]
    c[0] = -(c[1] + c[2] + c[3] + c[4]) + diag_shift
    return c.astype(dtype)


def _laplacian(N, offset=0.1):
    """5-point Laplacian + offset on an N x N grid (benchmark/cg_to_sparse/
    cgsolver.py compute_Ap: (4 + offset) x - neighbours, zero outside)."""
    n = N * N
    c = np.zeros((5, N, N))
    c[0] = 4.0 + offset
    c[1, 1:, :] = -1.0
    c[2, :-1, :] = -1.0
    c[3, :, :-1] = -1.0
    c[4, :, 1:] = -1.0
    return c.reshape(5, n)


def _t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


@pytest.mark.parametrize("n,S", [(1, 1), (7, 3), (320, 3), (1000, 33), (514 * 40 + 17, 514), (4096, 64),
                                 (5000, 1), (3 * 5000, 5000)])
def test_spmv_f64_matches_oracle(dev, n, S):
    from karman_taichi_gb300 import linalg
    c = _rand_system(n, S, seed=n + S)
    x = np.random.default_rng(3).standard_normal(n)
    y = linalg.spmv(linalg.Stencil(_t(c, dev), stride=S), _t(x, dev)).cpu().numpy()
    ref = O.spmv(c, x, S)
    assert np.abs(y - ref).max() <= 1e-13 * max(np.abs(ref).max(), 1.0)


def test_spmv_f32(dev):
    from karman_taichi_gb300 import linalg
    n, S = 9000, 90
    c = _rand_system(n, S, seed=5).astype(np.float32)
    x = np.random.default_rng(4).standard_normal(n).astype(np.float32)
    y = linalg.spmv(linalg.Stencil(_t(c, dev), stride=S), _t(x, dev)).cpu().numpy()
    ref = O.spmv(c.astype(np.float64), x.astype(np.float64), S)
    assert np.abs(y - ref).max() <= 1e-5 * np.abs(ref).max()


def test_spmv_aos_layout(dev):
    """The reference's coef[i, j, 0..4] layout (simple.py:42) read in place."""
    from karman_taichi_gb300 import linalg
    NX, NY = 37, 29
    c = _rand_system(NX * NY, NY, seed=9)
    aos = np.ascontiguousarray(c.reshape(5, NX, NY).transpose(1, 2, 0))
    x = np.random.default_rng(1).standard_normal((NX, NY))
    y = linalg.spmv(linalg.Stencil(_t(aos, dev)), _t(x, dev)).cpu().numpy()
    assert np.allclose(y.reshape(-1), O.spmv(c, x, NY), rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("dtype,NX,NY,form", [("f64", 2050, 514, 0), ("f32", 2050, 514, 1), ("f32", 300, 64, 0),
                                               ("f64", 41, 33, 1)])
def test_spmv_flat_vector_pass_is_bitwise_the_tile_pass(dev, dtype, NX, NY, form):
    """SoA planes with even (or multiple-of-4) strides take the flat vectorised pass (k_spmv_vec); the
    same coefficients in the reference's [NX, NY, 5] layout take the tile pass (k_spmv).  Both evaluate
    the stencil in the same operation order, so the results are bitwise equal (the odd 41 x 33 grid
    takes the tile pass both ways)."""
    import torch
    from karman_taichi_gb300 import _lib as L, linalg
    tdt = torch.float64 if dtype == "f64" else torch.float32
    c = _rand_system(NX * NY, NY, seed=NX).reshape(5, NX, NY)
    soa = torch.from_numpy(c).to(dev, tdt).contiguous()
    aos = soa.permute(1, 2, 0).contiguous()
    x = torch.from_numpy(np.random.default_rng(6).standard_normal((NX, NY))).to(dev, tdt)
    y1 = linalg.spmv(linalg.Stencil(soa, form=form), x)
    y2 = linalg.spmv(linalg.Stencil(aos, form=form), x)
    assert torch.equal(y1, y2)
    ref = O.spmv(c if form == 0 else _lap_to_std(c), x.double().cpu().numpy(), NY)
    tol = 1e-13 if dtype == "f64" else 1e-5
    assert np.abs(y1.double().cpu().numpy().reshape(-1) - ref).max() <= tol * np.abs(ref).max()


def _lap_to_std(c):
    """Standard-form planes of a Laplacian-form system (component 0 holds the row sum)."""
    s = c.copy()
    s[0] = c[0] - c[1:].sum(axis=0)
    return s


def test_dot_deterministic(dev):
    from karman_taichi_gb300 import linalg
    rng = np.random.default_rng(2)
    p, q = rng.standard_normal(1_000_003), rng.standard_normal(1_000_003)
    tp, tq = _t(p, dev), _t(q, dev)
    a = linalg.dot(tp, tq)
    b = linalg.dot(tp, tq)
    assert a == b
    assert abs(a - float(np.dot(p, q))) <= 1e-12 * np.abs(p * q).sum()


def test_bicgstab_kat_dense_solve(dev):
    """debug/ti_bicg_test.py:21-98 restated with a seed: 5-diagonal (offsets
    +-1, +-3), diag = -sum(off) + 0.1, n = 320, compared with np.linalg.solve."""
    from karman_taichi_gb300 import linalg
    n, S = 320, 3
    c = _rand_system(n, S, seed=2022)
    b = np.random.default_rng(2023).random(n)
    xs = np.linalg.solve(O.to_csr(c, S).toarray(), b)
    x = _t(np.zeros(n), dev)
    info = linalg.bicgstab(linalg.Stencil(_t(c, dev), stride=S), _t(b, dev), x, eps=1e-8, max_iter=100 * n)
    assert info.ok
    xg = x.cpu().numpy()
    assert np.allclose(xg, xs)
    ref = O.bicgstab(c, b, S, eps=1e-8, max_iter=100 * n)
    assert abs(info.iters - ref.iters) <= 1
    assert np.abs(xg - ref.x).max() <= 1e-6 * np.abs(ref.x).max()


def test_bicgstab_poisson_vs_direct(dev):
    """benchmark/cg_to_sparse/test_cg_sparse.py:10-41: Laplacian + 0.1 I,
    RHS sin*sin, BiCGSTAB vs a direct sparse solve."""
    import scipy.sparse.linalg as spla
    from karman_taichi_gb300 import linalg
    N = 96
    c = _laplacian(N)
    xl = np.arange(N) * 2.0 / N
    b = (np.sin(2 * np.pi * xl)[:, None] * np.sin(2 * np.pi * xl)[None, :]).reshape(-1)
    xs = spla.spsolve(O.to_csr(c, N).tocsc(), b)
    x = _t(np.zeros(N * N), dev)
    info = linalg.bicgstab(linalg.Stencil(_t(c, dev), stride=N), _t(b, dev), x, eps=1e-10)
    assert info.ok
    assert np.abs(x.cpu().numpy() - xs).max() <= 1e-7 * np.abs(xs).max()


def test_cg_poisson_and_history(dev):
    import scipy.sparse.linalg as spla
    from karman_taichi_gb300 import linalg
    import torch
    N = 64
    c = _laplacian(N)
    b = np.random.default_rng(0).standard_normal(N * N)
    xs = spla.spsolve(O.to_csr(c, N).tocsc(), b)
    x = _t(np.zeros(N * N), dev)
    hist = torch.zeros(1000, dtype=torch.float64, device=dev)
    info = linalg.cg(linalg.Stencil(_t(c, dev), stride=N), _t(b, dev), x, eps=1e-10, history=hist)
    assert info.ok
    assert np.abs(x.cpu().numpy() - xs).max() <= 1e-7 * np.abs(xs).max()
    ref = O.cg(c, b, N, eps=1e-10)
    assert abs(info.iters - ref.iters) <= 1
    h = hist[: info.iters + 1].cpu().numpy()
    assert h[0] == pytest.approx(math.sqrt(np.dot(b, b)), rel=1e-12)
    assert h[-1] < 1e-10 * h[0]


def test_jacobi_warm_start_matches_oracle(dev):
    """karman_taichi.py:342-456: right Jacobi with an M that differs from A's
    diagonal, warm start, omega == 0 break."""
    from karman_taichi_gb300 import linalg
    n, S = 2000, 40
    c = _rand_system(n, S, seed=11, diag_shift=0.5)
    M = c[0] * (1 + 0.1 * np.random.default_rng(1).random(n))
    b = np.random.default_rng(12).standard_normal(n)
    x0 = np.random.default_rng(13).standard_normal(n) * 0.1
    ref = O.bicgstab(c, b, S, eps=1e-8, max_iter=100 * n, x0=x0, M=M, omega_break=True, order="karman")
    x = _t(x0, dev)
    info = linalg.bicgstab(linalg.Stencil(_t(c, dev), stride=S), _t(b, dev), x, eps=1e-8, max_iter=100 * n,
                           warm=True, M=_t(M, dev), omega_break=True)
    assert info.ok and ref.status == O.OK
    assert abs(info.iters - ref.iters) <= 1
    assert np.abs(x.cpu().numpy() - ref.x).max() <= 1e-6 * np.abs(ref.x).max()


def test_launch_modes_deterministic_and_consistent(dev):
    """Graph-captured and direct multi-launch iterations are bitwise equal;
    the persistent cooperative solve repeats bitwise and agrees with them to
    rounding (its per-block partial sums are grouped differently)."""
    from karman_taichi_gb300 import linalg
    N = 80
    c = _laplacian(N, 0.05)
    b = np.random.default_rng(7).standard_normal(N * N)
    A = linalg.Stencil(_t(c, dev), stride=N)
    xs, its = {}, {}
    for mode in ("graph", "direct", "persist", "persist2"):
        x = _t(np.zeros(N * N), dev)
        info = linalg.bicgstab(A, _t(b, dev), x, eps=1e-9, use_graph=(mode == "graph"),
                               persistent=mode.startswith("persist"))
        assert info.ok
        xs[mode], its[mode] = x.cpu().numpy(), info.iters
    assert np.array_equal(xs["graph"], xs["direct"])
    assert np.array_equal(xs["persist"], xs["persist2"])
    assert abs(its["persist"] - its["graph"]) <= max(3, its["graph"] // 10)
    assert np.abs(xs["persist"] - xs["graph"]).max() <= 1e-6 * np.abs(xs["graph"]).max()


@pytest.mark.parametrize("persistent", [False, True])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_bicgstab_modes_match_oracle(dev, persistent, dtype):
    from karman_taichi_gb300 import linalg
    n, S = 40000, 200
    c = _rand_system(n, S, seed=21, diag_shift=0.3)
    b = np.random.default_rng(22).standard_normal(n)
    ref = O.bicgstab(c, b, S, eps=1e-6, max_iter=10 * n)
    x = _t(np.zeros(n, dtype=dtype), dev)
    info = linalg.bicgstab(linalg.Stencil(_t(c.astype(dtype), dev), stride=S), _t(b.astype(dtype), dev), x,
                           eps=1e-6, max_iter=10 * n, persistent=persistent)
    assert info.ok
    tol = 1e-5 if dtype == np.float64 else 1e-3
    assert np.abs(x.cpu().numpy() - ref.x).max() <= tol * np.abs(ref.x).max()
    assert abs(info.iters - ref.iters) <= max(2, ref.iters // 10)


@pytest.mark.parametrize("persistent", [False, True])
def test_cg_modes_and_history(dev, persistent):
    import torch
    from karman_taichi_gb300 import linalg
    N = 100
    c = _laplacian(N, 0.02)
    b = np.random.default_rng(3).standard_normal(N * N)
    ref = O.cg(c, b, N, eps=1e-9)
    hist = torch.zeros(2000, dtype=torch.float64, device=dev)
    x = _t(np.zeros(N * N), dev)
    info = linalg.cg(linalg.Stencil(_t(c, dev), stride=N), _t(b, dev), x, eps=1e-9, history=hist,
                     persistent=persistent)
    assert info.ok and abs(info.iters - ref.iters) <= 2
    h = hist[: info.iters + 1].cpu().numpy()
    assert np.allclose(h[1:len(ref.history)], ref.history[1:info.iters + 1][: len(h) - 1], rtol=1e-6)


def test_zero_rhs_nan_and_maxiter(dev):
    """Failure detection on the host side of the ABI: b = 0 converges at once,
    a NaN in b reports NONFINITE, a tiny cap reports MAXITER -- no trap."""
    from karman_taichi_gb300 import linalg, _lib as L
    N = 32
    c = _laplacian(N)
    A = linalg.Stencil(_t(c, dev), stride=N)
    x = _t(np.ones(N * N), dev)
    info = linalg.bicgstab(A, _t(np.zeros(N * N), dev), x)
    assert info.status == L.OK and info.iters == 0 and float(x.abs().max()) == 0.0
    b = np.random.default_rng(0).standard_normal(N * N)
    b[17] = np.nan
    info = linalg.bicgstab(A, _t(b, dev), _t(np.zeros(N * N), dev))
    assert info.status == L.NONFINITE
    b[17] = 1.0
    info = linalg.bicgstab(A, _t(b, dev), _t(np.zeros(N * N), dev), max_iter=3)
    assert info.status == L.MAXITER and info.iters == 3
    info = linalg.cg(A, _t(b, dev), _t(np.zeros(N * N), dev), max_iter=2)
    assert info.status == L.MAXITER and info.iters == 2


def test_bad_arguments_raise(dev):
    import torch
    from karman_taichi_gb300 import linalg, _lib as L
    c = _t(_laplacian(8), dev)
    A = linalg.Stencil(c, stride=8)
    with pytest.raises(ValueError):
        linalg.bicgstab(A, _t(np.zeros(10), dev), _t(np.zeros(10), dev))
    with pytest.raises(ValueError):
        linalg.spmv(A, torch.zeros(64, dtype=torch.float64))   # CPU tensor: no fallback
    lib = L.load()
    assert lib.kc_spmv(None, None, None, None) == L.ERR_ARG
    assert "null" in L.last_error()


def test_refined_mixed_precision(dev):
    import scipy.sparse.linalg as spla
    from karman_taichi_gb300 import linalg
    N = 128
    c = _laplacian(N, 0.01)
    b = np.random.default_rng(5).standard_normal(N * N)
    xs = spla.spsolve(O.to_csr(c, N).tocsc(), b)
    x = _t(np.zeros(N * N), dev)
    info = linalg.bicgstab_refined(linalg.Stencil(_t(c, dev), stride=N),
                                   linalg.Stencil(_t(c.astype(np.float32), dev), stride=N),
                                   _t(b, dev), x, eps=1e-9, eps_inner=1e-3)
    assert info.ok and info.refinements >= 2
    r = b - O.to_csr(c, N) @ x.cpu().numpy()
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1e-9
    assert np.abs(x.cpu().numpy() - xs).max() <= 1e-6 * np.abs(xs).max()


@pytest.mark.parametrize("sweeps", [1, 2, 3, 6])
@pytest.mark.parametrize("n,S", [(7, 3), (1000, 33), (514 * 40 + 17, 514), (3000, 1)])
def test_rbgs_sweeps_match_oracle(dev, n, S, sweeps):
    """k red-black Gauss-Seidel sweeps equal the restatement's (FP64, to rounding):
    odd and even sweep counts (the iterate alternates between x and a copy),
    flat links across row ends, strips of one column."""
    from karman_taichi_gb300 import linalg
    c = _rand_system(n, S, 3, diag_shift=0.5)
    b = np.random.default_rng(4).standard_normal(n)
    x0 = np.random.default_rng(5).standard_normal(n)
    x = _t(x0, dev)
    info = linalg.rbgs(linalg.Stencil(_t(c, dev), stride=S), _t(b, dev), x, eps=1e-30, max_iter=sweeps, warm=True)
    assert info.iters == sweeps and info.status == 1   # KC_MAXITER
    ref, norms = O.rbgs_sweeps(c, b, x0, sweeps, S)
    assert np.abs(x.cpu().numpy() - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
    # the last residual checked is that of the iterate the last sweep started from
    assert info.rel_res == pytest.approx(norms[-1] / np.linalg.norm(b), rel=1e-9)


def test_rbgs_momentum_system_converges(dev):
    """The channel's u-momentum system (diagonally dominant through the time
    term): Gauss-Seidel reaches ||b - A x|| / ||b|| < 1e-10 from zero and agrees
    with the FP64 BiCGSTAB solution; a warm start from that solution stops at
    the first check."""
    from karman_taichi_gb300 import linalg
    from karman_taichi_gb300.channel import ChannelSolver
    from karman_taichi_gb300.config import get
    s = ChannelSolver(get("channel_320x64"), device=dev, precision="mixed", native=False)
    s.assemble_momentum()
    x = _t(np.zeros(s.b_u.shape), dev)
    info = linalg.rbgs(s.A_u, s.b_u, x, eps=1e-10, max_iter=500, warm=False)
    assert info.ok and info.iters < 100, info
    c = s.coef_u.cpu().numpy().reshape(5, -1)
    S = s.coef_u.shape[2]
    b = s.b_u.cpu().numpy().reshape(-1)
    r = b - O.to_csr(c, S) @ x.cpu().numpy().reshape(-1)
    assert np.linalg.norm(r) <= 1e-10 * np.linalg.norm(b)
    xb = _t(np.zeros(s.b_u.shape), dev)
    ib = linalg.bicgstab(s.A_u, s.b_u, xb, eps=1e-12)
    assert ib.ok
    xa, xr = x.cpu().numpy(), xb.cpu().numpy()
    assert np.abs(xa - xr).max() <= 1e-8 * np.abs(xr).max()
    warm = linalg.rbgs(s.A_u, s.b_u, xb, eps=1e-8, max_iter=500, warm=True)
    assert warm.ok and warm.iters == 1


def test_rbgs_refined_momentum_system(dev):
    """FP32 red-black Gauss-Seidel inside FP64 refinement on the channel's
    u-momentum system: meets ||b - A x|| / ||b|| < 1e-8 in FP64 from zero in a
    few passes, agrees with the FP64 BiCGSTAB solution, and a warm start from
    that solution needs no sweep."""
    from karman_taichi_gb300 import linalg
    from karman_taichi_gb300.channel import ChannelSolver
    from karman_taichi_gb300.config import get
    s = ChannelSolver(get("channel_320x64"), device=dev, precision="mixed", native=False)
    s.assemble_momentum()
    x = _t(np.zeros(s.b_u.shape), dev)
    info = linalg.rbgs_refined(s.A_u, s.A_u32, s.b_u, x, eps=1e-8, max_iter=500)
    assert info.ok and 1 <= info.refinements <= 4 and info.iters < 200, info
    c = s.coef_u.cpu().numpy().reshape(5, -1)
    S = s.coef_u.shape[2]
    b = s.b_u.cpu().numpy().reshape(-1)
    r = b - O.to_csr(c, S) @ x.cpu().numpy().reshape(-1)
    assert np.linalg.norm(r) <= 1e-8 * np.linalg.norm(b)
    xb = _t(np.zeros(s.b_u.shape), dev)
    assert linalg.bicgstab(s.A_u, s.b_u, xb, eps=1e-12).ok
    assert np.abs(x.cpu().numpy() - xb.cpu().numpy()).max() <= 1e-6 * np.abs(xb.cpu().numpy()).max()
    warm = linalg.rbgs_refined(s.A_u, s.A_u32, s.b_u, xb, eps=1e-8, warm=True)
    assert warm.ok and warm.iters == 0 and warm.refinements == 0


def test_rbgs_refined_rows_linked_across_ends(dev):
    """A flat 5-point system whose rows link across their ends (every north and
    south link set): kc_rbgs_refined takes the one-sweep kernel (flat wrap
    handled) and meets the FP64 tolerance; the same system with those links
    cut takes the several-sweeps-per-launch tiles and meets it too."""
    from karman_taichi_gb300 import linalg
    n, S = 40 * 37, 37
    c = _rand_system(n, S, 11, diag_shift=1.0)
    b = np.random.default_rng(12).standard_normal(n)
    for cut in (False, True):
        cc = c.copy()
        if cut:
            j = np.arange(n) % S
            cc[3][j == S - 1] = 0.0
            cc[4][j == 0] = 0.0
            cc[0] = -(cc[1] + cc[2] + cc[3] + cc[4]) + 1.0
        A64 = linalg.Stencil(_t(cc, dev), stride=S)
        A32 = linalg.Stencil(_t(cc.astype(np.float32), dev), stride=S)
        x = _t(np.zeros(n), dev)
        info = linalg.rbgs_refined(A64, A32, _t(b, dev), x, eps=1e-8, max_iter=2000)
        assert info.ok, (cut, info)
        r = b - O.to_csr(cc, S) @ x.cpu().numpy()
        assert np.linalg.norm(r) <= 1e-8 * np.linalg.norm(b), cut


def test_rbgs_refined_blocked_sweeps_match_global_sweeps(dev):
    """The several-sweeps-per-launch tiles (shrinking halos, two sweeps per
    launch) compute what global red-black sweeps compute: one refinement pass
    of 4 sweeps from x = 0 on the channel's u-momentum system against the FP64
    restatement's 4 sweeps (FP32 arithmetic: 1e-5)."""
    from karman_taichi_gb300 import _lib as L, linalg
    from karman_taichi_gb300.channel import ChannelSolver
    from karman_taichi_gb300.config import get
    s = ChannelSolver(get("channel_320x64"), device=dev, precision="mixed", native=False)
    s.assemble_momentum()
    x = _t(np.zeros(s.b_u.shape), dev)
    lib = L.load()
    buf = linalg.Workspace(dev).get(lib.kc_refined_ws_bytes(s.A_u.n, s.A_u.stride))
    o = linalg._opts(1e-12, 500, L.X0_ZERO, L.PRECOND_NONE, 0, L.REL_R0, 4, True, None, False)
    info = L.KcSolveInfo()
    rc = lib.kc_rbgs_refined(ctypes.byref(s.A_u.system), ctypes.byref(s.A_u32.system), linalg.ptr(s.b_u),
                             linalg.ptr(x), linalg.ptr(buf), buf.numel(), ctypes.byref(o), 1e-5, 1,
                             ctypes.byref(info), linalg.stream_handle(dev))
    assert rc >= 0 and info.iters == 4 and info.refinements == 1, (rc, info.iters, info.refinements)
    S = s.coef_u.shape[2]
    ref, _ = O.rbgs_sweeps(s.coef_u.cpu().numpy().reshape(5, -1), s.b_u.cpu().numpy().reshape(-1),
                           np.zeros(s.b_u.numel()), 4, S)
    got = x.cpu().numpy().reshape(-1)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()


def test_rbgs_rel_to_r0_and_bad_arguments(dev):
    from karman_taichi_gb300 import linalg
    c = _rand_system(400, 20, 6, diag_shift=0.5)
    b = np.random.default_rng(7).standard_normal(400)
    A = linalg.Stencil(_t(c, dev), stride=20)
    x = _t(np.ones(400), dev)
    info = linalg.rbgs(A, _t(b, dev), x, eps=1e-6, max_iter=500, warm=True, rel_to_b=False)
    assert info.ok
    r = b - O.to_csr(c, 20) @ x.cpu().numpy()
    # stopped when the iterate the last sweep started from met the test; that sweep only lowered it
    assert np.linalg.norm(r) < 1e-6 * info.r0
    with pytest.raises(TypeError):
        linalg.rbgs(linalg.Stencil(_t(c.astype(np.float32), dev), stride=20), _t(b.astype(np.float32), dev),
                    _t(np.zeros(400, np.float32), dev))
    with pytest.raises(ValueError):
        linalg.rbgs(A, _t(b[:10], dev), _t(np.zeros(10), dev))
