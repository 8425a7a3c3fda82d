"""GPU multigrid preconditioner vs its CPU restatement, and the
multigrid-preconditioned mixed-precision solve.

Tolerances: one V-cycle agrees with the FP32 NumPy restatement to 1e-4
relative (both FP32; the GPU contracts to FMA); the refined solve meets the
FP64 tolerance ||b - A x|| / ||b|| < 1e-8 and matches a direct solve to 1e-6.
"""
import functools

import numpy as np
import pytest

from oracle import np_oracle as O

pytestmark = pytest.mark.gpu


def _channel_pcorr(nx, ny, D, ci, cj):
    """p' system of the first outer iteration of a small channel (oracle)."""
    from karman_taichi_gb300 import geometry
    solid = geometry.solid_mask(nx, ny, [("square", ci, cj, D)])
    u, v, p = geometry.channel_initial_fields(nx, ny, solid)
    h = 1.0 / ny
    P = O.ChannelParams(nx=nx, ny=ny, dx=h, dy=h, rho=1.0, mu=D * h / 150, dt=0.5 * h)
    orc = O.ChannelOracle(P, solid, u, v, p)
    orc.assemble_momentum()
    ru = O.bicgstab(orc.coef_u, orc.b_u, orc.b_u.shape[1])
    rv = O.bicgstab(orc.coef_v, orc.b_v, orc.b_v.shape[1])
    orc.relax(ru.x.reshape(orc.u.shape), rv.x.reshape(orc.v.shape))
    orc.assemble_p()
    return orc.coef_p, orc.b_p


def _poisson(NX, NY, block=None):
    """Standard-form 5-point Poisson system on a padded [NX][NY] grid: halo
    rows empty, Neumann walls, Dirichlet through the east halo, an optional
    blocked square (identity rows, links to it removed)."""
    c = np.zeros((5, NX, NY))
    inner = np.zeros((NX, NY), dtype=bool)
    inner[1:NX - 1, 1:NY - 1] = True
    if block is not None:
        i0, i1, j0, j1 = block
        inner[i0:i1, j0:j1] = False
    ii, jj = np.nonzero(inner)
    for q, (di, dj) in zip((1, 2, 3, 4), ((-1, 0), (1, 0), (0, 1), (0, -1))):
        ni, nj = ii + di, jj + dj
        link = inner[ni, nj] | (ni == NX - 1)          # east halo: Dirichlet
        c[q, ii, jj] = np.where(link, -1.0, 0.0)
    c[0, ii, jj] = -(c[1] + c[2] + c[3] + c[4])[ii, jj]
    if block is not None:
        c[0, i0:i1, j0:j1] = 1.0
    return c


def _t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _fp32(coef, lap):
    from karman_taichi_gb300 import _lib as L
    if lap:
        return O.to_laplacian32(coef), L.FORM_LAPLACIAN
    return coef.astype(np.float32), L.FORM_STANDARD


@pytest.mark.parametrize("coarsest", [0, 64])   # 0: exact coarsest solve (dense inverse); 64: Jacobi sweeps
@pytest.mark.parametrize("nu", [1, 2])   # 1: the fused two-launch-per-level cycle; 2: the general kernels
@pytest.mark.parametrize("lap", [False, True])
@pytest.mark.parametrize("alpha", [1.0, 1.6])
def test_vcycle_matches_restatement(dev, alpha, lap, nu, coarsest):
    from karman_taichi_gb300 import linalg
    coef, b = _channel_pcorr(96, 40, 6, 30, 20)
    NX, NY = coef.shape[1:]
    c32, form = _fp32(coef, lap)
    A = linalg.Stencil(_t(c32, dev), form=form)
    mg = linalg.Multigrid(A, alpha=alpha, nu_pre=nu, nu_post=nu, coarsest_sweeps=coarsest).setup()
    r = np.random.default_rng(0).standard_normal(NX * NY).astype(np.float32)
    r[coef[0].reshape(-1) == 0] = 0.0
    z = mg.apply(_t(r.reshape(NX, NY), dev)).cpu().numpy().reshape(-1)
    orc = O.MultigridOracle(c32.reshape(5, -1), NX, NY, alpha=alpha, lap=lap, nu_pre=nu, nu_post=nu,
                            coarsest_sweeps=coarsest)
    assert coarsest != 0 or orc.inv is not None
    ref = orc.apply(r)
    assert np.abs(z - ref).max() <= 1e-4 * np.abs(ref).max()


@functools.lru_cache(maxsize=None)
def _pcorr_320x64():
    return _channel_pcorr(320, 64, 8, 64, 32)


@pytest.mark.parametrize("tail", [False, True])
@pytest.mark.parametrize("big_cells", [1000, 200000])   # 1000: the large (64-wide) tiles on every level below 0
@pytest.mark.parametrize("nu_coarse", [1, 2, 3])
def test_vcycle_coarse_sweeps_match_restatement(dev, nu_coarse, big_cells, tail):
    """nu_coarse red-black sweeps before and after the coarse correction on the
    levels below level 0: the fused tile kernels (halo 2 nu_coarse) and the
    one-block tail against the restatement."""
    from karman_taichi_gb300 import linalg
    coef, b = _pcorr_320x64()
    NX, NY = coef.shape[1:]
    c32, form = _fp32(coef, True)
    A = linalg.Stencil(_t(c32, dev), form=form)
    mg = linalg.Multigrid(A, nu_coarse=nu_coarse, big_cells=big_cells, tail=tail).setup()
    r = np.random.default_rng(1).standard_normal(NX * NY).astype(np.float32)
    r[coef[0].reshape(-1) == 0] = 0.0
    z = mg.apply(_t(r.reshape(NX, NY), dev)).cpu().numpy().reshape(-1)
    ref = O.MultigridOracle(c32.reshape(5, -1), NX, NY, lap=True, nu_coarse=nu_coarse).apply(r)
    assert np.abs(z - ref).max() <= 1e-4 * np.abs(ref).max()


@pytest.mark.parametrize("tail", [False, True])
def test_vcycle_launch_count(dev, tail):
    """The fused cycle launches two kernels per level above the coarsest; with
    the tail, the levels of at most 1536 cells (here every level below level 0)
    and the coarsest solve are one launch."""
    from karman_taichi_gb300 import _lib as L, linalg
    coef, b = _channel_pcorr(96, 40, 6, 30, 20)
    NX, NY = coef.shape[1:]
    c32, form = _fp32(coef, True)
    mg = linalg.Multigrid(linalg.Stencil(_t(c32, dev), form=form), tail=tail).setup()
    levels = len(O.MultigridOracle(c32.reshape(5, -1), NX, NY, lap=True).levels)
    assert levels >= 3
    r = _t(np.ones((NX, NY), dtype=np.float32), dev)
    lib = L.load()
    n0 = lib.kc_launch_count()
    mg.apply(r)
    assert lib.kc_launch_count() - n0 == (3 if tail else 2 * (levels - 1) + 1)


# grids of the workloads (p' of the 320x64 and 2048x512 channels, the 1024^2 system,
# a 4096x1024 channel, small batched instances, a strip): the tail starts at levels 1..6
@pytest.mark.parametrize("nu_coarse", [2, 3])
@pytest.mark.parametrize("shape", [(98, 42), (130, 34), (322, 66), (1026, 1026), (2050, 514), (4098, 1026),
                                   (3000, 7)])
def test_tail_is_the_per_level_cycle(dev, shape, nu_coarse):
    """The smallest levels in one launch compute the V-cycle bit for bit as the
    one-launch-per-level cycle does."""
    import torch
    from karman_taichi_gb300 import _lib as L, linalg
    NX, NY = shape
    bi, bj = NX // 5, NY // 2
    c32 = O.to_laplacian32(_poisson(NX, NY, (bi, bi + 8, max(bj - 4, 1), min(bj + 4, NY - 1))))
    A = linalg.Stencil(_t(c32, dev), form=L.FORM_LAPLACIAN)
    r = np.random.default_rng(NX).standard_normal((NX, NY)).astype(np.float32)
    r[(c32[1:] == 0).all(axis=0)] = 0.0
    rt = _t(r, dev)
    lib = L.load()
    zs = []
    for tail in (False, True):
        mg = linalg.Multigrid(A, tail=tail, nu_coarse=nu_coarse).setup()
        n0 = lib.kc_launch_count()
        zs.append(mg.apply(rt))
        zs.append(mg.apply(rt))
        zs.append(lib.kc_launch_count() - n0)
    assert zs[5] < zs[2]   # fewer launches with the tail
    assert torch.equal(zs[0], zs[3]) and torch.equal(zs[1], zs[4]) and torch.equal(zs[0], zs[1])
    assert torch.isfinite(zs[3]).all()


def test_pcg_tail_same_iterates(dev):
    """The refined multigrid CG takes the same iterations to the same x with and
    without the tail (graph-captured chunks included)."""
    import torch
    from karman_taichi_gb300 import _lib as L, linalg
    NX, NY = 1026, 1026
    c64 = _poisson(NX, NY, (500, 540, 480, 520))
    A64 = linalg.Stencil(_t(c64, dev))
    A32 = linalg.Stencil(_t(O.to_laplacian32(c64), dev), form=L.FORM_LAPLACIAN)
    b = np.random.default_rng(5).standard_normal((NX, NY))
    b[(c64[1:] == 0).all(axis=0)] = 0.0
    out = []
    for tail in (False, True):
        mg = linalg.Multigrid(A32, tail=tail).setup()
        x = _t(np.zeros((NX, NY)), dev)
        info = linalg.pcg_refined(A64, A32, _t(b, dev), x, mg, eps=1e-8)
        assert info.ok
        out.append((info.iters, x))
    assert out[0][0] == out[1][0]
    assert torch.equal(out[0][1], out[1][1])


def test_laplacian_spmv_matches_standard(dev):
    """The Laplacian-form FP32 stencil is the same operator (FP32 tolerance)."""
    from karman_taichi_gb300 import linalg
    coef, b = _channel_pcorr(96, 40, 6, 30, 20)
    NX, NY = coef.shape[1:]
    x = np.random.default_rng(1).standard_normal((NX, NY)).astype(np.float32)
    c32, form = _fp32(coef, True)
    A = linalg.Stencil(_t(c32, dev), form=form)
    y = linalg.spmv(A, _t(x, dev)).cpu().numpy().reshape(-1)
    ref = O.spmv(coef.reshape(5, -1), x.reshape(-1).astype(np.float64), NY)
    assert np.abs(y - ref).max() <= 1e-5 * np.abs(ref).max()


@pytest.mark.parametrize("lap", [False, True])
def test_mg_preconditioned_solve(dev, lap):
    import scipy.sparse.linalg as spla
    from karman_taichi_gb300 import linalg
    coef, b = _channel_pcorr(256, 64, 8, 64, 32)
    NX, NY = coef.shape[1:]
    S = NY
    A64 = linalg.Stencil(_t(coef, dev))
    c32, form = _fp32(coef, lap)
    A32 = linalg.Stencil(_t(c32, dev), form=form)
    mg = linalg.Multigrid(A32).setup()
    x = _t(np.zeros((NX, NY)), dev)
    info = linalg.pbicgstab_refined(A64, A32, _t(b, dev), x, mg, eps=1e-8)
    assert info.ok, info
    xg = x.cpu().numpy().reshape(-1)
    res = b.reshape(-1) - O.spmv(coef.reshape(5, -1), xg, S)
    assert np.linalg.norm(res) / np.linalg.norm(b) < 1e-8
    plain = O.bicgstab(coef, b, S, eps=1e-8)
    assert info.iters * 8 < plain.iters          # the preconditioner must pay for itself
    Acsr = O.to_csr(coef.reshape(5, -1), S)
    rows = np.flatnonzero(coef[0].reshape(-1) != 0)
    xs = np.zeros_like(xg)
    xs[rows] = spla.spsolve(Acsr[rows][:, rows].tocsc(), b.reshape(-1)[rows])
    assert np.abs(xg - xs).max() <= 1e-6 * np.abs(xs).max()


def test_mg_initial_guess_is_used(dev):
    """An exact initial guess finishes with zero inner iterations."""
    from karman_taichi_gb300 import linalg
    coef, b = _channel_pcorr(128, 32, 6, 40, 16)
    NX, NY = coef.shape[1:]
    A64 = linalg.Stencil(_t(coef, dev))
    c32, form = _fp32(coef, True)
    A32 = linalg.Stencil(_t(c32, dev), form=form)
    mg = linalg.Multigrid(A32).setup()
    x = _t(np.zeros((NX, NY)), dev)
    linalg.pbicgstab_refined(A64, A32, _t(b, dev), x, mg, eps=1e-10)
    x2 = _t(np.zeros((NX, NY)), dev)
    info = linalg.pbicgstab_refined(A64, A32, _t(b, dev), x2, mg, eps=1e-8, x0=x)
    assert info.ok and info.iters == 0


def test_vcycle_matches_restatement_above_one_million_cells(dev):
    """More cells than one grid-stride pass of the capped launch covers."""
    from karman_taichi_gb300 import _lib as L, linalg
    NX, NY = 1026, 1026
    c32 = O.to_laplacian32(_poisson(NX, NY, (500, 540, 480, 520)))
    A = linalg.Stencil(_t(c32, dev), form=L.FORM_LAPLACIAN)
    mg = linalg.Multigrid(A).setup()
    r = np.random.default_rng(2).standard_normal(NX * NY).astype(np.float32)
    r[(c32[1:] == 0).all(axis=0).reshape(-1)] = 0.0
    z = mg.apply(_t(r.reshape(NX, NY), dev)).cpu().numpy().reshape(-1)
    ref = O.MultigridOracle(c32.reshape(5, -1), NX, NY, lap=True).apply(r)
    assert np.abs(z - ref).max() <= 1e-4 * np.abs(ref).max()


@pytest.mark.parametrize("case", ["channel", "poisson_large"])
def test_pcg_refined_solve(dev, case):
    import scipy.sparse.linalg as spla
    from karman_taichi_gb300 import _lib as L, linalg
    if case == "channel":
        coef, b = _channel_pcorr(256, 64, 8, 64, 32)
    else:
        coef = _poisson(1026, 1026, (500, 540, 480, 520))
        b = np.random.default_rng(3).standard_normal(coef.shape[1:])
        b[(coef[1:] == 0).all(axis=0)] = 0.0
    NX, NY = coef.shape[1:]
    A64 = linalg.Stencil(_t(coef, dev))
    A32 = linalg.Stencil(_t(O.to_laplacian32(coef), dev), form=L.FORM_LAPLACIAN)
    mg = linalg.Multigrid(A32).setup()
    x = _t(np.zeros((NX, NY)), dev)
    info = linalg.pcg_refined(A64, A32, _t(b, dev), x, mg, eps=1e-8)
    assert info.ok, info
    xg = x.cpu().numpy().reshape(-1)
    res = b.reshape(-1) - O.spmv(coef.reshape(5, -1), xg, NY)
    assert np.linalg.norm(res) / np.linalg.norm(b) < 1e-8
    assert info.iters < 150, info
    if case == "channel":
        Acsr = O.to_csr(coef.reshape(5, -1), NY)
        rows = np.flatnonzero(coef[0].reshape(-1) != 0)
        xs = np.zeros_like(xg)
        xs[rows] = spla.spsolve(Acsr[rows][:, rows].tocsc(), b.reshape(-1)[rows])
        assert np.abs(xg - xs).max() <= 1e-6 * np.abs(xs).max()


def test_graph_cache_tells_forms_apart(dev):
    """Captured iteration graphs bake in the coefficient form: solving a
    standard-form and then a Laplacian-form system in the same buffers (same
    addresses, as a recycling allocator would hand out) must not replay the
    first system's graph."""
    from karman_taichi_gb300 import _lib as L, linalg
    coef, b = _channel_pcorr(256, 64, 8, 64, 32)
    NX, NY = coef.shape[1:]
    A64 = linalg.Stencil(_t(coef, dev))
    buf = _t(coef.astype(np.float32), dev)
    ws = linalg.Workspace(dev)
    bt = _t(b, dev)
    mg = linalg.Multigrid(linalg.Stencil(buf)).setup()
    x = _t(np.zeros((NX, NY)), dev)
    first = linalg.pcg_refined(A64, linalg.Stencil(buf), bt, x, mg, eps=1e-8, ws=ws)
    assert first.ok, first
    buf.copy_(_t(O.to_laplacian32(coef), dev))                 # same address, Laplacian form
    lap = linalg.Stencil(buf, form=L.FORM_LAPLACIAN)
    mg.A = lap
    mg.setup()
    x.zero_()
    second = linalg.pcg_refined(A64, lap, bt, x, mg, eps=1e-8, ws=ws)
    assert second.ok, second
    res = b.reshape(-1) - O.spmv(coef.reshape(5, -1), x.cpu().numpy().reshape(-1), NY)
    assert np.linalg.norm(res) / np.linalg.norm(b) < 1e-8


def test_autotune_keeps_fields_and_state(dev):
    """The autotuner picks launch shapes from its candidates, leaves the solver's
    state as it found it, and the tuned solver steps to the same fields bit for bit."""
    import numpy as np
    from karman_taichi_gb300.autotune import BIG_CANDIDATES, CHUNK_CANDIDATES, TAIL_CANDIDATES, tune_pressure
    from karman_taichi_gb300.channel import ChannelSolver
    from karman_taichi_gb300.config import get
    cfg = get("channel_320x64")
    a = ChannelSolver(cfg, device=dev, precision="mixed")
    b = ChannelSolver(cfg, device=dev, precision="mixed")
    a.step(); b.step()
    before = a.state_numpy()
    c = tune_pressure(a, reps=1)
    assert c["tail"] in TAIL_CANDIDATES and c["big_cells"] in BIG_CANDIDATES
    assert c["check_every_p"] in CHUNK_CANDIDATES and c["ms"] > 0 and len(c["tried"]) >= 3
    after = a.state_numpy()
    for k in before:
        assert np.array_equal(before[k], after[k]), k
    for _ in range(2):
        ra, rb = a.step(), b.step()
        assert ra[0]["it_p"] == rb[0]["it_p"]
    sa, sb = a.state_numpy(), b.state_numpy()
    for k in ("u", "v", "p"):
        assert np.array_equal(sa[k], sb[k]), k


def test_autotune_cycle_stage(dev):
    """With cycles the tuner also picks the sweeps below level 0 (and their
    weight) from its candidates, restores the solver's state, and the tuned
    solver steps to the untuned solver's fields within the solve tolerance."""
    import numpy as np
    from karman_taichi_gb300.autotune import CYCLE_CANDIDATES, apply_choice, tune_pressure
    from karman_taichi_gb300.channel import ChannelSolver
    from karman_taichi_gb300.config import get
    cfg = get("channel_320x64")
    a = ChannelSolver(cfg, device=dev, precision="mixed")
    b = ChannelSolver(cfg, device=dev, precision="mixed")
    a.step(); b.step()
    before = a.state_numpy()
    c = tune_pressure(a, reps=1, cycles=CYCLE_CANDIDATES)
    assert (c["nu_coarse"], c["omega_coarse"]) in [(n, round(w, 6)) for n, w in CYCLE_CANDIDATES]
    assert a.mg.opts.nu_coarse == c["nu_coarse"] and abs(a.mg.opts.omega[3] - c["omega_coarse"]) < 1e-6
    assert sum(k.startswith("nu_coarse=") for k in c["tried"]) == len(CYCLE_CANDIDATES)
    after = a.state_numpy()
    for k in before:
        assert np.array_equal(before[k], after[k]), k
    # every candidate cycle steps to the same fields within the solve tolerance
    d = ChannelSolver(cfg, device=dev, precision="mixed")
    d.step()
    apply_choice(d, dict(c, nu_coarse=3, omega_coarse=1.6))
    for _ in range(2):   # (this early transient of the 320 x 64 case runs the 50 outer iterations)
        ra, rb, rd = a.step(), b.step(), d.step()
        for r in (ra, rd):
            assert abs(r[-1]["mass"] - rb[-1]["mass"]) <= 1e-4 * rb[-1]["mass"]
    sb = b.state_numpy()
    for s in (a, d):
        st = s.state_numpy()
        for k in ("u", "v", "p"):
            assert np.abs(st[k] - sb[k]).max() <= 1e-5 * np.abs(sb[k]).max(), k
