"""Failure detection without a GPU fault.

The reference's only guards are the breakdown tests rho == 0
(bicgsolver.py:96-98, karman_taichi.py:386-389), omega == 0
(karman_taichi.py:451-454) and its iteration caps (cgsolver.py:14,
karman_taichi.py:382, 633).  This library adds bounded device waits, a
NaN/Inf status and a fallback from the accelerated pressure solve to the
plain BiCGSTAB.  Every failure here is made on the host (a poisoned FP32
system, a NaN written into a field, a lowered poll bound) and every wait in
the kernels is bounded, so no test can hang or fault the GPU; each checks the
status the host reads back and that the context keeps working afterwards.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _laplacian(N, offset=0.05):
    c = np.zeros((5, N, N))
    c[0] = 4.0 + offset
    c[1, 1:, :] = -1.0
    c[2, :-1, :] = -1.0
    c[3, :, :-1] = -1.0
    c[4, :, 1:] = -1.0
    return c


def test_grid_barrier_wait_runs_out_and_context_survives(dev):
    """The persistent solver's grid barrier gives up after a bounded number of polls: with the bound
    lowered to one poll the blocks cannot all meet, every block leaves, the call returns KC_ERR_CUDA
    ("grid barrier timed out") and the next solve on the same context converges as before."""
    import torch
    from karman_taichi_gb300 import _lib as L, linalg
    lib = L.load()
    N = 512                                   # 262k unknowns: hundreds of cooperating blocks
    A = linalg.Stencil(torch.from_numpy(_laplacian(N)).to(dev))
    b = torch.from_numpy(np.random.default_rng(2).standard_normal((N, N))).to(dev)
    x_ref = torch.zeros_like(b)
    good = linalg.bicgstab(A, b, x_ref, eps=1e-8, max_iter=2000, persistent=True)
    assert good.ok
    old = lib.kc_debug_barrier_spin_limit(1)
    try:
        x = torch.zeros_like(b)
        with pytest.raises(L.KcError) as e:
            linalg.bicgstab(A, b, x, eps=1e-8, max_iter=2000, persistent=True)
        assert e.value.rc == L.ERR_CUDA
        assert "grid barrier timed out" in str(e.value)
    finally:
        lib.kc_debug_barrier_spin_limit(old)
    torch.cuda.synchronize()                  # no sticky error: the context is intact
    x = torch.zeros_like(b)
    again = linalg.bicgstab(A, b, x, eps=1e-8, max_iter=2000, persistent=True)
    assert again.ok and again.iters == good.iters
    assert torch.equal(x, x_ref)


@pytest.mark.parametrize("kind", ["bicgstab", "cg", "bicgstab_refined", "rbgs_refined", "pcg_refined"])
def test_nan_in_rhs_is_reported(dev, kind):
    """A NaN in the right-hand side stops the solve with KC_NONFINITE (the reference iterates on)."""
    import torch
    from karman_taichi_gb300 import _lib as L, linalg
    N = 64
    c = torch.from_numpy(_laplacian(N)).to(dev)
    A = linalg.Stencil(c)
    b = torch.from_numpy(np.random.default_rng(3).standard_normal((N, N))).to(dev)
    b[17, 23] = float("nan")
    x = torch.zeros_like(b)
    if kind == "bicgstab":
        info = linalg.bicgstab(A, b, x, eps=1e-8, max_iter=500)
    elif kind == "cg":
        info = linalg.cg(A, b, x, eps=1e-8, max_iter=500)
    elif kind == "pcg_refined":
        lap = c.clone()
        lap[0] = c[0] + c[1:].sum(dim=0)        # Laplacian form: component 0 holds the row sum
        A32 = linalg.Stencil(lap.float().contiguous(), form=L.FORM_LAPLACIAN)
        mg = linalg.Multigrid(A32)
        mg.setup()
        info = linalg.pcg_refined(A, A32, b, x, mg, eps=1e-8)
    else:
        A32 = linalg.Stencil(c.float())
        if kind == "bicgstab_refined":
            info = linalg.bicgstab_refined(A, A32, b, x, eps=1e-8, max_iter=500)
        else:
            info = linalg.rbgs_refined(A, A32, b, x, eps=1e-8, max_iter=200)
    assert info.status == L.NONFINITE, info


@pytest.mark.parametrize("native", [True, False])
def test_nan_in_a_field_ends_the_step_with_nonfinite(dev, native):
    """A NaN written into u on the host: the time step stops after its first outer iteration with
    KC_NONFINITE instead of running to max_outer, and a reset solver steps normally again."""
    import torch
    from karman_taichi_gb300 import _lib as L
    from karman_taichi_gb300.channel import ChannelSolver
    from karman_taichi_gb300.config import ChannelConfig
    cfg = ChannelConfig("nan", 64, 16, 1.0 / 16, 4, (("square", 20, 8, 4),), max_outer=6)
    s = ChannelSolver(cfg, device=dev, precision="mixed", native=native)
    s.u[10, 5] = float("nan")
    rec = s.step()
    assert len(rec) == 1 if not native else rec[0]["outer"] == 1
    assert rec[-1]["status"] == L.NONFINITE
    s.reset()
    rec = s.step()
    assert rec[-1].get("status", L.OK) != L.NONFINITE and np.isfinite(rec[-1]["mass"])
    assert (rec[0]["outer"] if native else len(rec)) == cfg.max_outer   # this small case needs them all


def test_poisoned_fp32_pressure_system_falls_back_to_plain_bicgstab(dev):
    """The accelerated p' solve refines an FP32 copy of the system.  With that copy poisoned (its
    links scaled by seeded random factors, so the FP32 solves aim at another operator) the FP64
    refinement cannot reach the tolerance, the solve reports a non-OK status, ChannelSolver counts a
    fallback and the plain FP64 BiCGSTAB (the reference method) solves p' -- so every outer
    iteration still converges, to the fields of an unpoisoned run within the solve tolerance."""
    import torch
    from karman_taichi_gb300 import _lib as L
    from karman_taichi_gb300.channel import ChannelSolver
    from karman_taichi_gb300.config import ChannelConfig
    cfg = ChannelConfig("stall", 64, 16, 1.0 / 16, 4, (("square", 20, 8, 4),), max_outer=4).with_(eps=1e-10)
    poisoned = ChannelSolver(cfg, device=dev, precision="mixed", native=False)
    clean = ChannelSolver(cfg, device=dev, precision="mixed", native=False)
    g = torch.Generator(device=dev).manual_seed(5)
    orig = poisoned.assemble_p

    def assemble_then_poison():
        orig()
        noise = 0.5 + torch.rand(poisoned.coef_p32[1:].shape, generator=g, device=dev, dtype=torch.float32)
        poisoned.coef_p32[1:].mul_(noise)

    poisoned.assemble_p = assemble_then_poison
    rp = poisoned.step()
    rc = clean.step()
    assert poisoned.fallbacks >= len(rp) and clean.fallbacks == 0
    assert poisoned.last_accel.status != L.OK
    assert len(rp) == len(rc) and all(r["st"][2] == L.OK for r in rp)   # the fallback converged
    a, b = poisoned.state_numpy(), clean.state_numpy()
    for k in ("u", "v", "p"):
        assert np.abs(a[k] - b[k]).max() <= 1e-6 * np.abs(b[k]).max(), k
