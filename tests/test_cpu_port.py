"""The C/OpenMP restatement of the channel plain path (``oracle/kc_cpu.c``, the
timed CPU baseline and the reference arm of bench.py) against the NumPy
oracle's ``ChannelOracle``.

Both run the same FP64 algorithm; they differ only in the order of their
sums (OpenMP reductions vs NumPy), so with the linear solves taken to a
relative residual of 1e-12 the fields agree to 1e-9 relative and every time
step takes the same number of outer iterations.
"""
import numpy as np
import pytest

from oracle import np_oracle as O


@pytest.fixture(autouse=True)
def _few_threads():
    # tiny systems: a few OpenMP threads (all host threads busy-wait badly when the host is shared)
    from oracle import cpu
    old = cpu.threads()
    cpu.set_threads(2)
    yield
    cpu.set_threads(old)


def _setup(nx, ny, obstacles, eps, max_outer=20):
    from karman_taichi_gb300 import geometry
    from karman_taichi_gb300.config import ChannelConfig
    cfg = ChannelConfig("cpu_port", nx, ny, 1.0 / ny, 4, obstacles, n_steps=2).with_(eps=eps, max_outer=max_outer)
    solid = geometry.solid_mask(nx, ny, cfg.obstacles)
    u, v, p = geometry.channel_initial_fields(nx, ny, solid, U=cfg.U, seed=cfg.seed)
    P = O.ChannelParams(nx=nx, ny=ny, dx=cfg.dx, dy=cfg.dy, rho=cfg.rho, mu=cfg.mu, dt=cfg.dt, U=cfg.U,
                        alpha_m=cfg.alpha_m, alpha_u=cfg.alpha_u, alpha_p=cfg.alpha_p, eps=cfg.eps,
                        mass_tol=cfg.mass_tol, max_outer=cfg.max_outer)
    return cfg, solid, u, v, p, P


@pytest.mark.parametrize("nx,ny,obstacles", [(48, 16, (("square", 16, 8, 4),)), (64, 24, (("circle", 18, 12, 6),))])
def test_c_port_matches_channel_oracle(nx, ny, obstacles):
    from oracle import cpu
    cfg, solid, u, v, p, P = _setup(nx, ny, obstacles, eps=1e-12)
    orc = O.ChannelOracle(P, solid, u, v, p)
    recs = [orc.step() for _ in range(2)]
    cu, cv, cp = u.copy(), v.copy(), p.copy()
    st = cpu.channel_run(cfg, solid, cu, cv, cp, n_steps=2)
    assert st["steps"] == 2
    assert st["outer"] == sum(len(r) for r in recs)
    assert st["mass"] == pytest.approx(recs[-1][-1]["mass"], rel=1e-6, abs=1e-14)
    for name, a in (("u", cu), ("v", cv), ("p", cp)):
        ref = getattr(orc, name)
        err = np.abs(a - ref).max() / max(np.abs(ref).max(), 1e-300)
        assert err < 1e-9, (name, err)


def test_c_port_stops_at_the_outer_cap():
    """max_outer bounds the outer loop of every step (karman_taichi.py:633's cap)."""
    from oracle import cpu
    cfg, solid, u, v, p, P = _setup(48, 16, (("square", 16, 8, 4),), eps=1e-8, max_outer=3)
    st = cpu.channel_run(cfg.with_(mass_tol=0.0), solid, u, v, p, n_steps=2)
    assert st["steps"] == 2 and st["outer"] == 6


def test_bench_cpu_whole_steps_times_real_steps():
    """bench.py's CPU baseline / reference arm times whole time steps (no extrapolation): the steps
    it reports are the steps the C port ran, from the seeded initial state."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    from karman_taichi_gb300.config import ChannelConfig
    cfg = ChannelConfig("tiny", 48, 16, 1.0 / 16, 4, (("square", 16, 8, 4),), max_outer=5)
    r = bench.cpu_whole_steps(cfg, budget_s=0.0, steps=2)
    assert r["steps_timed"] == 2 and r["outer_iterations"] >= 2
    assert r["value"] == pytest.approx(2 / r["seconds"], rel=0.05)
    r1 = bench.cpu_whole_steps(cfg, budget_s=0.0)        # the budget never drops below one step
    assert r1["steps_timed"] == 1 and r1["first_step_outer"] == r["first_step_outer"]
