"""The batched configuration as one persistent launch (kc_channel_batch_fused):
instance independence bit for bit, agreement with the per-instance native step
and with the oracle, and a poisoned instance that stops alone."""
import math

import numpy as np
import pytest
import torch

from oracle import np_oracle as O

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _cfgs(n, seed, max_outer=10):
    from karman_taichi_gb300.batch import batch_configs
    # the smaller sizes of the batched set keep the test short
    return [c.with_(max_outer=max_outer) for c in batch_configs(4 * n, seed=seed) if c.nx <= 320][:n]


def test_fused_instance_is_its_batch_of_one(dev):
    """Block k runs instance k alone: a batch computes bit for bit what each instance computes
    in a batch of one, and u0 / v0 follow u / v."""
    from karman_taichi_gb300.batch import BatchedChannels
    cfgs = _cfgs(4, seed=7)
    b = BatchedChannels(cfgs, device=dev, precision="mixed", workers=1)
    b.step_fused(2)
    assert all(t["outer"] >= 2 for t in b.fused_totals)
    for cfg, s in zip(cfgs, b.solvers):
        one = BatchedChannels([cfg], device=dev, precision="mixed", workers=1)
        one.step_fused(2)
        a, r = s.state_numpy(), one.solvers[0].state_numpy()
        for k in ("u", "v", "p", "u0", "v0"):
            assert np.array_equal(a[k], r[k]), (cfg.name, k)
        assert np.array_equal(a["u0"], a["u"]) and np.array_equal(a["v0"], a["v"])
        one.close()
    b.close()


def test_fused_matches_native_step(dev):
    """The fused launch against kc_channel_step (the same method with multi-block kernels,
    recycling off): both end every solve at ||b - A x|| / ||b|| < 1e-8, so the fields agree to
    the solves' tolerance and the outer iteration counts agree to one."""
    from karman_taichi_gb300.batch import BatchedChannels
    from karman_taichi_gb300.channel import ChannelSolver
    cfgs = _cfgs(3, seed=11)
    b = BatchedChannels(cfgs, device=dev, precision="mixed", workers=1)
    outer_f = []
    for _ in range(2):
        b.step_fused(1)
        outer_f.append([rec[-1][0]["outer"] for rec in b.records])
    for k, (cfg, s) in enumerate(zip(cfgs, b.solvers)):
        solo = ChannelSolver(cfg, device=dev, precision="mixed", recycle=0)
        for t in range(2):
            r = solo.step()
            assert abs(r[0]["outer"] - outer_f[t][k]) <= 1, (cfg.name, t, r[0]["outer"], outer_f[t][k])
        a, r = s.state_numpy(), solo.state_numpy()
        for f in ("u", "v", "p"):
            assert _rel(a[f], r[f]) <= 1e-6, (cfg.name, f, _rel(a[f], r[f]))
    b.close()


def test_fused_matches_oracle(dev):
    """Two time steps of the small channel: the fused launch vs the oracle's plain FP64 method,
    within the mixed path's field bound."""
    from karman_taichi_gb300.batch import BatchedChannels
    from karman_taichi_gb300.config import ChannelConfig
    cfg = ChannelConfig("test", 64, 16, 1.0 / 16, 4, (("square", 20, 8, 4),), n_steps=2, max_outer=12)
    b = BatchedChannels([cfg], device=dev, precision="mixed", workers=1)
    s = b.solvers[0]
    st = s.state_numpy()
    prm = O.ChannelParams(nx=cfg.nx, ny=cfg.ny, dx=cfg.dx, dy=cfg.dy, rho=cfg.rho, mu=cfg.mu, dt=cfg.dt,
                          U=cfg.U, alpha_m=cfg.alpha_m, alpha_u=cfg.alpha_u, alpha_p=cfg.alpha_p,
                          eps=cfg.eps, mass_tol=cfg.mass_tol, max_outer=cfg.max_outer)
    orc = O.ChannelOracle(prm, s.solid_np, st["u"], st["v"], st["p"])
    for _ in range(2):
        b.step_fused(1)
        ro = orc.step()
        assert abs(b.records[0][-1][0]["outer"] - len(ro)) <= 1
    st = s.state_numpy()
    for f in ("u", "v", "p"):
        assert _rel(st[f], getattr(orc, f)) <= 1e-5, (f, _rel(st[f], getattr(orc, f)))
    b.close()


def test_fused_poisoned_instance_stops_alone(dev):
    """A NaN in one instance's velocity: that instance reports KC_NONFINITE and stops; the
    others compute what they compute without it."""
    from karman_taichi_gb300.batch import BatchedChannels
    cfgs = _cfgs(3, seed=13, max_outer=6)
    b = BatchedChannels(cfgs, device=dev, precision="mixed", workers=1)
    with torch.no_grad():
        b.solvers[1].u[5, 5] = math.nan
    b.step_fused(2)
    assert b.fused_totals[1]["status"] == 4
    for k in (0, 2):
        assert b.fused_totals[k]["status"] in (0, 1)
        one = BatchedChannels([cfgs[k]], device=dev, precision="mixed", workers=1)
        one.step_fused(2)
        for f in ("u", "v", "p"):
            assert np.array_equal(b.solvers[k].state_numpy()[f], one.solvers[0].state_numpy()[f])
        one.close()
    b.close()


def test_fused_momentum_fallback_tracks_native_step(dev):
    """A 128 x 32 channel with a 15-cell cylinder at Re 181 (instance 238 of the seeded 256-instance
    batch): a few steps in, the Gauss-Seidel momentum solves miss eps and the refined BiCGSTAB takes
    over, in the fused launch as in the native step; the per-step mass residuals stay those of the
    native step (to the solves' tolerance) instead of drifting away."""
    from karman_taichi_gb300.batch import BatchedChannels, batch_configs
    from karman_taichi_gb300.channel import ChannelSolver
    cfg = batch_configs(256, seed=0)[238]
    assert (cfg.nx, cfg.ny, cfg.D) == (128, 32, 15)
    b = BatchedChannels([cfg], device=dev, precision="mixed", workers=1)
    solo = ChannelSolver(cfg, device=dev, precision="mixed", recycle=0)
    fallbacks = 0
    for t in range(12):
        b.step_fused(1)
        fallbacks += b.fused_totals[0]["fallbacks"]
        mf = b.records[0][-1][0]["mass"]
        ms = solo.step()[0]["mass"]
        assert abs(mf - ms) <= 1e-3 * ms + 1e-12, (t, mf, ms)
    assert solo.fallbacks > 0 and fallbacks > 0
    b.close()
