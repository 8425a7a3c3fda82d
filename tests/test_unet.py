"""Learned initial guess: the U-Net kernels against the CPU restatement.

* CPU: the restatement's analytic backward pass against central differences
  (float64, no bfloat16 rounding) -- pins the oracle.
* GPU: forward output and every parameter gradient of the kc_unet_* kernels
  against the restatement with bfloat16 rounding at the same points
  (tolerance: 2e-2 relative, from summation order and bfloat16 ties).
* GPU: a network trained on p' systems of a small channel lowers the CG
  iterations of held-out p' solves (the gain the learned guess must show).
"""
import numpy as np
import pytest

from oracle import unet_oracle as U


def _features(rng, H, W):
    f = np.zeros((H, W, U.CIN), dtype=np.float32)
    f[..., :4] = rng.standard_normal((H, W, 4)).astype(np.float32)
    return f


def _loss_fd(P, feat, target, weight, key, idx, eps):
    Q = {k: v.copy() for k, v in P.items()}
    Q[key] = Q[key].copy()
    Q[key][idx] += eps
    o = U.UNetOracle(Q, bf16=False, dtype=np.float64)
    lp, _ = o.mse(o.forward(feat)[0], target, weight)
    Q[key][idx] -= 2 * eps
    o = U.UNetOracle(Q, bf16=False, dtype=np.float64)
    lm, _ = o.mse(o.forward(feat)[0], target, weight)
    return (lp - lm) / (2 * eps)


def test_oracle_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    H, W = 16, 24
    P = {k: v.astype(np.float64) for k, v in U.init_params(seed=1).items()}
    for k in P:
        if k.endswith(".b"):
            P[k] = P[k] + 0.05 * rng.standard_normal(P[k].shape)
    feat = _features(rng, H, W).astype(np.float64)
    target = rng.standard_normal((H, W))
    weight = (rng.random((H, W)) > 0.2).astype(np.float64)
    o = U.UNetOracle(P, bf16=False, dtype=np.float64)
    out, A = o.forward(feat)
    _, dout = o.mse(out, target, weight)
    G = o.backward(A, dout)
    for key in ("e0a.w", "e1b.w", "b3a.w", "b3b.b", "d2a.w", "d1a.b", "d0b.w", "head.w", "head.b"):
        flat = np.argsort(-np.abs(G[key]).reshape(-1))[:2]
        for f in flat:
            idx = np.unravel_index(f, G[key].shape)
            fd = _loss_fd(P, feat, target, weight, key, idx, 1e-6)
            assert abs(fd - G[key][idx]) <= 1e-5 * max(abs(fd), 1e-8) + 1e-10, (key, idx, fd, G[key][idx])


@pytest.mark.gpu
def test_unet_forward_and_gradients_match_oracle(dev):
    import torch
    from karman_taichi_gb300 import learned
    rng = np.random.default_rng(5)
    H, W = 32, 72          # two column blocks of the convolution kernel, the second partial
    net = learned.UNet(dev, seed=2)
    P = net.params_numpy()
    for k in P:
        if k.endswith(".b"):
            P[k] = (P[k] + 0.05 * rng.standard_normal(P[k].shape)).astype(np.float32)
    net = learned.UNet(dev, params=P)
    feat = U.to_bf16(_features(rng, H, W))
    target = rng.standard_normal((H, W)).astype(np.float32)
    weight = (rng.random((H, W)) > 0.2).astype(np.float32)
    count = int(weight.sum())
    tf = torch.from_numpy(feat).to(dev).to(torch.bfloat16)
    out = net.forward(tf)
    net.zero_grad()
    loss, dout = net.mse(out, torch.from_numpy(target).to(dev), torch.from_numpy(weight).to(dev), count)
    net.backward(dout)
    torch.cuda.synchronize()
    o = U.UNetOracle(P, bf16=True)
    out_ref, A = o.forward(feat)
    loss_ref, dout_ref = o.mse(out_ref, target, weight)
    G_ref = o.backward(A, dout_ref)
    out_g = out.cpu().numpy()
    assert np.abs(out_g - out_ref).max() <= 2e-2 * np.abs(out_ref).max()
    assert abs(float(loss.item()) - loss_ref) <= 2e-2 * loss_ref
    G = net.grads_numpy()
    for k in G:
        err = np.linalg.norm(G[k] - G_ref[k]) / max(np.linalg.norm(G_ref[k]), 1e-30)
        assert err <= 2e-2, (k, err)


@pytest.mark.gpu
def test_learned_initial_guess_saves_cg_iterations(dev):
    import torch
    from karman_taichi_gb300 import learned, linalg
    from karman_taichi_gb300.channel import ChannelSolver
    from karman_taichi_gb300.config import get
    base = get("channel_2048x512")
    cfg = base.with_(name="channel_256x64", nx=256, ny=64, h=1.0 / 64, D=4, obstacles=(("circle", 50, 32, 4),))
    solver = ChannelSolver(cfg, device=dev, precision="mixed")
    pairs = learned.collect_pairs(solver, 6)
    net = learned.UNet(dev, seed=0)
    before = learned.mean_loss(net, pairs)
    learned.train(net, pairs, 300, lr=1e-3, batch=4)
    after = learned.mean_loss(net, pairs)
    assert after < 0.5 * before, (before, after)
    # held-out systems: a run from another seeded initial state.  The network's
    # own gain is the initial error: ||x0 - p'|| / ||p'|| against 1 for x0 = 0.
    # In CG iterations it pays against the uniform one-sweep cycle (omega 1.1,
    # alpha 1.8, one sweep on every level); the default cycle's per-level
    # weights and sweeps remove the smooth error it predicts within a few
    # iterations themselves.
    solver2 = ChannelSolver(cfg.with_(seed=1), device=dev, precision="mixed")
    weak = linalg.Multigrid(solver2.A_p32, omega=1.1, alpha=1.8, nu_coarse=1)
    guess = learned.LearnedGuess(net)
    it0 = it1 = 0
    errs = []
    for _ in range(6):
        for _ in range(cfg.max_outer):
            solver2.assemble_momentum(); solver2.solve_momentum(); solver2.relax(); solver2.assemble_p()
            solver2.mg.setup()
            weak.setup()
            x = torch.zeros_like(solver2.pcor)
            assert linalg.pcg_refined(solver2.A_p, solver2.A_p32, solver2.b_p, x, solver2.mg, eps=1e-8).ok
            x0 = guess.predict(solver2).clone()
            errs.append(float(torch.linalg.norm(x0 - x) / torch.linalg.norm(x)))
            for start, which in ((None, 0), (x0, 1)):
                y = torch.zeros_like(solver2.pcor)
                info = linalg.pcg_refined(solver2.A_p, solver2.A_p32, solver2.b_p, y, weak, eps=1e-8, x0=start)
                assert info.ok
                if which:
                    it1 += info.iters
                else:
                    it0 += info.iters
            solver2.pcor.copy_(x)
            solver2.correct()
            if float(solver2.mass[0].item()) <= cfg.mass_tol:
                break
        solver2.time_forward()
    assert sum(errs) / len(errs) < 1.0, errs
    assert it1 < it0, (it0, it1, len(errs))


@pytest.mark.gpu
def test_feature_pipeline_matches_oracle(dev):
    """kc_unet_features / pool / target_down2 / guess_up2 against their restatements."""
    import torch
    from karman_taichi_gb300 import learned
    from karman_taichi_gb300.channel import ChannelSolver
    from karman_taichi_gb300.config import get
    cfg = get("channel_2048x512").with_(name="c", nx=200, ny=40, h=1.0 / 40, D=4, obstacles=(("circle", 40, 20, 4),))
    s = ChannelSolver(cfg, device=dev, precision="mixed")
    s.assemble_momentum(); s.solve_momentum(); s.relax(); s.assemble_p(); s.solve_p()
    NX, NY = s.b_p.shape
    fz = learned.Featurizer(NX, NY, dev)
    half = fz(s.b_p, s.coef_p32).float().cpu().numpy()
    b, c32 = s.b_p.cpu().numpy(), s.coef_p32.cpu().numpy()
    feat, fluid, sc = U.features_np(b, c32, fz.H, fz.W)
    assert np.allclose(fz.scales.cpu().numpy(), sc, rtol=1e-12, atol=0)
    assert np.array_equal(fz.fluid.cpu().numpy() > 0, fluid)
    full = fz.full.float().cpu().numpy()
    assert np.abs(full - U.to_bf16(feat)).max() <= 8e-3 * np.abs(feat).max()
    ref_half = U.to_bf16(feat).reshape(fz.Hh, 2, fz.Wh, 2, U.CIN).mean(axis=(1, 3))
    assert np.abs(half - ref_half).max() <= 8e-3 * np.abs(ref_half).max()
    tgt, wgt = fz.target(s.pcor, s.coef_p32)
    t_ref, w_ref = U.target_down2_np(s.pcor.cpu().numpy(), fluid, sc[2], fz.Hh, fz.Wh)
    assert np.allclose(tgt.cpu().numpy(), t_ref, rtol=1e-5, atol=1e-6 * np.abs(t_ref).max())
    assert np.array_equal(wgt.cpu().numpy(), w_ref)
    out = torch.from_numpy(t_ref.astype(np.float32)).to(dev)
    x0 = torch.zeros((NX, NY), dtype=torch.float64, device=dev)
    fz.guess(out, s.coef_p32, x0)
    ref = U.guess_up2_np(t_ref.astype(np.float32).astype(np.float64), fluid, sc[2])
    assert np.abs(x0.cpu().numpy() - ref).max() <= 1e-5 * np.abs(ref).max()
