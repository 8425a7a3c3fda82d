"""Batched channel instances: the configuration generator (CPU) and bitwise
equality of an instance run in a batch with the same instance run alone (GPU)."""
import numpy as np
import pytest


def test_batch_configs_follow_the_spec():
    from karman_taichi_gb300.batch import SIZES, batch_configs
    cfgs = batch_configs(256, seed=0)
    assert len(cfgs) == 256 and cfgs == batch_configs(256, seed=0)
    for c in cfgs:
        assert (c.nx, c.ny) in SIZES
        assert 4 <= c.D <= 16 and 60 <= c.Re <= 200
        shape, ci, cj, D = c.obstacles[0]
        assert 0.15 * c.nx - 1 <= ci <= 0.3 * c.nx + 1 and abs(cj - c.ny / 2) <= 0.1 * c.ny + 1
    assert len({c.seed for c in cfgs}) > 250
    mean_cells = np.mean([c.cells for c in cfgs])
    assert 25_000 < mean_cells < 50_000


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_instances_match_solo_runs(dev, precision):
    from karman_taichi_gb300.batch import BatchedChannels, batch_configs
    from karman_taichi_gb300.channel import ChannelSolver
    cfgs = [c.with_(max_outer=8) for c in batch_configs(6, seed=3)]
    b = BatchedChannels(cfgs, device=dev, precision=precision, workers=3)
    b.step(2)
    for cfg, s in zip(cfgs, b.solvers):
        solo = ChannelSolver(cfg, device=dev, precision=precision)
        solo.persistent = False          # the batch solves in graph chunks (another reduction order)
        solo.step(); solo.step()
        a, r = s.state_numpy(), solo.state_numpy()
        for k in ("u", "v", "p"):
            assert np.array_equal(a[k], r[k]), (cfg.name, k)
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision,momentum", [("fp64", "bicgstab"), ("mixed", "bicgstab"), ("mixed", "rbgs"),
                                                ("mixed", "rbgs_refined")])
def test_native_step_matches_python_step(dev, precision, momentum):
    """kc_channel_step makes the calls ChannelSolver's Python loop makes: same fields bit for bit
    (momentum by the refined BiCGSTAB or by Gauss-Seidel)."""
    from karman_taichi_gb300.batch import batch_configs
    from karman_taichi_gb300.channel import ChannelSolver
    cfg = batch_configs(1, seed=5)[0].with_(max_outer=10)
    a = ChannelSolver(cfg, device=dev, precision=precision, native=True, momentum=momentum)
    b = ChannelSolver(cfg, device=dev, precision=precision, native=False, momentum=momentum)
    for _ in range(2):
        ra, rb = a.step(), b.step()
        assert ra[0]["outer"] == len(rb)
        assert ra[0]["it_p"] == sum(r["it_p"] for r in rb)
        assert ra[0]["it_u"] == sum(r["it_u"] for r in rb)
    assert a.fallbacks == b.fallbacks
    sa, sb = a.state_numpy(), b.state_numpy()
    for k in ("u", "v", "p", "u0", "v0"):
        assert np.array_equal(sa[k], sb[k]), k


@pytest.mark.gpu
def test_native_batch_matches_solo_runs(dev):
    from karman_taichi_gb300.batch import BatchedChannels, batch_configs
    from karman_taichi_gb300.channel import ChannelSolver
    cfgs = [c.with_(max_outer=8) for c in batch_configs(8, seed=4)]
    b = BatchedChannels(cfgs, device=dev, precision="mixed", workers=4)
    b.step_native(2)
    for cfg, s in zip(cfgs, b.solvers):
        solo = ChannelSolver(cfg, device=dev, precision="mixed")
        solo.persistent = False
        solo.step(); solo.step()
        a, r = s.state_numpy(), solo.state_numpy()
        for k in ("u", "v", "p"):
            assert np.array_equal(a[k], r[k]), (cfg.name, k)
    b.close()


@pytest.mark.gpu
def test_native_batch_with_graph_cache_eviction(dev):
    """More captured-graph keys than the cache holds: 12 instances (at least three graph keys each:
    workspaces, coefficients and iterates differ) stepped by 6 worker threads with the cache limited
    to 8 entries, so graphs are evicted while other threads launch theirs.  Fields stay bitwise those
    of solo runs, and the cache never holds more than its limit."""
    from karman_taichi_gb300 import _lib as L
    from karman_taichi_gb300.batch import BatchedChannels, batch_configs
    from karman_taichi_gb300.channel import ChannelSolver
    lib = L.load()
    old = lib.kc_graph_cache_limit(8)
    try:
        cfgs = [c.with_(max_outer=6) for c in batch_configs(12, seed=9)]
        b = BatchedChannels(cfgs, device=dev, precision="mixed", workers=6)
        b.step_native(2)
        assert lib.kc_graph_cache_size() <= 8
        for cfg, s in zip(cfgs, b.solvers):
            solo = ChannelSolver(cfg, device=dev, precision="mixed")
            solo.persistent = False
            solo.step(); solo.step()
            a, r = s.state_numpy(), solo.state_numpy()
            for k in ("u", "v", "p"):
                assert np.array_equal(a[k], r[k]), (cfg.name, k)
        b.close()
    finally:
        lib.kc_graph_cache_limit(old)
    assert lib.kc_graph_cache_limit(0) == old
