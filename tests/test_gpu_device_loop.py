"""The multigrid CG's device-side iteration loop (a conditional WHILE graph node) against the
chunked graphs with a host check between chunks (kc_device_loop): same kernels, same results."""
import pytest

pytestmark = pytest.mark.gpu


def test_device_loop_and_chunked_graphs_agree_bitwise(dev):
    import torch
    from karman_taichi_gb300 import _lib as L, linalg
    from karman_taichi_gb300.channel import ChannelSolver
    from karman_taichi_gb300.config import ChannelConfig
    cfg = ChannelConfig("loop", 256, 64, 1.0 / 64, 8, (("circle", 60, 32, 8),), max_outer=6)
    s = ChannelSolver(cfg, device=dev, precision="mixed", recycle=0)
    s.step()
    s.assemble_momentum(); s.solve_momentum(); s.relax(); s.assemble_p()
    s.mg.setup()
    lib = L.load()
    prev = lib.kc_device_loop(-1)
    try:
        out = {}
        for loop in (1, 0):
            assert lib.kc_device_loop(loop) in (0, 1)
            x = torch.zeros_like(s.b_p)
            info = linalg.pcg_refined(s.A_p, s.A_p32, s.b_p, x, s.mg, eps=1e-8)
            assert info.ok, info
            out[loop] = (x, info.iters)
        assert out[1][1] == out[0][1]
        assert torch.equal(out[1][0], out[0][0])
    finally:
        lib.kc_device_loop(prev)
