"""Headless field output: post_process_field (karman_taichi.py:545-583) on the
GPU against the NumPy restatement, and the file formats of write_matrix
(karman_taichi.py:157-159), the timestep dump (:677-683), SIMPLESolver's
dump_matrix / dump_coef (simple.py:51-75) and the PGM canvases."""
import os

import numpy as np
import pytest

from oracle import np_oracle as O


def test_write_matrix_is_numpy_savetxt(tmp_path):
    from karman_taichi_gb300 import fields
    a = np.random.default_rng(0).standard_normal((7, 5))
    fields.write_matrix(a, str(tmp_path / "m"))
    ref = tmp_path / "ref.csv"
    np.savetxt(ref, a, delimiter=",")
    assert (tmp_path / "m.csv").read_bytes() == ref.read_bytes()
    assert np.array_equal(np.loadtxt(tmp_path / "m.csv", delimiter=","), a)


def test_pgm_round_trip(tmp_path):
    from karman_taichi_gb300 import fields
    c = np.random.default_rng(1).random((12, 9))
    path = fields.write_pgm(c, str(tmp_path / "c.pgm"))
    back = fields.read_pgm(path)
    assert back.shape == c.shape
    assert np.abs(back - c).max() <= 0.5 / 255 + 1e-12
    with open(path, "rb") as f:
        assert f.read(2) == b"P5"


@pytest.mark.gpu
def test_post_process_matches_oracle(dev):
    import torch
    from karman_taichi_gb300 import fields
    rng = np.random.default_rng(2)
    nx, ny, dx, dy = 61, 23, 0.03, 0.02
    u = rng.standard_normal((nx + 3, ny + 2)) + 1.0
    v = rng.standard_normal((nx + 2, ny + 3))
    p = rng.standard_normal((nx + 2, ny + 2)) + 5.0      # all positive: the minimum is not 0
    pc = rng.standard_normal((nx + 2, ny + 2)) - 3.0     # all negative: the maximum is the starting 0
    udiv0 = rng.standard_normal((nx + 2, ny + 2))        # halo entries must be left as they are
    t = lambda a: torch.from_numpy(a).to(dev)
    ud = t(udiv0)
    out = fields.post_process_field(t(u), t(v), t(p), t(pc), ud, dx, dy)
    up, vp, udr, mm, disp = O.post_process_field(u, v, p, pc, udiv0, dx, dy)
    assert np.array_equal(out["u_post"].cpu().numpy(), up)
    assert np.array_equal(out["v_post"].cpu().numpy(), vp)
    assert np.abs(ud.cpu().numpy() - udr).max() <= 1e-15 * np.abs(udr).max()
    assert np.allclose(out["minmax"].cpu().numpy().reshape(5, 2), mm, rtol=1e-15, atol=0)
    for k, name in enumerate(fields.CANVASES):
        assert np.abs(out[name + "_disp"].cpu().numpy() - disp[k]).max() <= 1e-6, name


@pytest.mark.gpu
def test_channel_write_fields(dev, tmp_path):
    from karman_taichi_gb300.channel import ChannelSolver
    from karman_taichi_gb300.config import get
    cfg = get("channel_320x64").with_(nx=64, ny=16, h=1 / 16, D=2, obstacles=(("square", 16, 8, 2),))
    s = ChannelSolver(cfg, device=dev, precision="fp64")
    s.step()
    paths = s.write_fields(10, str(tmp_path), images=True)
    names = sorted(os.path.basename(q) for q in paths)
    assert "timestep000010_p.csv" in names and "timestep000010_udiv.csv" in names and "timestep000010_u.pgm" in names
    assert np.array_equal(np.loadtxt(tmp_path / "timestep000010_u.csv", delimiter=","), s.u.cpu().numpy())
    st = s.state_numpy()
    _, _, udiv, _, disp = O.post_process_field(st["u"], st["v"], st["p"], st["pcor"], np.zeros_like(st["p"]),
                                               cfg.dx, cfg.dy)
    assert np.abs(np.loadtxt(tmp_path / "timestep000010_udiv.csv", delimiter=",") - udiv).max() <= 1e-15
    from karman_taichi_gb300 import fields
    assert np.abs(fields.read_pgm(str(tmp_path / "timestep000010_p.pgm")) - disp[2]).max() <= 0.5 / 255 + 1e-6


@pytest.mark.gpu
def test_simple_dump_files(dev, tmp_path):
    from karman_taichi_gb300.simple import SIMPLESolver
    s = SIMPLESolver(1.0, 1.0, 16, 16, device=dev)
    s.dump_matrix(3, "x", directory=str(tmp_path))
    s.dump_coef(3, "x", directory=str(tmp_path))
    names = set(os.listdir(tmp_path))
    for n in ("000003-u-x.csv", "000003-pcor-x.csv", "000003-mdiv-x.csv", "000003-apu-x.csv", "000003-asv-x.csv",
              "000003-bu -x.csv", "000003-bp -x.csv"):
        assert n in names, n
    assert np.array_equal(np.loadtxt(tmp_path / "000003-aep-x.csv", delimiter=","), s.coef_p[2].cpu().numpy())
