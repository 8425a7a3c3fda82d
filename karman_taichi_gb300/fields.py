"""Headless field output: post-processing on the GPU, CSV and image files.

* :func:`post_process_field` -- karman_taichi.py:545-583 (cell-centre
  velocities, cell divergence, the five display canvases scaled to [0, 1]) by
  ``kc_post_process``.
* :func:`write_matrix` -- karman_taichi.py:157-159: ``np.savetxt(name +
  ".csv", field, delimiter=",")``, the same file format.
* :func:`write_timestep` -- the every-10-steps dump of karman_taichi.py:677-683
  (``timestep{step:06}_{pcor,p,u,v,udiv}.csv``).
* :func:`write_pgm` -- a display canvas as an 8-bit greyscale PGM image, the
  headless stand-in for the ti.GUI PNG (karman_taichi.py:670-674): i along the
  image's x axis, j upwards, as the GUI shows it.
* ``SIMPLESolver.dump_matrix`` / ``dump_coef`` (simple.py:51-75) are in
  ``simple.py`` and write through :func:`savetxt`.
"""
from __future__ import annotations

import os

import numpy as np
import torch

from . import _lib as L
from .linalg import ptr, require_cuda, stream_handle

CANVASES = ("u", "v", "p", "pcor", "udiv")


class PostProcessor:
    """Device buffers for post_process_field on one [nx, ny] grid."""

    def __init__(self, nx, ny, device="cuda"):
        self.nx, self.ny = nx, ny
        self.device = torch.device(device)
        f = dict(dtype=torch.float64, device=self.device)
        self.u_post = torch.zeros((nx + 2, ny + 2), **f)
        self.v_post = torch.zeros((nx + 2, ny + 2), **f)
        self.minmax = torch.zeros(10, **f)
        self.disp = torch.zeros((5, 3 * (nx + 2), 3 * (ny + 2)), dtype=torch.float32, device=self.device)
        self.ws = torch.zeros(L.load().kc_post_process_ws_bytes(), dtype=torch.uint8, device=self.device)

    def __call__(self, u, v, p, pcor, udiv, dx, dy, canvases=True):
        require_cuda(u, v, p, pcor, udiv)
        L.check(L.load().kc_post_process(self.nx, self.ny, float(dx), float(dy), ptr(u), ptr(v), ptr(p), ptr(pcor),
                                         ptr(self.u_post), ptr(self.v_post), ptr(udiv), ptr(self.minmax),
                                         ptr(self.disp) if canvases else None, ptr(self.ws), self.ws.numel(),
                                         stream_handle(self.device)), "kc_post_process")
        out = {"u_post": self.u_post, "v_post": self.v_post, "udiv": udiv, "minmax": self.minmax}
        if canvases:
            for k, name in enumerate(CANVASES):
                out[name + "_disp"] = self.disp[k]
        return out


def post_process_field(u, v, p, pcor, udiv, dx, dy, canvases=True, pp=None):
    """karman_taichi.py:545-583 on device tensors; udiv is updated in place on the interior."""
    nx, ny = p.shape[0] - 2, p.shape[1] - 2
    pp = pp or PostProcessor(nx, ny, p.device)
    return pp(u, v, p, pcor, udiv, dx, dy, canvases)


def savetxt(path, field):
    """np.savetxt with the reference's delimiter (default '%.18e' format)."""
    a = field.detach().cpu().numpy() if isinstance(field, torch.Tensor) else np.asarray(field)
    np.savetxt(path, a, delimiter=",")


def write_matrix(mat, name):
    """karman_taichi.py:157-159."""
    print("    >> Writing matrix data to", name, ".csv ...")
    savetxt(name + ".csv", mat)


def write_timestep(step, fields, directory="."):
    """The dump of karman_taichi.py:677-683: timestep{step:06}_{name}.csv for
    pcor, p, u, v, udiv (fields: a dict with those keys)."""
    os.makedirs(directory, exist_ok=True)
    paths = []
    for name in ("pcor", "p", "u", "v", "udiv"):
        path = os.path.join(directory, f"timestep{step:06}_{name}")
        write_matrix(fields[name], path)
        paths.append(path + ".csv")
    return paths


def write_pgm(canvas, path):
    """An [I][J] canvas with values in [0, 1] as a binary PGM (P5), I along x, J upwards."""
    a = canvas.detach().cpu().numpy() if isinstance(canvas, torch.Tensor) else np.asarray(canvas)
    img = np.clip(np.rint(a.T[::-1] * 255.0), 0, 255).astype(np.uint8)
    with open(path, "wb") as f:
        f.write(b"P5\n%d %d\n255\n" % (img.shape[1], img.shape[0]))
        f.write(np.ascontiguousarray(img).tobytes())
    return path


def read_pgm(path):
    """Inverse of write_pgm (for tests): the canvas rounded to 1/255."""
    with open(path, "rb") as f:
        data = f.read()
    parts = data.split(b"\n", 3)
    w, h = map(int, parts[1].split())
    img = np.frombuffer(parts[3], dtype=np.uint8).reshape(h, w)
    return img[::-1].T.astype(np.float64) / 255.0
