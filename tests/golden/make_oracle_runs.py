"""Oracle runs too long for a test: the 320 x 64 channel case for all 20 time
steps, computed by the C/OpenMP restatement of the plain FP64 method
(``oracle/kc_cpu.c``, itself pinned to ``oracle/np_oracle.py``'s
ChannelOracle by ``tests/test_cpu_port.py``) and written to
``tests/golden/oracle_channel_320x64_eps*.npz``.

The case: 320 x 64 cells, dx = dy = 1/64, 8 x 8 blocked square at cells
i in [60, 67], j in [28, 35], uniform inlet u = 1, zero-gradient outlet,
no-slip walls, Re = 150 on the block width, dt at CFL 0.5, u = 1 and
v = seeded uniform noise of amplitude 1e-3 (seed 0), p = 0; per time step
SIMPLE outer iterations until the predicted field's max |mdiv| <= 1e-6 or
50 iterations; BiCGSTAB (no preconditioner) to a relative residual eps;
relaxation 0.7 (u, v) and 0.3 (p).  Two runs: eps = 1e-8 (the case as
stated) and eps = 1e-12 (solves taken far enough that two implementations
differ by rounding only, not by where each solve happened to stop).

Usage:  python tests/golden/make_oracle_runs.py [eps ...]   (default: 1e-8 1e-12)
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def run(eps: float, n_steps: int = 20):
    from karman_taichi_gb300 import geometry
    from karman_taichi_gb300.config import PRESETS
    from oracle import cpu
    cfg = PRESETS["channel_320x64"].with_(eps=eps)
    solid = geometry.solid_mask(cfg.nx, cfg.ny, cfg.obstacles)
    u, v, p = geometry.channel_initial_fields(cfg.nx, cfg.ny, solid, U=cfg.U, noise=cfg.noise, seed=cfg.seed)
    u0, v0 = u.copy(), v.copy()
    steps, arrays = [], {}
    t0 = time.time()
    for s in range(n_steps):
        st = cpu.channel_run(cfg, solid, u, v, p, u0, v0, n_steps=1)
        steps.append(dict(outer=st["outer"], mass=st["mass"], solver_iters=st["solver_iters"],
                          seconds=round(st["seconds"], 2)))
        print(s, steps[-1], flush=True)
        if s + 1 in (1, n_steps):
            # float32 copies: the tests compare fields to 1e-6 relative at the tightest, far above the
            # float32 rounding of the stored values
            arrays.update({f"step{s + 1}_{k}": a.astype(np.float32) for k, a in (("u", u), ("v", v), ("p", p))})
    meta = dict(case="channel_320x64", eps=eps, n_steps=n_steps, steps=steps, threads=cpu.threads(),
                seconds=round(time.time() - t0, 1), generated_by="tests/golden/make_oracle_runs.py",
                oracle="oracle/kc_cpu.c (C/OpenMP FP64 plain method)")
    tag = f"{eps:.0e}".replace("-0", "-")
    path = os.path.join(HERE, f"oracle_channel_320x64_eps{tag}.npz")
    np.savez_compressed(path, meta=np.array(json.dumps(meta)), **arrays)
    print(f"wrote {path} ({os.path.getsize(path)} bytes)")


if __name__ == "__main__":
    for e in (sys.argv[1:] or ["1e-8", "1e-12"]):
        run(float(e))
