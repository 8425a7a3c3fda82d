"""The lid-driven cavity of bicgsimp.py, run to its substep cap on the GPU,
and the centreline profiles its plot compares with Ghia et al. (1982).

bicgsimp.py:355-371 sets up a 50 x 50 cavity (lx = ly = 1, lid u = 1,
mu = 0.01, rho = 1: Re = 100) and runs at most 10000 SIMPLE substeps
(bicgsimp.py:311-328), plotting u at x = 0.5 (``u[26, 1:51]``) against y and
v at y = 0.5 (``v[1:51, 26]``) against x, both at the cell centres
0.01, 0.03, .. 0.99 (bicgsimp.py:291-305), over the centreline data of
data/ghia1982.dat.  This script runs the same case through the drop-in
``karman_taichi_gb300.simple.SIMPLESolver(bicgsimp=True)`` and writes those
two profiles and the last residuals to
``tests/golden/cavity_bicgsimp_50x50_profiles.npz`` -- this build's own output,
no reference data.  ``compare_ghia.py`` sets them against the data file.

Usage (a GPU is needed):  python tests/golden/make_cavity_profiles.py [substeps] [output.npz]
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    n = int(argv[0]) if argv else 10000
    out = argv[1] if len(argv) > 1 else os.path.join(HERE, "cavity_bicgsimp_50x50_profiles.npz")
    import torch
    from karman_taichi_gb300.simple import SIMPLESolver
    s = SIMPLESolver(1.0, 1.0, 50, 50, bicgsimp=True)
    s.bc["n"][1] = 1.0
    last = {}

    def cb(step, mres, cres):
        last.update(step=step, momentum=mres, continuity=cres)

    t0 = time.time()
    s.solve(n_steps=n, callback=cb)
    torch.cuda.synchronize()
    u = s.u.cpu().numpy()
    v = s.v.cpu().numpy()
    np.savez(out, coord=np.linspace(0.01, 0.99, 50), u_at_x05=u[26, 1:51], v_at_y05=v[1:51, 26],
             substeps=last.get("step", -1) + 1, momentum_residual=last.get("momentum", np.nan),
             continuity_residual=last.get("continuity", np.nan))
    print(f"{last.get('step', -1) + 1} substeps in {time.time() - t0:.1f} s; last momentum residual "
          f"{last.get('momentum')}, continuity {last.get('continuity')}; wrote {out}")


if __name__ == "__main__":
    main()
