"""Sets the cavity centreline profiles of make_cavity_profiles.py against the
Ghia et al. (1982) Re = 100 columns of the reference's data/ghia1982.dat,
read from the reference tree at run time (its values are not copied into
this repository).  The profiles are linearly interpolated at Ghia's
coordinates, with the wall values (u = 0 at y = 0, the lid's u = 1 at y = 1;
v = 0 at both walls) at the ends.

Usage:  python tests/golden/compare_ghia.py [path/to/ghia1982.dat]
        (default: /root/reference/data/ghia1982.dat)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def compare(ghia_path, prof_path=os.path.join(HERE, "cavity_bicgsimp_50x50_profiles.npz")):
    y_ref, u_ref = np.loadtxt(ghia_path, unpack=True, skiprows=2, usecols=(0, 1))
    x_ref, v_ref = np.loadtxt(ghia_path, unpack=True, skiprows=2, usecols=(6, 7))
    d = np.load(prof_path)
    c = d["coord"]
    yc = np.concatenate([[0.0], c, [1.0]])
    uc = np.concatenate([[0.0], d["u_at_x05"], [1.0]])
    vc = np.concatenate([[0.0], d["v_at_y05"], [0.0]])
    du = np.interp(y_ref, yc, uc) - u_ref
    dv = np.interp(x_ref, yc, vc) - v_ref
    return {"substeps": int(d["substeps"]), "momentum_residual": float(d["momentum_residual"]),
            "continuity_residual": float(d["continuity_residual"]),
            "u_max_abs_dev": float(np.abs(du).max()), "u_rms_dev": float(np.sqrt((du ** 2).mean())),
            "v_max_abs_dev": float(np.abs(dv).max()), "v_rms_dev": float(np.sqrt((dv ** 2).mean())),
            "u_min": float(d["u_at_x05"].min()), "u_min_ghia": float(u_ref.min()),
            "v_max": float(d["v_at_y05"].max()), "v_max_ghia": float(v_ref.max()),
            "v_min": float(d["v_at_y05"].min()), "v_min_ghia": float(v_ref.min())}


if __name__ == "__main__":
    path = sys.argv[1] if len(sys.argv) > 1 else "/root/reference/data/ghia1982.dat"
    for k, v in compare(path).items():
        print(f"{k}: {v}")
