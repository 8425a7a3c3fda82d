"""ctypes front end of oracle/libkc_cpu.so (C/OpenMP FP64 channel plain path).
Test infrastructure and timed CPU baseline only."""
import ctypes as C
import os

import numpy as np

from . import build_c


class CpuParams(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("dx", C.c_double), ("dy", C.c_double), ("rho", C.c_double),
                ("mu", C.c_double), ("dt", C.c_double), ("U", C.c_double), ("alpha_m", C.c_double),
                ("alpha_u", C.c_double), ("alpha_p", C.c_double), ("eps", C.c_double), ("mass_tol", C.c_double),
                ("max_outer", C.c_int)]


_lib = None


def load():
    global _lib
    if _lib is None:
        h = C.CDLL(build_c.build())
        h.kc_cpu_channel_run.restype = C.c_int
        h.kc_cpu_channel_run.argtypes = [C.POINTER(CpuParams)] + [C.c_void_p] * 6 + [C.c_int, C.c_long, C.c_long,
                                                                                      C.c_void_p]
        h.kc_cpu_threads.restype = C.c_int
        h.kc_cpu_set_threads.restype = None
        h.kc_cpu_set_threads.argtypes = [C.c_int]
        _lib = h
    return _lib


def threads() -> int:
    return load().kc_cpu_threads()


def set_threads(n: int) -> None:
    load().kc_cpu_set_threads(int(n))


def params_of(cfg) -> CpuParams:
    return CpuParams(cfg.nx, cfg.ny, cfg.dx, cfg.dy, cfg.rho, cfg.mu, cfg.dt, cfg.U, cfg.alpha_m, cfg.alpha_u,
                     cfg.alpha_p, cfg.eps, cfg.mass_tol, cfg.max_outer)


def channel_run(cfg, solid, u, v, p, u0=None, v0=None, n_steps=1, max_total_outer=10**9, max_solver_iter=10**12):
    """Runs the C baseline in place on float64 numpy arrays; returns a dict of
    stats (outer iterations, completed steps, solver iterations, mass, seconds)."""
    lib = load()
    u0 = u.copy() if u0 is None else u0
    v0 = v.copy() if v0 is None else v0
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (u, v, p, u0, v0)]
    for a, b in zip(arrs, (u, v, p, u0, v0)):
        assert a is b, "arrays must be contiguous float64 (updated in place)"
    sol = np.ascontiguousarray(solid, dtype=np.uint8)
    stats = np.zeros(5)
    P = params_of(cfg)
    rc = lib.kc_cpu_channel_run(C.byref(P), sol.ctypes.data, u.ctypes.data, v.ctypes.data, p.ctypes.data,
                                u0.ctypes.data, v0.ctypes.data, int(n_steps), int(max_total_outer), int(max_solver_iter),
                                stats.ctypes.data)
    if rc != 0:
        raise RuntimeError("kc_cpu_channel_run failed")
    return dict(outer=int(stats[0]), steps=int(stats[1]), solver_iters=int(stats[2]), mass=float(stats[3]),
                seconds=float(stats[4]))
