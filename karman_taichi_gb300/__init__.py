"""karman_taichi_gb300 -- GB300-native kernels for the karman_taichi SIMPLE hot path.

Drop-in modules mirroring the reference's entry points:

* ``karman_taichi_gb300.bicgsolver.BICGSolver``  (bicgsolver.py)
* ``karman_taichi_gb300.cgsolver.CGSolver``      (cgsolver.py)
* ``karman_taichi_gb300.simple.SIMPLESolver``    (simple.py / bicgsimp.py)
* ``karman_taichi_gb300.karman_taichi``          (karman_taichi.py functions)
* ``karman_taichi_gb300.channel.ChannelSolver``  (the channel benchmark cases)

All compute runs in ``libkarman_gb300.so`` (sm_103a CUDA, C ABI in
``include/karman_gb300.h``); there is no CPU fallback.
"""
from . import _lib
from ._lib import KcError, KcLibraryMissing, load

__all__ = ["KcError", "KcLibraryMissing", "load", "lib_version"]


def lib_version() -> int:
    return load().kc_version()
