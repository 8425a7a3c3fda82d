"""Channel-flow presets (blocked-cell cylinder in a channel).

``channel_320x64`` is the 320 x 64 plain-method case (dx = dy = 1/64, 8 x 8
square block centred at cell (64, 32) = cells i in [60, 67], j in [28, 35],
Re = 150, 20 time steps).  ``channel_2048x512`` is the 2048 x 512 case with a
32-cell cylinder at (400, 256) (dx = dy = 1/512 by analogy with the smaller
case, 200 time steps), and ``channel_4096x1024`` the 4096 x 1024 two-cylinder
Re = 400 case.  Cell indices are the padded-array indices used by the
reference (interior cells i in [1, nx], j in [1, ny]).

``karman_640x128`` / ``karman_320x64`` are the reference's own drivers
(karman_taichi.py:7-25; debug/karman_taichi.py:11-12).
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace


@dataclass(frozen=True)
class ChannelConfig:
    name: str
    nx: int
    ny: int
    h: float                      # dx = dy
    D: int                        # obstacle diameter in cells (defines Re)
    obstacles: tuple = ()         # ((shape, ci, cj, D), ...)
    Re: float = 150.0
    U: float = 1.0
    rho: float = 1.0
    cfl: float = 0.5
    alpha_m: float = 0.7          # momentum under-relaxation
    alpha_u: float = 1.0          # velocity-correction factor
    alpha_p: float = 0.3          # pressure under-relaxation
    eps: float = 1e-8             # inner solver relative tolerance
    mass_tol: float = 1e-6        # outer SIMPLE stop: max |mdiv| of the predicted field
    max_outer: int = 50
    n_steps: int = 20
    noise: float = 1e-3           # amplitude of the seeded uniform noise on v
    seed: int = 0
    copies: int = 1

    @property
    def dx(self) -> float:
        return self.h

    @property
    def dy(self) -> float:
        return self.h

    @property
    def lx(self) -> float:
        return self.nx * self.h

    @property
    def ly(self) -> float:
        return self.ny * self.h

    @property
    def mu(self) -> float:
        return self.rho * self.U * (self.D * self.h) / self.Re

    @property
    def dt(self) -> float:
        return self.cfl * self.h / self.U

    @property
    def cells(self) -> int:
        return self.nx * self.ny

    def with_(self, **kw) -> "ChannelConfig":
        return replace(self, **kw)


PRESETS = {
    "channel_320x64": ChannelConfig("channel_320x64", 320, 64, 1.0 / 64, 8, (("square", 64, 32, 8),),
                                    Re=150.0, n_steps=20),
    "channel_2048x512": ChannelConfig("channel_2048x512", 2048, 512, 1.0 / 512, 32, (("circle", 400, 256, 32),),
                                      Re=150.0, n_steps=200),
    "channel_4096x1024": ChannelConfig("channel_4096x1024", 4096, 1024, 1.0 / 1024, 48,
                                       (("circle", 600, 400, 48), ("circle", 600, 624, 48)),
                                       Re=400.0, n_steps=1000, copies=4),
}


@dataclass(frozen=True)
class KarmanConfig:
    """Constants of karman_taichi.py:7-25 (module globals of the reference)."""
    nx: int = 640
    ny: int = 128
    lx: float = 0.5
    ly: float = 0.1
    rho: float = 1.0
    mu: float = 0.01
    dt: float = 0.00001
    velo_rel: float = 0.8
    p_rel: float = 0.2
    circle: tuple = (64, 32, 144)      # (ci, cj, r^2): karman_taichi.py:149
    eps: float = 1e-8
    max_sub: int = 500                 # karman_taichi.py:633
    pcor_ratio: float = 1e-4           # karman_taichi.py:655

    @property
    def dx(self) -> float:
        return self.lx / self.nx

    @property
    def dy(self) -> float:
        return self.ly / self.ny


KARMAN_PRESETS = {
    "karman_640x128": KarmanConfig(),
    "karman_320x64": KarmanConfig(nx=320, ny=64),
}


def get(name: str):
    if name in PRESETS:
        return PRESETS[name]
    if name in KARMAN_PRESETS:
        return KARMAN_PRESETS[name]
    raise KeyError(f"unknown preset {name!r}; known: {sorted(PRESETS) + sorted(KARMAN_PRESETS)}")
