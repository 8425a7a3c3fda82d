"""Launch-shape autotuner for the accelerated pressure-correction solve.

The multigrid-preconditioned CG has three free choices that change its
launches but not its arithmetic:

* which coarse levels run in the one-block tail (``Multigrid.opts.tail``,
  cells per level; 0 launches every level separately);
* which levels below level 0 use the large tiles (64-wide staged rows:
  16 x 60, 12 x 56 or 8 x 52 owned cells for one, two or three sweeps)
  instead of the small ones (32-wide rows: 8 x 28, 8 x 24, 8 x 20)
  (``Multigrid.opts.big_cells``);
* how many CG iterations one captured graph chunk holds before the host reads
  the solver state (``ChannelSolver.check_every_p``): fewer host round trips
  against more launches of iterations that return at once once the solve has
  converged.

:func:`tune_pressure` times the solver's own p' solve under each candidate,
one choice after the other (coordinate descent from the defaults), and keeps
the fastest.  Every candidate computes the same fields bit for bit: the tail
and the tile shapes do the same arithmetic per cell, and the convergence test
runs on the device every iteration, whatever the chunk length.

Optionally (``cycles``) it first picks the iteration schedule of the cycle
itself: the red-black sweeps on the levels below level 0
(``Multigrid.opts.nu_coarse``) with the smoother weight that goes with them.
More sweeps cost more per V-cycle and save CG iterations; which wins depends
on the grid (on GB300: three sweeps at 2048 x 512 and 4096 x 1024, two at
320 x 64 and on the random 1024^2 system).  This choice changes the iterates
-- every candidate still solves to the same tolerance -- so it is opt-in.
"""
from __future__ import annotations

import math

import torch

from .linalg import TAIL_CELLS

TAIL_CANDIDATES = (0, 384, TAIL_CELLS, 4352)
BIG_CANDIDATES = (60000, 200000, 600000)
CHUNK_CANDIDATES = (2, 4, 8)
# (sweeps on the levels below level 0, their smoother weight): the weight measured best for each
# sweep count over the channel's p' systems
CYCLE_CANDIDATES = ((2, 1.5), (3, 1.6))


def _solve_ms(solver, reps: int) -> float:
    """Best CUDA-event time of solver.solve_p() from p' = 0 (the first run of a
    new launch shape also captures its graphs and is not timed)."""
    dev = solver.device
    best = math.inf
    for k in range(reps + 1):
        solver.pcor.zero_()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        solver.solve_p()
        e1.record()
        torch.cuda.synchronize(dev)
        if k > 0:
            best = min(best, e0.elapsed_time(e1))
    return best


def _apply(solver, tail: int, big: int, chunk: int) -> None:
    solver.mg.opts.tail = int(tail)
    solver.mg.opts.big_cells = int(big)
    solver.check_every_p = int(chunk)
    solver._chan = None   # the native descriptor copies these: rebuild it


def _apply_cycle(solver, nu: int, omega: float) -> None:
    """Sweeps and smoother weight of the levels below level 0 (the p' solve's
    own kc_mg_setup recomputes the weights it derives from them)."""
    o = solver.mg.opts
    o.nu_coarse = int(nu)
    for l in range(1, len(o.omega)):
        o.omega[l] = float(omega)
    solver._chan = None


def apply_choice(solver, choice: dict) -> None:
    """Apply a :func:`tune_pressure` result to another solver of the same grid."""
    if "nu_coarse" in choice:
        _apply_cycle(solver, choice["nu_coarse"], choice["omega_coarse"])
    _apply(solver, choice["tail"], choice["big_cells"], choice["check_every_p"])


def tune_pressure(solver, reps: int = 3, tails=TAIL_CANDIDATES, bigs=BIG_CANDIDATES,
                  chunks=CHUNK_CANDIDATES, cycles=None) -> dict:
    """Pick the fastest launch shapes of ``solver``'s p' solve on its current
    state and apply them; with ``cycles`` (e.g. CYCLE_CANDIDATES: (nu_coarse,
    omega below level 0) pairs) first the fastest cycle.  Runs one outer
    iteration's stages up to the p' assembly on the solver itself, then puts
    every field back, so the solver continues exactly as if it had not been
    tuned (bit for bit without ``cycles``).  Returns the choice and the
    timings (ms per p' solve) behind it."""
    if solver.mg is None:
        raise ValueError("tuning needs the multigrid p' solve (precision='mixed', pcorr_precond='mg')")
    names = ("u", "v", "p", "u0", "v0", "u_mid", "v_mid", "pcor")
    saved = {k: getattr(solver, k).clone() for k in names}
    fallbacks, history = solver.fallbacks, list(solver.history)
    # the trial solves start from zero and leave the ring of earlier p' solutions untouched
    recycle = getattr(solver, "recycle", 0)
    solver.recycle = 0
    try:
        solver.assemble_momentum()
        solver.solve_momentum()
        solver.relax()
        solver.assemble_p()
        o = solver.mg.opts
        cycle = (int(o.nu_coarse), round(float(o.omega[1]), 6))
        if cycles:
            cyc_ms = {}
            for nu, om in cycles:
                _apply_cycle(solver, nu, om)
                cyc_ms[(int(nu), round(float(om), 6))] = _solve_ms(solver, reps)
            cycle = min(cyc_ms, key=cyc_ms.get)
            _apply_cycle(solver, *cycle)
        choice = {"tail": int(solver.mg.opts.tail), "big_cells": int(solver.mg.opts.big_cells),
                  "check_every_p": int(solver.check_every_p)}
        timings = {}

        def measure(c):
            key = (c["tail"], c["big_cells"], c["check_every_p"])
            if key not in timings:
                _apply(solver, *key)
                timings[key] = _solve_ms(solver, reps)
            return timings[key]

        for field, cands in (("tail", tails), ("big_cells", bigs), ("check_every_p", chunks)):
            best_v, best_t = choice[field], measure(choice)
            for v in cands:
                t = measure(dict(choice, **{field: v}))
                if t < best_t:
                    best_v, best_t = v, t
            choice[field] = best_v
        _apply(solver, choice["tail"], choice["big_cells"], choice["check_every_p"])
        result = dict(choice, nu_coarse=cycle[0], omega_coarse=cycle[1],
                      ms=round(timings[(choice["tail"], choice["big_cells"], choice["check_every_p"])], 4),
                      tried={f"tail={k[0]},big_cells={k[1]},check_every_p={k[2]}": round(t, 4)
                             for k, t in timings.items()})
        if cycles:
            result["tried"].update({f"nu_coarse={k[0]},omega_coarse={k[1]}": round(t, 4) for k, t in cyc_ms.items()})
    finally:
        for k in names:
            getattr(solver, k).copy_(saved[k])
        solver.fallbacks, solver.history = fallbacks, history
        solver.recycle = recycle
        torch.cuda.synchronize(solver.device)
    return result
