#!/usr/bin/env python
"""Time steps/s of the channel SIMPLE hot path (karman_taichi) on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--config channel_2048x512] [--mode fp64|mixed|learned]

One "step" is one time step of the channel case: SIMPLE outer iterations
(momentum assembly + BiCGSTAB u/v solves, relaxation, pressure-correction
assembly + BiCGSTAB p' solve, correction) until the predicted field's mass
residual <= 1e-6 or 50 outer iterations, then u0 <- u.  W untimed warm-up
steps, then exactly K timed steps between barriers + synchronizes, CUDA
events on the solver stream, max over ranks.  Inputs: seeded synthetic
channel initial state.  The working set of one step (fields, three systems of
coefficient planes and the solver workspaces, several hundred MB) is larger
than the 129 MB L2, so no separate L2 flush is inserted.

Under torchrun every rank advances its own replica (replicas only: the path
has no exchange step) and `value` is all ranks' time steps / the slowest
rank's time.

`--impl reference` times the CPU restatement of the same plain method
(oracle/kc_cpu.c, C + OpenMP, FP64) on all host cores: whole time steps of
the seeded case from its initial state, every solve to convergence.  A
2048 x 512 time step is about a minute of CPU work, so the arm times as many
whole steps as fit its budget (at least one) and reports that count as
"steps"; nothing is extrapolated.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Time steps/s at 2048x512: learned+mixed vs plain BiCGSTAB, same GB300, resid<=1e-6"
# (the value line runs the fastest accelerated configuration; the learned variant is reported beside it)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="channel_2048x512")
    ap.add_argument("--mode", default="auto", choices=["auto", "fp64", "mixed", "learned"])
    ap.add_argument("--momentum", default="rbgs_refined", choices=["rbgs_refined", "bicgstab", "rbgs"],
                    help="momentum solver of the mixed path (ChannelSolver(momentum=...))")
    ap.add_argument("--compare-steps", type=int, default=2, help="timed steps of the FP64 plain comparison run")
    ap.add_argument("--no-compare", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default cycle and launch shapes of the p' solve instead of tuning them "
                         "before timing")
    ap.add_argument("--cpu-budget", type=float, default=150.0,
                    help="seconds of whole CPU time steps (at least one step is always timed)")
    ap.add_argument("--spmv-sweep", action="store_true",
                    help="time k_spmv (FP64, FP32) on random 5-point systems of 1M, 4M and 17M cells and exit")
    ap.add_argument("--pcorr1024", action="store_true",
                    help="the isolated 1024 x 1024 pressure-correction solve (random aP, 5%% blocked blobs), plain "
                         "FP64 BiCGSTAB and FP32 multigrid CG in FP64 refinement, to rel. tol 1e-8, and exit")
    ap.add_argument("--batch-instances", type=int, default=0, metavar="N",
                    help="time the batched configuration (N independent channel instances, stream-parallel) and exit")
    ap.add_argument("--batch-workers", type=int, default=16)
    ap.add_argument("--batch-executors", default="fused,native",
                    help="comma-separated executors of the batched configuration, timed in turn: fused (one "
                         "persistent launch for all instances and steps), native (one stream per instance, native "
                         "threads), sequential (one stream); the first gives the line's value")
    ap.add_argument("--copies", type=int, default=0, metavar="N",
                    help="step N seeded copies of --config concurrently (the batch executor) and one after another")
    ap.add_argument("--long-run", type=int, default=0, metavar="N",
                    help="the long run of --config (default channel_4096x1024): its seeded copies advanced "
                         "together for N time steps with wake probes (shedding period and its drift), then the "
                         "plain FP64 method's first --fp64-steps steps against copy 0, and exit")
    ap.add_argument("--fp64-steps", type=int, default=0,
                    help="the long run's FP64 comparison: steps of the plain method against copy 0 (at 4096x1024 "
                         "its p' BiCGSTAB stagnates within the first step)")
    ap.add_argument("--no-device-loop", action="store_true",
                    help="run the multigrid CG's iterations as graph-captured chunks instead of a conditional "
                         "WHILE graph node (kc_device_loop(0)): the same kernels, listed by ncu")
    ap.add_argument("--profile-outer", type=int, default=0, metavar="N",
                    help="run N SIMPLE outer iterations of --mode from the seeded state, untimed, and exit "
                         "(the command the committed ncu summaries were captured on)")
    return ap.parse_args()


# ---------------------------------------------------------------------------------------------
class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                power.append(float(r[3]))
                for nm, val in zip(names, r[5:9]):
                    if val.strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w_max": max(power) if power else None}


def dist_init(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    """The slowest rank's value (every rank gets it); on the process group's own
    device (CUDA under NCCL, the host under gloo)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(world, steps, ms):
    """Whole-job time steps/s of `world` replicas that each advanced `steps`
    time steps, over the slowest rank's time `ms` (weak scaling)."""
    return world * steps / (ms * 1e-3)


# ---------------------------------------------------------------------------------------------
def make_solver(cfg, mode, dev, momentum="rbgs_refined"):
    from karman_taichi_gb300.channel import ChannelSolver
    if mode == "learned":
        from karman_taichi_gb300 import learned
        return learned.make_channel_solver(cfg, dev)
    if mode == "fp64":
        return ChannelSolver(cfg, device=dev, precision="fp64")
    return ChannelSolver(cfg, device=dev, precision="mixed", momentum=momentum)


def resolve_mode(mode, config="channel_2048x512"):
    """auto: the fastest accelerated configuration measured on GB300 -- mixed
    precision + multigrid CG (native step).  The learned initial guess is timed
    beside it (out["learned"]): with the exact-coarse multigrid the p' solve
    needs ~30 CG iterations and the guess (~10% error) saves less than its
    inference costs."""
    if mode != "auto":
        return mode
    return "mixed"


def summarize(recs_per_step):
    outer = [sum(s.get("outer", 1) for s in r) for r in recs_per_step]
    its = [sum(s["it_u"] + s["it_v"] + s["it_p"] for s in r) for r in recs_per_step]
    itp = [sum(s["it_p"] for s in r) for r in recs_per_step]
    mass = [r[-1]["mass"] for r in recs_per_step]
    return dict(outer_per_step=statistics.mean(outer), solver_iters_per_step=statistics.mean(its),
                p_iters_per_step=statistics.mean(itp), mass_residual_last=mass,
                mass_residual_max=max(mass), steps_converged=sum(1 for m in mass if m <= 1e-6))


def timed_steps(solver, K, W, world, lib, clocks=None):
    import torch
    for _ in range(W):
        solver.step()
    torch.cuda.synchronize()
    barrier(world)
    l0 = lib.kc_launch_count()
    if clocks:
        clocks.start()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(K + 1)]
    ev[0].record()
    recs = []
    for k in range(K):
        recs.append(solver.step())
        ev[k + 1].record()
    torch.cuda.synchronize()
    ck = clocks.stop() if clocks else None
    barrier(world)
    ms = max_over_ranks(ev[0].elapsed_time(ev[K]), world)
    per_step = [ev[k].elapsed_time(ev[k + 1]) for k in range(K)]
    return ms, recs, lib.kc_launch_count() - l0, ck, per_step


def e2e_steps(solver, K, W, world):
    """The same time steps as the device-timed run (reset, W untimed warm-up
    steps, K timed) through the public API with host-resident fields: every
    timed step copies u, v, p, u0, v0 from pinned host memory and reads u, v,
    p back."""
    import torch
    solver.reset()
    for _ in range(W):
        solver.step()
    names_in = ("u", "v", "p", "u0", "v0")
    names_out = ("u", "v", "p")
    host = {k: torch.empty(getattr(solver, k).shape, dtype=torch.float64, pin_memory=True) for k in names_in}
    for k in names_in:
        host[k].copy_(getattr(solver, k))
    torch.cuda.synchronize()
    barrier(world)
    h2d = sum(host[k].numel() * 8 for k in names_in)
    d2h = sum(host[k].numel() * 8 for k in names_out)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(K):
        for k in names_in:
            getattr(solver, k).copy_(host[k], non_blocking=True)
        solver.step()
        for k in names_out:
            host[k].copy_(getattr(solver, k), non_blocking=True)
        torch.cuda.current_stream().synchronize()
        host["u0"].copy_(host["u"])
        host["v0"].copy_(host["v"])
    e1.record()
    torch.cuda.synchronize()
    ms = max_over_ranks(e0.elapsed_time(e1), world)
    return ms, h2d, d2h


# Algorithmic bytes per fine cell of one iteration of the single-reduction
# multigrid-preconditioned CG (FP32 vectors and coefficients, FP64 iterate),
# each array read or written once per kernel:
#   k_pcc_down0  s = w + beta s, r = r - alpha s, p = z + beta p, x += alpha p
#                (FP64), pre-smooth, restrict: read r, w, s, W, 5 coef, z, p,
#                x(8); write s, r, p, x(8), x_pre, b_1/4                         77
#   k_pcc_up0    prolong + post-smooth, w = A z, (r, z), (w, z): read x_pre,
#                x_1/4, r, W, 5 coef; write z, w                                 41
#   levels >= 1  DOWN 33 + UP 37 bytes per coarse cell, n/3 coarse cells         23
PCG_MG_BYTES_PER_CELL = 77 + 41 + 23


def roofline_p_solve(solver, mode, peak):
    """Roofline of the dominant unit of work, the pressure-correction solve.

    fp64: one persistent BiCGSTAB launch, 27 words/cell/iteration.
    mixed: the multigrid-preconditioned CG, PCG_MG_BYTES_PER_CELL
    bytes/cell/iteration over its 2L launches per iteration (L multigrid
    levels); each FP64 refinement residual adds (5 coef + x + b) x 8 B/cell."""
    import torch
    solver.outer_iteration()   # one untimed outer iteration through the same Python-driven stages first
    solver.assemble_momentum()
    solver.solve_momentum()
    solver.relax()
    solver.assemble_p()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    info = solver.solve_p()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    n = solver.A_p.n
    if mode == "fp64":
        alg = 27 * 8 * n * info.iters
        kernel = "k_bicg_persist<double>"
        note = "27 words/cell/iteration (A 9R+2W, B 7R+1W, C 6R+2W)"
    else:
        alg = PCG_MG_BYTES_PER_CELL * n * info.iters + (info.refinements + 1) * 7 * 8 * n
        kernel = "kc_pcg_refined"
        note = (f"{PCG_MG_BYTES_PER_CELL} B/cell/CG iteration (k_pcc_down0 77, k_pcc_up0 41, "
                f"levels>=1 23) + 56 B/cell per FP64 refinement residual")
    achieved = alg / (ms * 1e-3) / 1e9
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            t = json.load(f).get(kernel)
            if t:   # bytes per iteration per cell from an ncu capture, scaled to this launch
                traffic = t["dram_bytes_per_cell_iter"] * n * info.iters
    except (OSError, ValueError):
        pass
    return {"bound": "hbm", "kernel": kernel, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic,
            "algorithmic_bytes": alg, "iters": info.iters, "ms": round(ms, 3),
            "note": note + "; peak = hbm_gbs of MEASURED_PEAKS.json (burst)"}


def spmv_roofline(solver, peak):
    """SpMV (k_spmv) on the workload's assembled pressure-correction system,
    FP64 and FP32, each launch timed with CUDA events after writing a
    256 MB buffer (larger than L2); 7 words/cell algorithmic."""
    import torch
    from karman_taichi_gb300 import linalg
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=solver.device)
    out = {}
    systems = [("f64", solver.A_p, torch.float64, 8)]
    if getattr(solver, "A_p32", None) is not None:
        systems.append(("f32", linalg.Stencil(solver.coef_p32), torch.float32, 4))
    for name, A, dt, w in systems:
        x = torch.rand(A.n, dtype=dt, device=solver.device)
        y = torch.empty_like(x)
        for _ in range(3):
            linalg.spmv(A, x, y)
        ts = []
        for _ in range(10):
            flush.add_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            linalg.spmv(A, x, y)
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        t = sorted(ts)[len(ts) // 2]
        gbs = 7 * w * A.n / (t * 1e-3) / 1e9
        out[name] = {"cells": A.n, "us": round(t * 1e3, 2), "achieved_gbs": round(gbs, 1),
                     "frac": round(gbs / peak, 4)}
        # back to back, as inside a solver: 16 launches in one CUDA graph cycling over four copies of
        # the system and its vectors (4 x 7 words x cells > L2, so every launch reads HBM)
        coefs = [A.coef.clone() for _ in range(4)]
        As = [linalg.Stencil(c, stride=A.stride, form=A.form) for c in coefs]
        xs = [torch.rand(A.n, dtype=dt, device=solver.device) for _ in range(4)]
        ys = [torch.empty_like(v) for v in xs]
        side = torch.cuda.Stream(device=solver.device)
        side.wait_stream(torch.cuda.current_stream(solver.device))
        with torch.cuda.stream(side):
            for q in range(4):
                linalg.spmv(As[q], xs[q], ys[q])
        torch.cuda.current_stream(solver.device).wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            for r in range(16):
                q = r % 4
                linalg.spmv(As[q], xs[q], ys[q])
        tg = []
        for _ in range(5):
            flush.add_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            graph.replay()
            e1.record()
            torch.cuda.synchronize()
            tg.append(e0.elapsed_time(e1) / 16)
        tb = sorted(tg)[len(tg) // 2]
        gb2 = 7 * w * A.n / (tb * 1e-3) / 1e9
        out[name]["back_to_back"] = {"us": round(tb * 1e3, 2), "achieved_gbs": round(gb2, 1),
                                     "frac": round(gb2 / peak, 4),
                                     "note": "16 launches in a CUDA graph over four copies of the system (> L2)"}
        del graph, coefs, As, xs, ys
    return out


def field_writer_roofline(solver, peak):
    """post_process_field (kc_post_process: cell-centre velocities, udiv, the
    five display canvases) on the final state, timed with CUDA events after an
    L2 flush.  Algorithmic bytes: u, v, p, pcor, udiv read and u_post, v_post,
    udiv written (FP64) by the first kernel, the five fields read again (FP64)
    and the canvases written (9 FP32 pixels per cell) by the second."""
    import torch
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=solver.device)
    solver.post_process()
    ts = []
    for _ in range(5):
        flush.add_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        solver.post_process()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    t = sorted(ts)[len(ts) // 2]
    n = solver.p.numel()
    alg = 8 * (solver.u.numel() + solver.v.numel() + 3 * n) + 8 * 3 * n + 8 * 5 * n + 4 * 5 * 9 * n
    gbs = alg / (t * 1e-3) / 1e9
    return {"kernels": "k_post_cells + k_post_disp", "us": round(t * 1e3, 1), "algorithmic_bytes": alg,
            "achieved_gbs": round(gbs, 1), "frac": round(gbs / peak, 4)}


def cpu_whole_steps(cfg, budget_s, steps=None):
    """C/OpenMP FP64 plain path on all host cores: whole time steps of the
    seeded case from its initial state (every solve to its tolerance, outer
    loop to its stop rule), as many as fit ``budget_s`` (at least one), or
    exactly ``steps``.  Returns the time-steps/s figure and what was timed."""
    from karman_taichi_gb300 import geometry
    from oracle import cpu
    solid = geometry.solid_mask(cfg.nx, cfg.ny, cfg.obstacles)
    u, v, p = geometry.channel_initial_fields(cfg.nx, cfg.ny, solid, cfg.U, cfg.noise, cfg.seed)
    u0, v0 = u.copy(), v.copy()
    # the library is loaded and its threads started before anything is timed
    cpu.channel_run(cfg, solid, u.copy(), v.copy(), p.copy(), n_steps=1, max_total_outer=1, max_solver_iter=2)
    done, secs, outer, its, first_ms, first_outer = 0, 0.0, 0, 0, None, None
    while True:
        st = cpu.channel_run(cfg, solid, u, v, p, u0, v0, n_steps=1)
        done += 1
        secs += st["seconds"]
        outer += st["outer"]
        its += st["solver_iters"]
        if first_ms is None:
            first_ms, first_outer = st["seconds"] * 1e3, st["outer"]
        if steps is not None:
            if done >= steps:
                break
        elif secs + st["seconds"] > budget_s:
            break
    return {"value": done / secs, "unit": "time steps/s", "cores": cpu.threads(), "kind": "port",
            "steps_timed": done, "seconds": secs, "outer_iterations": outer,
            "bicgstab_iterations": its, "first_step_ms": first_ms, "first_step_outer": first_outer,
            "sample": f"time steps 1..{done} of {cfg.name} from the seeded initial state, whole steps "
                      f"(BiCGSTAB solves to rel. tol {cfg.eps}, outer loop to max|mdiv| <= {cfg.mass_tol} "
                      f"or {cfg.max_outer} iterations), {cpu.threads()} OpenMP threads"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------------------------
def run_gpu(args):
    import torch
    from karman_taichi_gb300 import _lib as L
    from karman_taichi_gb300.config import PRESETS
    rank, world, local = dist_init(args)
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    lib = L.load()
    cfg = PRESETS[args.config]
    mode = resolve_mode(args.mode, args.config)
    peak, peak_kind = peaks()
    out = {"metric": METRIC, "unit": "time steps/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None}

    solver = make_solver(cfg, mode, dev, args.momentum)
    tuned = None
    if mode == "mixed" and not args.no_autotune:
        # the p' solve's cycle (sweeps below level 0) and launch shapes (multigrid tail, tile sizes,
        # CG chunk length), picked on this solver's state before anything is timed
        from karman_taichi_gb300.autotune import CYCLE_CANDIDATES, tune_pressure
        tuned = tune_pressure(solver, cycles=CYCLE_CANDIDATES)
    ms, recs, launches, ck, per_step = timed_steps(solver, args.steps, args.warmup, world, lib, Clocks(local))
    summ = summarize(recs)
    value = replica_value(world, args.steps, ms)
    out.update(value=round(value, 5), ms_per_step=round(ms / args.steps, 3),
               dtype="f64" if mode == "fp64" else ("f32+f64 (FP32 stencils/vectors, FP64 dots/residuals)"
                                                   + (" + bf16 U-Net initial guess" if mode == "learned" else "")),
               data="synthetic: seeded channel initial state (u=1, v = U(-1e-3,1e-3) noise, p=0)",
               config={"workload": cfg.name, "nx": cfg.nx, "ny": cfg.ny, "cells": cfg.cells, "Re": cfg.Re,
                       "mode": mode, "mass_tol": cfg.mass_tol, "max_outer": cfg.max_outer, "eps": cfg.eps,
                       "parallelism": f"replicas x{world}",
                       "l2": "working set per step > 129 MB L2 (no flush needed)"},
               gpu_launches=launches, clocks=ck)
    if tuned is not None:
        out["config"]["autotune"] = {k: tuned[k] for k in ("nu_coarse", "omega_coarse", "tail", "big_cells",
                                                           "check_every_p", "ms")}
    out["cell_updates_per_s"] = round(value * cfg.cells, 1)
    out["stats"] = summ

    if rank == 0 and not args.no_e2e:
        e2e_ms, h2d, d2h = e2e_steps(solver, args.steps, args.warmup, 1)
        out["e2e"] = {"value": round(args.steps / (e2e_ms * 1e-3), 5), "unit": "time steps/s",
                      "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                      "note": "the same K time steps (after reset + W warm-up) through the public "
                              "ChannelSolver.step() with u, v, p, u0, v0 copied from pinned host memory and "
                              "u, v, p read back every step"}
    if rank == 0:
        out["roofline"] = roofline_p_solve(solver, mode, peak)
        out["roofline"]["peak_kind"] = peak_kind
        out["spmv"] = spmv_roofline(solver, peak)
        out["field_writer"] = field_writer_roofline(solver, peak)

    if rank == 0 and mode == "mixed" and not args.no_compare:
        try:
            from karman_taichi_gb300 import learned
            have = learned.available(cfg.name)
        except ImportError:
            have = False
        if have:
            lsol = make_solver(cfg, "learned", dev)
            if tuned is not None:   # the same p' cycle and launch shapes as the timed run
                from karman_taichi_gb300.autotune import apply_choice
                apply_choice(lsol, tuned)
            lms, lrecs, _, _, _ = timed_steps(lsol, args.steps, args.warmup, 1, lib)
            lsum = summarize(lrecs)
            out["learned"] = {"value": round(args.steps / (lms * 1e-3), 5), "unit": "time steps/s",
                              "ms_per_step": round(lms / args.steps, 3), "p_iters_per_step": lsum["p_iters_per_step"],
                              "outer_per_step": lsum["outer_per_step"], "mass_residual_max": lsum["mass_residual_max"],
                              "network_applied": lsol.learned_stats[0], "network_rejected": lsol.learned_stats[1],
                              "fallbacks": lsol.fallbacks,
                              "window": f"time steps {args.warmup + 1}..{args.warmup + args.steps}, as value",
                              "note": "same steps, native step; every p' solve a flexible CG whose first "
                                      "preconditioner application is the U-Net's prediction, then multigrid CG "
                                      "passes (kc_pcg_flexible); p_iters_per_step counts the inner CG iterations"}
            del lsol

    if rank == 0 and not args.no_compare and mode != "fp64":
        # plain FP64 BiCGSTAB on the same GPU over time steps W+1 .. W+C of the same seeded case; the
        # accelerated path's time for the same steps comes from the per-step events of the timed run
        C = min(args.compare_steps, args.steps)
        ref = make_solver(cfg, "fp64", dev)
        cms, crecs, _, _, _ = timed_steps(ref, C, args.warmup, 1, lib)
        same = sum(per_step[:C])
        out["fp64_plain"] = {"value": round(C / (cms * 1e-3), 5), "unit": "time steps/s",
                             "ms_per_step": round(cms / C, 3), "steps": C, "warmup": args.warmup,
                             "window": f"time steps {args.warmup + 1}..{args.warmup + C}",
                             "stats": summarize(crecs),
                             "accelerated_same_steps": {"value": round(C / (same * 1e-3), 5),
                                                        "ms_per_step": round(same / C, 3),
                                                        "stats": summarize(recs[:C])}}
        out["speedup_vs_fp64_plain"] = round(cms / same, 3)
        out["speedup_vs_fp64_plain_window"] = f"time steps {args.warmup + 1}..{args.warmup + C}, both paths"
        # field error after the same W + C steps from the same initial state
        solver.reset()
        for _ in range(args.warmup + C):
            solver.step()
        a, b = solver.state_numpy(), ref.state_numpy()
        out["field_error_vs_fp64"] = {k: float(abs(a[k] - b[k]).max() / max(abs(b[k]).max(), 1e-300))
                                      for k in ("u", "v", "p")}
        out["field_error_vs_fp64"]["after_steps"] = args.warmup + C
        out["field_error_vs_fp64"]["definition"] = ("max |x - x_fp64| / max |x_fp64| over the padded field; "
                                                    "x_fp64: the GPU plain FP64 path (the oracle's algorithm)")
        del ref
    if rank == 0 and world == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_whole_steps(cfg, args.cpu_budget)
        # the GPU's time for the same time step (step 1 from the seeded state, kernels warm)
        solver.reset()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        r1 = solver.step()
        e1.record()
        torch.cuda.synchronize()
        g1 = e0.elapsed_time(e1)
        cb = out["cpu_baseline"]
        out["first_step"] = {"gpu_ms": round(g1, 3), "gpu_outer": sum(s.get("outer", 1) for s in r1),
                             "cpu_ms": round(cb["first_step_ms"], 1), "cpu_outer": cb["first_step_outer"],
                             "gpu_vs_cpu": round(cb["first_step_ms"] / g1, 1),
                             "note": "time step 1 of the seeded case on both: the same work, timed on both sides"}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_reference(args):
    """The reference arm: the plain method's CPU implementation (C + OpenMP
    restatement; the reference's Taichi CPU path needs taichi==0.9.0, which is
    not installed), on all host cores, same config/metric/unit.  Whole time
    steps from the seeded initial state, as many as fit a budget of about two
    minutes (at least one); "steps" is the number actually timed."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from karman_taichi_gb300.config import PRESETS
    cfg = PRESETS[args.config]
    cb = cpu_whole_steps(cfg, budget_s=120.0)
    value = cb["value"]
    out = {"metric": METRIC, "value": value, "unit": "time steps/s", "impl": "reference", "n_gpus": 0,
           "steps": cb["steps_timed"], "warmup": 0, "steps_requested": args.steps, "warmup_requested": args.warmup,
           "ms_per_step": 1e3 / value, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic: seeded channel initial state",
           "config": {"workload": cfg.name, "nx": cfg.nx, "ny": cfg.ny, "cells": cfg.cells, "mode": "fp64 plain",
                      "timed": "whole time steps from the seeded initial state; a step is about a minute of CPU "
                               "work, so fewer steps than requested are timed and no warm-up step is run"},
           "cpu_baseline": {"value": value, "unit": "time steps/s", "cores": cb["cores"], "kind": "port",
                            "sample": cb["sample"], "seconds": cb["seconds"],
                            "outer_iterations": cb["outer_iterations"],
                            "bicgstab_iterations": cb["bicgstab_iterations"]},
           "e2e": {"value": value, "unit": "time steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_spmv_sweep(args):
    """k_spmv bandwidth against system size: random coefficients and operand,
    each launch timed with CUDA events after writing a 256 MB buffer; 7
    words/cell algorithmic."""
    import torch
    from karman_taichi_gb300 import linalg
    peak, kind = peaks()
    dev = torch.device("cuda", 0)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    rows = []
    for NX, NY in ((2050, 514), (4098, 1026), (8194, 2050)):
        for dt, w in ((torch.float64, 8), (torch.float32, 4)):
            g = torch.Generator(device=dev).manual_seed(0)
            A = linalg.Stencil(torch.rand((5, NX, NY), dtype=dt, device=dev, generator=g))
            x = torch.rand((NX, NY), dtype=dt, device=dev, generator=g)
            y = torch.empty_like(x)
            for _ in range(3):
                linalg.spmv(A, x, y)
            ts = []
            for _ in range(20):
                flush.add_(1)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                linalg.spmv(A, x, y)
                e1.record()
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1))
            t = sorted(ts)[len(ts) // 2]
            gbs = 7 * w * NX * NY / (t * 1e-3) / 1e9
            rows.append({"grid": f"{NX}x{NY}", "dtype": "f64" if w == 8 else "f32", "us": round(t * 1e3, 2),
                         "achieved_gbs": round(gbs, 1), "frac": round(gbs / peak, 4), "peak_kind": kind})
    print(json.dumps({"spmv_sweep": rows}), flush=True)


def run_pcorr1024(args):
    """The isolated 1024 x 1024 p' solve: plain FP64 BiCGSTAB (the reference
    method, persistent launch) and the FP32 multigrid-preconditioned CG in FP64
    refinement (kc_pcg_refined), both to ||r||/||b|| < 1e-8 from x = 0.  Each
    solve is timed with CUDA events after one untimed solve of the same
    system (graphs instantiated, multigrid set up); the multigrid setup is
    timed separately.  Error: max |x - x_fp64| / max |x_fp64|."""
    import torch
    from karman_taichi_gb300 import _lib as L, linalg
    from karman_taichi_gb300.workloads import pcorr_random_system
    peak, kind = peaks()
    dev = torch.device("cuda", 0)
    c, b = pcorr_random_system(1024, seed=0)
    n = c[0].size
    c64 = torch.from_numpy(c).to(dev)
    lap = c64.clone()
    lap[0] = c64[0] + (((c64[1] + c64[2]) + c64[3]) + c64[4])
    A64 = linalg.Stencil(c64)
    A32 = linalg.Stencil(lap.float().contiguous(), form=L.FORM_LAPLACIAN)
    bt = torch.from_numpy(b).to(dev)
    ev = lambda: torch.cuda.Event(enable_timing=True)
    out = {"metric": "isolated p' solve, 1024 x 1024, rel. tol 1e-8", "config": {"workload": "pcorr_random_1024",
           "cells": int(n), "blocked": 0.05, "aP_face": "log-uniform [1, 10]"}, "peak_gbs": peak, "peak_kind": kind}
    # plain FP64 BiCGSTAB
    ws = linalg.Workspace(dev)
    x64 = torch.zeros_like(bt)
    linalg.bicgstab(A64, bt, x64, eps=1e-8, max_iter=n, ws=ws)
    x64.zero_()
    torch.cuda.synchronize()
    e0, e1 = ev(), ev()
    e0.record()
    i64 = linalg.bicgstab(A64, bt, x64, eps=1e-8, max_iter=n, ws=ws)
    e1.record()
    torch.cuda.synchronize()
    t64 = e0.elapsed_time(e1)
    alg64 = 27 * 8 * n * i64.iters
    out["fp64_bicgstab"] = {"status": i64.status_name, "iters": i64.iters, "ms": round(t64, 3),
                            "ms_per_iter": round(t64 / max(i64.iters, 1), 4),
                            "achieved_gbs": round(alg64 / (t64 * 1e-3) / 1e9, 1),
                            "frac": round(alg64 / (t64 * 1e-3) / 1e9 / peak, 4),
                            "bytes_note": "27 words (8 B) per cell per iteration"}
    # FP32 multigrid CG in FP64 refinement
    mg = linalg.Multigrid(A32)
    torch.cuda.synchronize()
    e0.record()
    mg.setup()
    e1.record()
    torch.cuda.synchronize()
    tsetup = e0.elapsed_time(e1)
    wsp = linalg.Workspace(dev)
    x32 = torch.zeros_like(bt)
    linalg.pcg_refined(A64, A32, bt, x32, mg, eps=1e-8, ws=wsp)
    x32.zero_()
    torch.cuda.synchronize()
    e0.record()
    im = linalg.pcg_refined(A64, A32, bt, x32, mg, eps=1e-8, ws=wsp)
    e1.record()
    torch.cuda.synchronize()
    tm = e0.elapsed_time(e1)
    algm = PCG_MG_BYTES_PER_CELL * n * im.iters + (im.refinements + 1) * 7 * 8 * n
    out["mixed_mg_cg"] = {"status": im.status_name, "iters": im.iters, "refinements": im.refinements,
                          "ms": round(tm, 3), "ms_per_iter": round(tm / max(im.iters, 1), 4),
                          "setup_ms": round(tsetup, 3),
                          "achieved_gbs": round(algm / (tm * 1e-3) / 1e9, 1),
                          "frac": round(algm / (tm * 1e-3) / 1e9 / peak, 4),
                          "bytes_note": f"{PCG_MG_BYTES_PER_CELL} B per cell per CG iteration + 56 B per cell per "
                                        "FP64 refinement residual"}
    res = lambda x: float((bt - linalg.spmv(A64, x)).norm() / bt.norm())
    out["rel_residual"] = {"fp64_bicgstab": res(x64), "mixed_mg_cg": res(x32)}
    out["error_vs_fp64"] = float((x32 - x64).abs().max() / x64.abs().max())
    out["speedup_mixed_vs_fp64"] = round(t64 / tm, 2)
    print(json.dumps(out), flush=True)


def run_batch(args, cfgs=None, workload=None):
    """Instance time steps/s of the batched configuration: N instances (sizes
    128x32 .. 640x128, D 4-16, Re 60-200).  Executors (--batch-executors):
    ``fused``, every instance and every timed step in ONE persistent launch
    (kc_channel_batch_fused: each large instance on a block of its own, the others four to a block); ``native``, one CUDA stream
    per instance driven by native threads (kc_channel_batch_step);
    ``sequential``, the instances one after another on one stream.  Each
    executor starts from the seeded initial state: W warm-up steps, then K
    timed steps of every instance.  With ``cfgs`` (``--copies``): those
    instances instead, e.g. seeded copies of one preset (native and
    sequential only)."""
    import numpy as np
    import torch
    from karman_taichi_gb300.batch import BatchedChannels, batch_configs
    mode = "fp64" if args.mode == "fp64" else "mixed"
    if cfgs is None:
        cfgs = batch_configs(args.batch_instances, seed=0)
        workload = f"{len(cfgs)} channel instances, 128x32 .. 640x128"
    out = {"metric": "instance time steps/s, batched channel instances", "unit": "instance time steps/s",
           "config": {"workload": workload}, "instances": len(cfgs), "cells": int(sum(c.cells for c in cfgs)),
           "mode": mode, "steps": args.steps, "warmup": args.warmup}
    execs = [e.strip() for e in args.batch_executors.split(",") if e.strip()]
    if args.copies:
        execs = [e for e in execs if e != "fused"] or ["native"]
    plan = {"fused": ("fused", 1), "native": ("native_concurrent", args.batch_workers),
            "sequential": ("sequential", 1)}
    first = None
    for e in execs:
        key, workers = plan[e]
        b = BatchedChannels(cfgs, precision=mode, workers=workers)
        if mode == "mixed" and not args.no_autotune:   # per grid size, before anything is timed
            from karman_taichi_gb300.autotune import CYCLE_CANDIDATES
            chosen = b.autotune(cycles=CYCLE_CANDIDATES)
            out.setdefault("autotune", {k: {f: c[f] for f in ("nu_coarse", "tail", "big_cells", "check_every_p")}
                                        for k, c in chosen.items()})
        if e == "fused":
            from karman_taichi_gb300 import _lib as L
            lib = L.load()
            run = b.step_fused
            run(args.warmup)
            l0 = lib.kc_launch_count()
            t = run(args.steps)
            launches = lib.kc_launch_count() - l0
            tot = b.fused_totals
            outer = float(np.mean([x["outer"] for x in tot])) / max(1, args.steps)
            out[key] = {"driver": "one persistent launch (kc_channel_batch_fused): instances of >= 40k p cells on a 1024-thread block each, the others on 256 threads four to a block",
                        "seconds": round(t, 3), "value": round(len(cfgs) * args.steps / t, 2),
                        "cell_updates_per_s": round(out["cells"] * args.steps / t, 1),
                        "outer_per_step": round(outer, 2), "gpu_launches": int(launches),
                        "it_p_per_step": round(float(np.mean([x["it_p"] for x in tot])) / max(1, args.steps), 1),
                        "mass_residual_max": max(x["mass_max"] for x in tot),
                        "fallbacks": int(sum(x["fallbacks"] for x in tot)),
                        "instances_with_an_unconverged_solve": int(sum(x["status"] not in (0, 4) for x in tot)),
                        "instances_not_finite": int(sum(x["status"] == 4 for x in tot))}
        else:
            run = b.step_native
            run(args.warmup)
            t = run(args.steps)
            # the native driver records one entry per call (its last step's statistics): the timed call's
            outer = np.mean([sum(s.get("outer", 1) for s in rec[-1]) for rec in b.records])
            out[key] = {"workers": workers, "driver": "native threads", "seconds": round(t, 3),
                        "value": round(len(cfgs) * args.steps / t, 2),
                        "cell_updates_per_s": round(out["cells"] * args.steps / t, 1),
                        "outer_per_step_last": round(float(outer), 2)}
        first = first or key
        b.close()
        del b
        torch.cuda.empty_cache()
    out["value"] = out[first]["value"]
    keys = [plan[e][0] for e in execs]
    for a in keys[1:]:
        out[f"speedup_{first}_vs_{a}"] = round(out[first]["value"] / out[a]["value"], 2)
    print(json.dumps(out), flush=True)


def shedding(sig, dt, min_amp=1e-3, frac=0.6):
    """Shedding period of one wake probe (v behind a cylinder, one sample per
    time step).  Over the last ``frac`` of the run the signal less a quadratic
    fit is taken; where its half peak-to-peak amplitude exceeds ``min_amp`` (in
    units of the inlet velocity) the period is twice the mean spacing of its
    zero crossings (interpolated), and with five crossings or more the drift is
    the relative change of that period between the first and the second half
    of the crossings."""
    import numpy as np
    x = np.asarray(sig, dtype=np.float64)
    n = len(x)
    lo = int(n * (1 - frac))
    t = np.arange(lo, n, dtype=np.float64)
    d = x[lo:] - np.polyval(np.polyfit(t, x[lo:], 2), t)
    amp = float(np.ptp(d) / 2)
    out = {"window": [lo, n], "amplitude": round(amp, 6)}
    if amp < min_amp:
        out.update(period_steps=None, note="no oscillation above the threshold")
        return out
    k = np.nonzero(np.signbit(d[1:]) != np.signbit(d[:-1]))[0]
    tz = lo + k + d[k] / (d[k] - d[k + 1])
    out["crossings"] = int(len(tz))
    if len(tz) < 2:
        out.update(period_steps=None, note="fewer than two crossings: the period is longer than the window")
        return out
    half = np.diff(tz)
    per = 2.0 * float(np.mean(half))
    out.update(period_steps=round(per, 2), period_time=per * dt)
    if len(tz) >= 5:
        m = len(half) // 2
        p_a, p_b = 2.0 * float(np.mean(half[:m])), 2.0 * float(np.mean(half[m:]))
        out.update(period_first_half=round(p_a, 2), period_second_half=round(p_b, 2), drift=round((p_b - p_a) / p_a, 4))
    else:
        out.update(drift=None, note="fewer than five crossings: drift not measurable")
    return out


def run_long(args):
    """The long run: the preset's seeded copies (inlet noise seed k for copy k)
    advanced together by the batch executor, mixed path, autotuned, for N time
    steps; after every step v is sampled four diameters behind each cylinder on
    its axis (device-side gather, read once at the end).  Reports instance time
    steps/s, the mass residual reached, the shedding period per copy and probe
    and its drift, the spread of the period over the copies, and the field error
    of copy 0 against the plain FP64 method after its first --fp64-steps steps."""
    import numpy as np
    import torch
    from karman_taichi_gb300.batch import BatchedChannels
    from karman_taichi_gb300.channel import ChannelSolver
    from karman_taichi_gb300.config import PRESETS
    from karman_taichi_gb300.autotune import CYCLE_CANDIDATES
    name = args.config if args.config != "channel_2048x512" else "channel_4096x1024"
    base = PRESETS[name]
    copies = max(1, base.copies)
    cfgs = [base.with_(seed=k) for k in range(copies)]
    N = args.long_run
    dev = torch.device("cuda", 0)
    b = BatchedChannels(cfgs, precision="mixed", workers=copies)
    chosen = b.autotune(cycles=CYCLE_CANDIDATES)
    for s in b.solvers:
        s.reset()
    probes = [(ci + 4 * D, cj) for (_, ci, cj, D) in base.obstacles]
    idx = torch.tensor([i * (base.ny + 3) + j for (i, j) in probes], dtype=torch.long, device=dev)
    samples = torch.zeros(N, copies, len(probes), dtype=torch.float64, device=dev)
    snap = None
    mass_max, outer, status_bad = 0.0, [], 0
    t_total = 0.0
    clocks = Clocks(0)
    clocks.start()
    for t in range(N):
        t_total += b.step_native(1)
        for k, s in enumerate(b.solvers):
            samples[t, k] = s.v.reshape(-1).index_select(0, idx)
            rec = b.records[k][-1][0]
            mass_max = max(mass_max, rec["mass"])
            outer.append(rec["outer"])
            status_bad += rec["status"] != 0
        if t + 1 == args.fp64_steps:
            snap = {f: getattr(b.solvers[0], f).clone() for f in ("u", "v", "p")}
        for rec in b.records:   # keep only the last record per instance
            del rec[:-1]
    ck = clocks.stop()
    sig = samples.cpu().numpy()
    dt = base.dt
    shed = [[shedding(sig[:, k, q], dt) for q in range(len(probes))] for k in range(copies)]
    pers = [x["period_steps"] for row in shed for x in row if x.get("period_steps")]
    out = {"metric": "instance time steps/s, long run", "unit": "instance time steps/s",
           "config": {"workload": f"{name} x {copies} seeded copies", "nx": base.nx, "ny": base.ny,
                      "Re": base.Re, "obstacles": [list(o) for o in base.obstacles], "dt": dt, "steps": N,
                      "mode": "mixed", "autotune": {k: {f: c[f] for f in ("nu_coarse", "tail", "big_cells",
                                                                           "check_every_p")}
                                                    for k, c in chosen.items()}},
           "value": round(copies * N / t_total, 3), "seconds": round(t_total, 1),
           "cell_updates_per_s": round(copies * base.cells * N / t_total, 1),
           "outer_per_step": round(float(np.mean(outer)), 2), "mass_residual_max": mass_max,
           "steps_not_converged": int(status_bad), "clocks": ck,
           "probes": {"points": [list(p) for p in probes], "field": "v", "per_copy": shed},
           "period_spread_over_copies": (round((max(pers) - min(pers)) / float(np.mean(pers)), 4)
                                         if len(pers) >= 2 else None),
           "probe_history_copy0_every_10_steps": np.round(sig[::10, 0, :], 7).tolist()}
    b.close()
    del b
    torch.cuda.empty_cache()
    if args.fp64_steps > 0 and snap is not None:
        ref = ChannelSolver(cfgs[0], device=dev, precision="fp64")
        ref.reset()
        t0 = time.perf_counter()
        for _ in range(args.fp64_steps):
            ref.step()
        torch.cuda.synchronize()
        err = {f: float((snap[f] - getattr(ref, f)).abs().max() / getattr(ref, f).abs().max())
               for f in ("u", "v", "p")}
        out["field_error_vs_fp64"] = dict(err, after_steps=args.fp64_steps, fp64_seconds=round(time.perf_counter() - t0, 1),
                                          definition="max |x - x_fp64| / max |x_fp64| over the padded field, copy 0")
    print(json.dumps(out), flush=True)


def run_profile_outer(args):
    import torch
    from karman_taichi_gb300.config import PRESETS
    cfg = PRESETS[args.config]
    solver = make_solver(cfg, resolve_mode(args.mode, cfg.name), torch.device("cuda", 0))
    for _ in range(args.profile_outer):
        rec = solver.outer_iteration()
    torch.cuda.synchronize()
    print(json.dumps({"config": cfg.name, "outer_iterations": args.profile_outer, "last": rec}), flush=True)


if __name__ == "__main__":
    a = parse()
    if a.no_device_loop:
        from karman_taichi_gb300 import _lib as _L
        _L.load().kc_device_loop(0)
    if a.impl == "reference":
        run_reference(a)
    elif a.profile_outer > 0:
        run_profile_outer(a)
    elif a.long_run > 0:
        run_long(a)
    elif a.spmv_sweep:
        run_spmv_sweep(a)
    elif a.pcorr1024:
        run_pcorr1024(a)
    elif a.copies > 0:
        from karman_taichi_gb300.config import PRESETS
        base = PRESETS[a.config]
        run_batch(a, [base.with_(seed=k) for k in range(a.copies)], f"{base.name} x {a.copies} seeded copies")
    elif a.batch_instances > 0:
        run_batch(a)
    else:
        run_gpu(a)
