"""Many independent channel instances on one GPU (the batched configuration).

Each instance is a full :class:`ChannelSolver` (its own fields, systems and
workspaces) bound to its own CUDA stream.  A pool of host threads drives the
instances -- worker w steps instances w, w + W, w + 2W, ... -- and every
library call enqueues on the calling thread's current stream, so kernels of
different instances run concurrently: an instance of 4k-82k cells fills a
few SMs, a batch fills the 152.  Solves run as graph-captured iteration
chunks, not single cooperative launches: a cooperative launch does not
overlap with the other streams' work (7.2x vs 3.8x over one stream, 64
instances).  Small device-to-host readbacks go through per-thread pinned
buffers, which keeps the driver from serialising the workers.  The C library is safe for this use: error
messages are thread-local, the captured-graph cache is guarded, captures run
in thread-local mode on private streams, and the launch counter is atomic.
The ctypes calls and stream synchronisations release the Python GIL.

An instance run in a batch computes bit for bit what it computes alone (the
kernels and reductions are deterministic and instances share no buffers).
The reference has no batched mode; instances are independent, so there is no
exchange between them ("replicas" at the scale of one GPU).
"""
from __future__ import annotations

import threading
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import torch

from .channel import ChannelSolver
from .config import ChannelConfig

SIZES = ((128, 32), (256, 64), (320, 64), (512, 128), (640, 128))


def batch_configs(n=256, seed=0, n_steps=50):
    """The batched configuration: n channel instances, sizes from SIZES, obstacle
    diameter D in [4, 16] cells, centre x in [0.15, 0.3] of the length, y within
    +-10% of the centre line, Re ~ U[60, 200], per-instance noise seed; dx = dy =
    1/ny (unit channel height)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        nx, ny = SIZES[int(rng.integers(len(SIZES)))]
        D = int(rng.integers(4, 17))
        ci = int(round(nx * rng.uniform(0.15, 0.3)))
        cj = int(round(ny * (0.5 + rng.uniform(-0.1, 0.1))))
        Re = float(rng.uniform(60.0, 200.0))
        out.append(ChannelConfig(f"batch{k:03d}_{nx}x{ny}", nx, ny, 1.0 / ny, D, (("circle", ci, cj, D),), Re=Re,
                                 n_steps=n_steps, seed=int(rng.integers(2 ** 31))))
    return out


class BatchedChannels:
    def __init__(self, configs, device="cuda", precision="mixed", workers=16, use_graph=True, persistent=False):
        dev = torch.device(device)
        self.device = torch.device("cuda", torch.cuda.current_device() if dev.index is None else dev.index)
        self.configs = list(configs)
        self.workers = max(1, min(workers, len(self.configs)))
        self.streams = [torch.cuda.Stream(device=self.device) for _ in self.configs]
        self.solvers = []
        for cfg, st in zip(self.configs, self.streams):
            with torch.cuda.stream(st):
                self.solvers.append(ChannelSolver(cfg, device=self.device, precision=precision, use_graph=use_graph))
                # cooperative (persistent) launches do not overlap with other streams' kernels:
                # a batch solves in graph-captured iteration chunks instead
                self.solvers[-1].persistent = persistent
        torch.cuda.synchronize(self.device)
        self.pool = ThreadPoolExecutor(max_workers=self.workers)
        self.records = [[] for _ in self.configs]
        self._err = None
        self._fused_ws = None
        self.fused_totals = None

    def _run_group(self, w, n_steps):
        torch.cuda.set_device(self.device)
        for k in range(w, len(self.solvers), self.workers):
            with torch.cuda.stream(self.streams[k]):
                for _ in range(n_steps):
                    self.records[k].append(self.solvers[k].step())
            self.streams[k].synchronize()

    def autotune(self, reps=2, cycles=None):
        """Pick the p' solve's launch shapes (multigrid tail, tile sizes, CG chunk
        length; :mod:`karman_taichi_gb300.autotune`) once per grid size: tuned on
        the first instance of each size, applied to every instance of that size.
        The fields each instance computes do not change.  With ``cycles`` the
        sweeps below level 0 are chosen too (the iterates then change within the
        solve tolerance).  Returns {"nx x ny": choice}."""
        from .autotune import apply_choice, tune_pressure
        chosen = {}
        for k, s in enumerate(self.solvers):
            key = f"{s.cfg.nx}x{s.cfg.ny}"
            if key not in chosen:
                with torch.cuda.stream(self.streams[k]):
                    chosen[key] = tune_pressure(s, reps=reps, cycles=cycles)
            apply_choice(s, chosen[key])
        torch.cuda.synchronize(self.device)
        return chosen

    def step_native(self, n_steps=1):
        """n_steps time steps of every instance by the library's native thread pool
        (kc_channel_batch_step); returns the wall time in seconds."""
        import ctypes as C
        from . import _lib as L
        n = len(self.solvers)
        chans = [s.native_struct() for s in self.solvers]
        arr = (C.POINTER(L.KcChannel) * n)(*[C.pointer(c) for c in chans])
        streams = (C.c_void_p * n)(*[st.cuda_stream for st in self.streams])
        stats = (L.KcChannelStats * n)()
        torch.cuda.synchronize(self.device)
        t0 = time.perf_counter()
        L.check(L.load().kc_channel_batch_step(arr, n, streams, self.workers, n_steps, stats), "kc_channel_batch_step")
        torch.cuda.synchronize(self.device)
        t = time.perf_counter() - t0
        for k in range(n):
            st = stats[k]
            self.records[k].append([dict(mass=st.mass, it_u=st.it_u, it_v=st.it_v, it_p=st.it_p, outer=st.outer,
                                         status=st.status)])
        return t

    def step_fused(self, n_steps=1):
        """n_steps time steps of every instance in ONE kernel launch
        (kc_channel_batch_fused: block k runs instance k's time steps, every
        stage of the mixed path inside the kernel).  Statistics go to
        ``records`` as for step_native (the last step) and ``fused_totals``
        (sums over the call's steps); returns the wall time in seconds."""
        import ctypes as C
        from . import _lib as L
        n = len(self.solvers)
        lib = L.load()
        chans = [s.native_struct() for s in self.solvers]
        arr = (C.POINTER(L.KcChannel) * n)(*[C.pointer(c) for c in chans])
        need = lib.kc_channel_batch_fused_ws_bytes(arr, n)
        if need == 0:
            raise RuntimeError("kc_channel_batch_fused_ws_bytes: " + lib.kc_last_error().decode())
        if self._fused_ws is None or self._fused_ws.numel() < need + 256:
            self._fused_ws = torch.empty(need + 256, dtype=torch.uint8, device=self.device)
        off = (-self._fused_ws.data_ptr()) % 256
        last = (L.KcChannelStats * n)()
        total = (L.KcChannelStats * n)()
        torch.cuda.synchronize(self.device)
        t0 = time.perf_counter()
        stream = torch.cuda.current_stream(self.device).cuda_stream
        L.check(lib.kc_channel_batch_fused(arr, n, n_steps, self._fused_ws.data_ptr() + off, need, last, total,
                                           stream), "kc_channel_batch_fused")
        torch.cuda.synchronize(self.device)
        t = time.perf_counter() - t0
        self.fused_totals = []
        for k in range(n):
            st, tt = last[k], total[k]
            self.records[k].append([dict(mass=st.mass, it_u=st.it_u, it_v=st.it_v, it_p=st.it_p, outer=st.outer,
                                         status=st.status)])
            self.fused_totals.append(dict(outer=tt.outer, it_u=tt.it_u, it_v=tt.it_v, it_p=tt.it_p,
                                          mass_max=tt.mass, status=tt.status, fallbacks=tt.fallbacks))
        return t

    def step(self, n_steps=1):
        """n_steps time steps of every instance (Python worker threads, one stream per
        instance); returns the wall time in seconds."""
        torch.cuda.synchronize(self.device)
        t0 = time.perf_counter()
        futs = [self.pool.submit(self._run_group, w, n_steps) for w in range(self.workers)]
        for f in futs:
            f.result()
        torch.cuda.synchronize(self.device)
        return time.perf_counter() - t0

    def cells(self):
        return sum(c.cells for c in self.configs)

    def close(self):
        self.pool.shutdown(wait=True)
