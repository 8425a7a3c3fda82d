"""Build recipe for libkarman_gb300.so (sm_103a only).

Each translation unit is compiled by its own nvcc process (in parallel), then
linked into one shared library placed next to this file.  The assembly units
are compiled with ``-fmad=false`` so their arithmetic keeps the reference's
IEEE operation order; the solver units keep FMA contraction.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libkarman_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# translation unit -> extra flags
SOURCES = {
    "kc_api.cu": [],
    "kc_solver.cu": [],
    "kc_simple.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"],
    "kc_karman.cu": ["-fmad=false"],
    "kc_mg.cu": [],
    "kc_unet.cu": [],
    "kc_fields.cu": [],
    "kc_channel.cu": [],
    "kc_smoothers.cu": [],
    "kc_flex.cu": [],
    "kc_recycle.cu": [],
    "kc_batch.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"],
}


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libkarman_gb300")


def _needs_rebuild(src: str, obj: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(INCLUDE, "karman_gb300.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose: bool = False, force: bool = False, extra: list[str] | None = None) -> str:
    """Compile every CUDA translation unit for sm_103a and link the library.
    Returns the library path."""
    nvcc = nvcc_path()
    os.makedirs(BUILD, exist_ok=True)
    extra = list(extra or [])
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    objs = []

    def compile_one(name: str) -> str:
        src = os.path.join(CSRC, name)
        obj = os.path.join(BUILD, name.replace(".cu", ".o"))
        if force or _needs_rebuild(src, obj):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-I", INCLUDE, "-I", CSRC, *SOURCES[name], *extra, "-c", src, "-o", obj]
            if verbose:
                print(" ".join(cmd), flush=True)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {name}:\n{r.stdout}\n{r.stderr}")
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr, flush=True)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    if force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
