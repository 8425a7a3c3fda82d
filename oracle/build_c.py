"""Builds oracle/libkc_cpu.so, the C/OpenMP restatement of the channel plain
path (test infrastructure and timed CPU baseline only)."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "kc_cpu.c")
LIB = os.path.join(HERE, "libkc_cpu.so")


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O3", "-std=c17", "-fopenmp", "-fPIC", "-shared", "-o", LIB + ".tmp", SRC, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"gcc failed:\n{r.stdout}\n{r.stderr}")
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="-f" in sys.argv))
