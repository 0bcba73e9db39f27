"""Build recipe of the oracle's multi-core C++ restatement (test and CPU
baseline infrastructure only): ``oracle/refcpu.cpp`` -> ``oracle/_build/
librefcpu.so`` with g++ and OpenMP.  Portable flags only (no -march), so the
same recipe builds on x86_64 and aarch64 hosts."""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "refcpu.cpp")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "librefcpu.so")
FLAGS = ["-std=c++17", "-O3", "-fopenmp", "-fPIC", "-shared", "-Wall"]


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("g++ not found: the oracle's C++ restatement cannot be built")
    os.makedirs(OUT, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    r = subprocess.run([cxx, *FLAGS, SRC, "-o", tmp], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed for {SRC}:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
