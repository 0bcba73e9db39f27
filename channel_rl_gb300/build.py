"""Build the in-tree CUDA library ``channel_rl_gb300/_build/libchl.so``.

Every translation unit under ``csrc/`` is compiled for sm_103a only, in
parallel, then linked into one shared library with the CUDA runtime linked
statically.  No cmake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libchl.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


# variants: None (the library) or "bounds" (every field index checked and
# clamped, violations recorded in the instance's status word)
VARIANTS = {None: (OUT, LIB, []),
            "bounds": (os.path.join(OUT, "bounds"), os.path.join(OUT, "libchl_bounds.so"), ["-DCHL_BOUNDS_CHECK"])}


def _stale(srcs, lib=LIB):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = srcs + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "chl.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False, extra=None, variant=None) -> str:
    out_dir, lib, vflags = VARIANTS[variant]
    srcs = sources()
    if not force and not _stale(srcs, lib):
        return lib
    os.makedirs(out_dir, exist_ok=True)
    nv = nvcc()
    extra = list(extra or []) + vflags

    def comp(src):
        obj = os.path.join(out_dir, os.path.basename(src)[:-3] + ".o")
        cmd = [nv, *ARCH, *FLAGS, *extra, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(comp, srcs))
    tmp = lib + ".tmp"
    cmd = [nv, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


PEAKS_SRC = os.path.join(HERE, "..", "bench_peaks.cu")
PEAKS_BIN = os.path.join(OUT, "bench_peaks")


def build_peaks(force: bool = False) -> str:
    """The peak probes of bench.py (bench_peaks.cu at the repository root),
    next to the library: bench.py measures the FP64 issue rate of the GPU it
    runs on with them.  Returns the binary's path, or "" where the source is
    absent."""
    if not os.path.exists(PEAKS_SRC):
        return ""
    if not force and os.path.exists(PEAKS_BIN) and os.path.getmtime(PEAKS_BIN) >= os.path.getmtime(PEAKS_SRC):
        return PEAKS_BIN
    os.makedirs(OUT, exist_ok=True)
    cmd = [nvcc(), *ARCH, "-O3", "-o", PEAKS_BIN + ".tmp", PEAKS_SRC]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for bench_peaks.cu:\n{r.stderr}")
    os.replace(PEAKS_BIN + ".tmp", PEAKS_BIN)
    return PEAKS_BIN


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
