"""The allocation-free divergence check agrees with chl_check_divergence.

chl_check_divergence_noalloc serves callers that own all device memory and
must not let a library allocate (their memory comes from their own pool or a
framework's allocator, or their loop cannot take the synchronisation of
cudaMalloc).  It reads caller-owned device arrays and keeps its reduction
partials in a fixed 64 KiB device array shared by every call.  This file is
collected last so that a failure here comes after every other test has run.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from channel_rl_gb300 import cases as CS

F64P = C.POINTER(C.c_double)


def _bind(lib):
    f = lib.chl_check_divergence_noalloc
    f.argtypes = [C.c_void_p] * 6 + [C.c_int, C.c_int, C.c_int, C.c_void_p, F64P, F64P]
    f.restype = C.c_int
    lib.chl_noalloc_last_error.restype = C.c_char_p
    return f


def test_rejects_grids_beyond_its_scratch(lib):
    f = _bind(lib)
    a, b = C.c_double(), C.c_double()
    dummy = C.c_void_p(16)   # never dereferenced: the size check comes first
    rc = f(dummy, dummy, dummy, dummy, dummy, dummy, 34, 49, 5000, None, C.byref(a), C.byref(b))
    assert rc == 1
    assert b"4096" in lib.chl_noalloc_last_error()


@pytest.mark.gpu
def test_noalloc_divergence_matches_handle_version_twice(lib):
    import torch
    from channel_rl_gb300.host import Channel
    f = _bind(lib)
    case = CS.smaller(CS.c2_wm64(), 48, 32, 64)
    ch = Channel(case)
    U, V, W = CS.initial_fields(case)
    ch.upload(U, V, W)
    x, y, z = (torch.tensor(a, dtype=torch.float64, device="cuda") for a in CS.faces(case))
    stream = torch.cuda.current_stream()
    for call in range(2):
        if call == 1:
            ch.step(1)            # a different, divergence-free field for the second call
        ch.synchronize()
        d = ch.download(fields=("U", "V", "W"))
        dev = [torch.tensor(np.asfortranarray(d[k]).ravel(order="F"), device="cuda") for k in "UVW"]
        torch.cuda.synchronize()
        ref = ch.check_divergence()
        a, b = C.c_double(), C.c_double()
        rc = f(*(C.c_void_p(t.data_ptr()) for t in dev), *(C.c_void_p(t.data_ptr()) for t in (x, y, z)),
               case.nx, case.ny, case.nz, C.c_void_p(stream.cuda_stream), C.byref(a), C.byref(b))
        assert rc == 0, lib.chl_noalloc_last_error()
        # The two kernels differ only in rounding (this one divides by the
        # spacings, the handle's kernel multiplies by stored reciprocals), so
        # they agree to rounding of the terms being summed: the velocity
        # differences over the spacings.  After a projected step the
        # divergence itself is at that rounding level, so it cannot be the scale.
        h = min(np.diff(a_).min() for a_ in CS.faces(case))
        grad = sum(np.abs(d[k]).max() for k in "UVW") * 2.0 / h
        scale = max(abs(ref[1]), grad)
        assert abs(b.value - ref[1]) <= 1e-12 * scale, (call, b.value, ref)
        assert abs(a.value - ref[0]) <= 1e-12 * scale, (call, a.value, ref)
        if call == 0:
            assert ref[1] > 1e-3           # random initial field: far from solenoidal
        else:
            assert ref[1] < 1e-12          # after a projected step
    ch.close()


# Run in a child process: it drives contexts through the driver API, which
# must not disturb the test process's own CUDA context.
_CONTEXTS = r"""
import ctypes as C, sys
from dataclasses import replace
import numpy as np
sys.path.insert(0, sys.argv[1])
from channel_rl_gb300 import cases as CS
from channel_rl_gb300.host import load

lib = load(build_if_missing=False)
f = lib.chl_check_divergence_noalloc
F64P = C.POINTER(C.c_double)
f.argtypes = [C.c_void_p] * 6 + [C.c_int, C.c_int, C.c_int, C.c_void_p, F64P, F64P]
f.restype = C.c_int
lib.chl_noalloc_last_error.restype = C.c_char_p
cu = C.CDLL("libcuda.so.1")

def ck(r, what):
    if r != 0:
        raise SystemExit(f"{what}: CUresult {r}")

def expected(U, V, W, x, y, z):
    # centres i = 2..nxg-1, j = 2..nyg-1, k = 2..nzg-1 (Fortran), 0-based here
    d = ((U[1:, 1:-1, 1:-1] - U[:-1, 1:-1, 1:-1]) / np.diff(x)[:, None, None]
         + (V[1:-1, 1:, 1:-1] - V[1:-1, :-1, 1:-1]) / np.diff(y)[None, :, None]
         + (W[1:-1, 1:-1, 1:] - W[1:-1, 1:-1, :-1]) / np.diff(z)[None, None, :])
    return max(0.0, float(d.max())), float(np.abs(d).max())

def call(case, seed):
    U, V, W = CS.initial_fields(case if seed is None else replace(case, seed=seed))
    x, y, z = CS.faces(case)
    ptrs = []
    for a in (U, V, W, x, y, z):
        a = np.asfortranarray(a, dtype=np.float64)
        d = C.c_uint64()
        ck(cu.cuMemAlloc_v2(C.byref(d), C.c_size_t(a.nbytes)), "cuMemAlloc")
        ck(cu.cuMemcpyHtoD_v2(d, a.ctypes.data_as(C.c_void_p), C.c_size_t(a.nbytes)), "cuMemcpyHtoD")
        ptrs.append(d)
    a, b = C.c_double(), C.c_double()
    rc = f(*(C.c_void_p(p.value) for p in ptrs), case.nx, case.ny, case.nz, None, C.byref(a), C.byref(b))
    for p in ptrs:
        ck(cu.cuMemFree_v2(p), "cuMemFree")
    if rc != 0:
        raise SystemExit(f"noalloc rc {rc}: {lib.chl_noalloc_last_error()}")
    ref = expected(U, V, W, x, y, z)
    h = min(np.diff(q).min() for q in (x, y, z))
    scale = sum(np.abs(q).max() for q in (U, V, W)) * 2.0 / h
    if abs(a.value - ref[0]) > 1e-12 * scale or abs(b.value - ref[1]) > 1e-12 * scale:
        raise SystemExit(f"mismatch: {(a.value, b.value)} vs {ref}")
    return b.value

case = CS.smaller(CS.c2_wm64(), 48, 32, 64)
ck(cu.cuInit(0), "cuInit")
dev = C.c_int()
ck(cu.cuDeviceGet(C.byref(dev), 0), "cuDeviceGet")
prim = C.c_void_p()
ck(cu.cuDevicePrimaryCtxRetain(C.byref(prim), dev), "cuDevicePrimaryCtxRetain")
ck(cu.cuCtxSetCurrent(prim), "cuCtxSetCurrent")
r1 = call(case, None)                       # primary context
other = C.c_void_p()
ck(cu.cuCtxCreate_v2(C.byref(other), 0, dev), "cuCtxCreate")     # now current
r2 = call(case, 99)                         # a second context: the array has another address there
ck(cu.cuCtxDestroy_v2(other), "cuCtxDestroy")
ck(cu.cuCtxSetCurrent(prim), "cuCtxSetCurrent")
r3 = call(case, 7)                          # back in the primary context, fresh buffers
# a device reset through the library's own runtime: the primary context and
# every allocation in it go; the next call finds the array in the new one
lib.chl_device_reset.restype = C.c_int
if lib.chl_device_reset() != 0:
    raise SystemExit("chl_device_reset failed")
again = C.c_void_p()
ck(cu.cuDevicePrimaryCtxRetain(C.byref(again), dev), "cuDevicePrimaryCtxRetain after the reset")
ck(cu.cuCtxSetCurrent(again), "cuCtxSetCurrent after the reset")
r4 = call(case, 5)                          # fresh buffers in the reset context
cu.cuDevicePrimaryCtxRelease_v2(dev)
cu.cuDevicePrimaryCtxRelease_v2(dev)
print("ok", r1, r2, r3, r4)
"""


@pytest.mark.gpu
def test_noalloc_in_a_second_context_and_after_a_reset():
    """A caller may run the library in a context it created with the driver
    API, or reset the device between calls.  The scratch array then sits at
    another address, and each call must find it there: the primary context,
    a second context with fresh buffers, the primary context again, and,
    after chl_device_reset, the new primary context with fresh buffers, each
    checked against the divergence computed on the host."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _CONTEXTS, root], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok"), r.stdout
