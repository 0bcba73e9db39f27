"""The allocation-free divergence check agrees with chl_check_divergence.

chl_check_divergence_noalloc serves callers that own all device memory and
must not let a library allocate (their memory comes from their own pool or a
framework's allocator, or their loop cannot take the synchronisation of
cudaMalloc).  It reads caller-owned device arrays and keeps its reduction
partials in a fixed 64 KiB device array shared by every call.  This file is
collected last so that a failure here comes after every other test has run.
"""
import ctypes as C

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
