"""ctypes wrapper of the oracle's multi-core C++ restatement (refcpu.cpp) —
TEST AND CPU-BASELINE INFRASTRUCTURE ONLY.

``RefCPU`` runs the reference's solver loop (compute_dt then
compute_time_step_RK3, app_main.f90:114-117) on the host cores with OpenMP
threads over the z loops, in the reference's Fortran array layout.  It is
checked against the NumPy oracle (tests/test_refcpu_cpu.py) and timed as the
host-core baseline; the GPU product never calls it.
"""
from __future__ import annotations

import ctypes as ct
import os

import numpy as np

from . import build_c

_lib = None


def load():
    global _lib
    if _lib is None:
        lib = ct.CDLL(build_c.build())
        P = ct.POINTER(ct.c_double)
        lib.refcpu_create.restype = ct.c_void_p
        lib.refcpu_create.argtypes = [ct.c_int, ct.c_int, ct.c_int, P, P, P, ct.c_double, ct.c_double,
                                      ct.c_double, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_double]
        lib.refcpu_upload.argtypes = [ct.c_void_p, P, P, P]
        lib.refcpu_step.argtypes = [ct.c_void_p, ct.c_int]
        lib.refcpu_download.argtypes = [ct.c_void_p, P, P, P, P]
        lib.refcpu_threads.restype = ct.c_int
        lib.refcpu_set_threads.argtypes = [ct.c_int]
        lib.refcpu_destroy.argtypes = [ct.c_void_p]
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(ct.POINTER(ct.c_double))


class RefCPU:
    """One channel on the host cores.  ``threads`` sets OMP_NUM_THREADS for
    the process before the library is first loaded (OpenMP reads it once)."""

    def __init__(self, case, threads=None):
        from channel_rl_gb300 import cases as C
        if threads is not None and _lib is None:
            os.environ["OMP_NUM_THREADS"] = str(int(threads))
        lib = load()
        self.case = case
        x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in C.faces(case))
        self._faces = (x, y, z)
        wm = case.wall_model
        if wm not in (C.WM_NONE, C.WM_STRESS, C.WM_EQLOG):
            raise ValueError("RefCPU covers the no/stress/equilibrium wall models only")
        if case.LES_model not in (C.LES_NONE, C.LES_SMAG, C.LES_DSM, C.LES_AMD, C.LES_VREMAN):
            raise ValueError("unsupported LES model")
        self.h = lib.refcpu_create(case.nx, case.ny, case.nz, _p(x), _p(y), _p(z), case.nu, case.CFL,
                                   case.dPdx, case.x_mass_cte, case.LES_model, case.Dirichlet_nu_t,
                                   wm, case.Cs)
        self.shapes = {"U": (case.nx, case.ny + 1, case.nz + 1), "V": (case.nx + 1, case.ny, case.nz + 1),
                       "W": (case.nx + 1, case.ny + 1, case.nz)}

    @staticmethod
    def threads():
        return int(load().refcpu_threads())

    @staticmethod
    def set_threads(n):
        load().refcpu_set_threads(int(n))

    def upload(self, U, V, W):
        a = [np.asfortranarray(f, dtype=np.float64) for f in (U, V, W)]
        load().refcpu_upload(self.h, *(_p(f) for f in a))

    def step(self, n=1):
        load().refcpu_step(self.h, int(n))

    def download(self):
        out = {k: np.zeros(s, dtype=np.float64, order="F") for k, s in self.shapes.items()}
        dt = np.zeros(1)
        load().refcpu_download(self.h, _p(out["U"]), _p(out["V"]), _p(out["W"]), _p(dt))
        out["dt"] = float(dt[0])
        return out

    def close(self):
        if self.h:
            load().refcpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
