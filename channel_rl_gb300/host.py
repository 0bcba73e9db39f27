"""Python mirror of the reference's hot-path interface over the C ABI.

``Channel`` exposes the Fortran subroutines of wadaniel/channel_RL that the
library replaces, under their own names (compute_dt, compute_time_step_RK3,
compute_eddy_viscosity, compute_wall_model, compute_rhs_u/v/w,
compute_projection_step, compute_dPx_for_constant_mass_flow,
compute_pressure, check_divergence, compute_statistics), operating on the
GPU-resident state of one or more channel instances.  Arrays crossing the
boundary are Fortran-ordered float64 with the reference's ghosted extents.

There is no CPU path: if ``libchl.so`` cannot be loaded or CUDA reports an
error, the call raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build
from .cases import Case, faces

_LIB = None
_F64P = C.POINTER(C.c_double)


class ChlError(RuntimeError):
    """A C-ABI call returned an error; ``rc`` is its CHL_E_* code."""

    def __init__(self, msg, rc=None):
        super().__init__(msg)
        self.rc = rc


# CHL_E_* (include/chl.h)
E_ARG, E_CUDA, E_NOMEM, E_STATE, E_NAN, E_IO, E_TIMEOUT = 1, 2, 3, 4, 5, 6, 7


class GridDesc(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("x", _F64P), ("y", _F64P), ("z", _F64P),
                ("nu", C.c_double), ("CFL", C.c_double), ("dPdx", C.c_double),
                ("x_mass_cte", C.c_int), ("LES_model", C.c_int), ("Dirichlet_nu_t", C.c_int),
                ("wall_model", C.c_int), ("Cs", C.c_double), ("Re_tau", C.c_double)]


class ParamsOut(C.Structure):
    """chl_parameters: the reference's parameter file (input_output.f90:20-91)."""
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("CFL", C.c_double), ("nu", C.c_double), ("dPdx", C.c_double),
                ("x_mass_cte", C.c_int), ("LES_model", C.c_int),
                ("nsteps", C.c_int), ("nsave", C.c_int), ("nstats", C.c_int), ("nmonitor", C.c_int),
                ("filein", C.c_char * 256), ("fileout", C.c_char * 256),
                ("nstep_init", C.c_int), ("random_init", C.c_int), ("Dirichlet_nu_t", C.c_int)]


class StatsOut(C.Structure):
    _fields_ = [(n, C.c_double) for n in
                ("utau", "Retau", "tau_wall", "Qflow_x", "Qflow_y", "dt", "t", "dPdx",
                 "max_div", "max_abs_div")]


# every symbol declared in include/chl.h
EXPORTS = (
    "chl_create", "chl_batch_create", "chl_destroy", "chl_last_error", "chl_num_instances",
    "chl_upload", "chl_download", "chl_download_pseudo_pressure", "chl_set_wall_stress",
    "chl_get_wall_stress", "chl_get_scalars", "chl_set_scalars", "chl_compute_dt",
    "chl_compute_time_step_RK3", "chl_rk3_step", "chl_compute_eddy_viscosity",
    "chl_compute_wall_model", "chl_compute_rhs", "chl_compute_projection_step",
    "chl_compute_dPx_for_constant_mass_flow", "chl_compute_pressure", "chl_check_divergence",
    "chl_stats", "chl_stats_profiles", "chl_synchronize", "chl_grid_constants_size",
    "chl_grid_constants", "chl_fft_pass_table", "chl_set_fields", "chl_download_async", "chl_time_steps",
    "chl_graph_kernel_count", "chl_profile_step",
    "chl_autotune", "chl_get_tile_shapes", "chl_set_tile_shapes",
    "chl_check_divergence_noalloc", "chl_noalloc_last_error", "chl_device_reset",
    "chl_mlp_set_params", "chl_mlp_get_params", "chl_mlp_configure", "chl_mlp_read_trace",
    "chl_mlp_eval", "chl_mlp_set_exploration", "chl_mlp_debug", "chl_mlp_read_record", "chl_tc_selftest",
    "chl_sqrt_selftest",
    "chl_snapshot_dims", "chl_snapshot_read", "chl_snapshot_write", "chl_io_last_error",
    "chl_read_parameters", "chl_save_snapshot", "chl_load_snapshot",
    "chl_agent_observe", "chl_agent_act", "chl_status_flags",
)
MLP_NPARAM = 4545
_F32P = C.POINTER(C.c_float)


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libchl.so (building it in-tree if asked and absent)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    # CHL_LIBRARY selects another build of the same ABI (e.g. the
    # bounds-checked variant); default: the in-tree library
    path = os.environ.get("CHL_LIBRARY") or _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise ChlError(f"{path} missing: run channel_rl_gb300.build.build()")
        _build.build()
    lib = C.CDLL(path)
    H = C.c_void_p
    lib.chl_create.argtypes = [C.POINTER(GridDesc), C.POINTER(H)]
    lib.chl_batch_create.argtypes = [C.c_int, C.POINTER(GridDesc), C.POINTER(H)]
    lib.chl_destroy.argtypes = [H]
    lib.chl_last_error.argtypes = [H]
    lib.chl_last_error.restype = C.c_char_p
    lib.chl_num_instances.argtypes = [H]
    lib.chl_upload.argtypes = [H, C.c_int, _F64P, _F64P, _F64P]
    lib.chl_download.argtypes = [H, C.c_int, _F64P, _F64P, _F64P, _F64P, _F64P]
    lib.chl_download_pseudo_pressure.argtypes = [H, C.c_int, _F64P]
    lib.chl_set_wall_stress.argtypes = [H, C.c_int, _F64P]
    lib.chl_get_wall_stress.argtypes = [H, C.c_int, _F64P]
    lib.chl_get_scalars.argtypes = [H, C.c_int, _F64P]
    lib.chl_set_scalars.argtypes = [H, C.c_int, _F64P]
    for n in ("chl_compute_dt", "chl_compute_time_step_RK3", "chl_compute_eddy_viscosity",
              "chl_compute_wall_model", "chl_compute_projection_step", "chl_compute_pressure",
              "chl_synchronize"):
        getattr(lib, n).argtypes = [H]
    lib.chl_rk3_step.argtypes = [H, C.c_int]
    lib.chl_compute_rhs.argtypes = [H, C.c_int, _F64P, _F64P, _F64P]
    lib.chl_compute_dPx_for_constant_mass_flow.argtypes = [H, C.c_int, _F64P]
    lib.chl_check_divergence.argtypes = [H, C.c_int, _F64P, _F64P]
    lib.chl_stats.argtypes = [H, C.c_int, C.POINTER(StatsOut)]
    lib.chl_stats_profiles.argtypes = [H, C.c_int] + [_F64P] * 7
    lib.chl_grid_constants_size.argtypes = [C.POINTER(GridDesc)]
    lib.chl_fft_pass_table.argtypes = [C.c_int, _F64P, C.c_int]
    lib.chl_grid_constants.argtypes = [C.POINTER(GridDesc), _F64P]
    lib.chl_set_fields.argtypes = [H, C.c_int, _F64P, _F64P, _F64P]
    lib.chl_download_async.argtypes = [H, C.c_int, _F64P, _F64P, _F64P]
    lib.chl_time_steps.argtypes = [H, C.c_int, _F64P]
    lib.chl_graph_kernel_count.argtypes = [H, C.POINTER(C.c_int)]
    lib.chl_profile_step.argtypes = [H, C.c_int, C.c_int, C.c_char_p, _F64P, C.POINTER(C.c_int)]
    lib.chl_autotune.argtypes = [H, C.c_int, C.c_char_p, C.c_int]
    lib.chl_get_tile_shapes.argtypes = [H, C.POINTER(C.c_int)]
    lib.chl_set_tile_shapes.argtypes = [H, C.c_int, C.c_int, C.c_int, C.c_int]
    lib.chl_mlp_set_params.argtypes = [H, _F32P]
    lib.chl_mlp_get_params.argtypes = [H, _F32P]
    lib.chl_mlp_configure.argtypes = [H, C.c_float, C.c_ulonglong, C.c_int]
    lib.chl_mlp_read_trace.argtypes = [H, C.c_int, _F32P, C.c_int]
    lib.chl_mlp_eval.argtypes = [H, _F32P, _F32P, C.c_int, _F32P, _F32P]
    lib.chl_mlp_set_exploration.argtypes = [H, C.c_int]
    lib.chl_mlp_debug.argtypes = [H, C.c_int, C.c_int]
    lib.chl_mlp_read_record.argtypes = [H, C.c_int, _F32P]
    lib.chl_tc_selftest.argtypes = [C.POINTER(C.c_ushort), C.POINTER(C.c_ushort), _F32P, C.c_int]
    lib.chl_sqrt_selftest.argtypes = [_F64P, _F64P, C.c_long]
    I = C.POINTER(C.c_int)
    lib.chl_snapshot_dims.argtypes = [C.c_char_p, I, I, I]
    lib.chl_snapshot_read.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int] + [_F64P] * 6
    lib.chl_snapshot_write.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int] + [_F64P] * 8
    lib.chl_io_last_error.restype = C.c_char_p
    lib.chl_read_parameters.argtypes = [C.c_char_p, C.POINTER(ParamsOut)]
    lib.chl_save_snapshot.argtypes = [H, C.c_int, C.c_char_p, C.c_int]
    lib.chl_load_snapshot.argtypes = [H, C.c_int, C.c_char_p]
    lib.chl_agent_observe.argtypes = [H, C.c_int, C.c_int, I, _F64P, _F64P, _F64P]
    lib.chl_agent_act.argtypes = [H, C.c_int, C.c_int, _F64P]
    lib.chl_status_flags.argtypes = [H, C.c_int, C.POINTER(C.c_int)]
    _LIB = lib
    return lib


def _ptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64
    return a.ctypes.data_as(_F64P)


@dataclass
class _Keep:
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray


def grid_desc(case: Case, keep: list):
    x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in faces(case))
    keep.append(_Keep(x, y, z))
    return GridDesc(case.nx, case.ny, case.nz, _ptr(x), _ptr(y), _ptr(z), case.nu, case.CFL,
                    case.dPdx, case.x_mass_cte, case.LES_model, case.Dirichlet_nu_t, case.wall_model,
                    case.Cs, case.Retau)


def _io_check(rc, what):
    if rc:
        raise ChlError(f"{what} failed ({rc}): {load().chl_io_last_error().decode()}")


def snapshot_dims(path):
    """(nx, ny, nz) face counts of a snapshot file."""
    n = [C.c_int(0) for _ in range(3)]
    _io_check(load().chl_snapshot_dims(os.fsencode(path), *(C.byref(v) for v in n)), "chl_snapshot_dims")
    return tuple(v.value for v in n)


def read_snapshot(path):
    """Mesh and fields of a snapshot in the reference's stream layout
    (read_input_data, input_output.f90:390-560): x, y, z and Fortran-ordered
    U(nx,nyg,nzg), V(nxg,ny,nzg), W(nxg,nyg,nz)."""
    nx, ny, nz = snapshot_dims(path)
    x, y, z = np.zeros(nx), np.zeros(ny), np.zeros(nz)
    U = np.zeros((nx, ny + 1, nz + 1), order="F")
    V = np.zeros((nx + 1, ny, nz + 1), order="F")
    W = np.zeros((nx + 1, ny + 1, nz), order="F")
    _io_check(load().chl_snapshot_read(os.fsencode(path), nx, ny, nz, *(_ptr(a) for a in (x, y, z)),
                                       *(a.ctypes.data_as(_F64P) for a in (U, V, W))), "chl_snapshot_read")
    return {"x": x, "y": y, "z": z, "U": U, "V": V, "W": W}


def write_snapshot(path, x, y, z, U, V, W, P=None, nu_t=None):
    """Write a snapshot as output_data does (input_output.f90:593-730);
    without P and nu_t it is an initial-field file."""
    x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
    nx, ny, nz = x.size, y.size, z.size
    shapes = {"U": (nx, ny + 1, nz + 1), "V": (nx + 1, ny, nz + 1), "W": (nx + 1, ny + 1, nz),
              "P": (nx + 1, ny + 1, nz + 1), "nu_t": (nx + 1, ny + 1, nz + 1)}
    arrs = []
    for name, a in (("U", U), ("V", V), ("W", W), ("P", P), ("nu_t", nu_t)):
        if a is None:
            arrs.append(None)
            continue
        a = np.asfortranarray(a, dtype=np.float64)
        if a.shape != shapes[name]:
            raise ValueError(f"{name}: shape {a.shape} != {shapes[name]}")
        arrs.append(a)
    ptrs = [a.ctypes.data_as(_F64P) if a is not None else None for a in arrs]
    _io_check(load().chl_snapshot_write(os.fsencode(path), nx, ny, nz, _ptr(x), _ptr(y), _ptr(z), *ptrs),
              "chl_snapshot_write")


def read_parameters(path):
    """The reference's parameter file (read_input_parameters, input_output.f90:20-91) as a dict."""
    p = ParamsOut()
    _io_check(load().chl_read_parameters(os.fsencode(path), C.byref(p)), "chl_read_parameters")
    out = {n: getattr(p, n) for n, _ in ParamsOut._fields_}
    out["filein"] = p.filein.decode()
    out["fileout"] = p.fileout.decode()
    return out


def _f32(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(_F32P)


def tc_selftest(A_bf16_bits, B_bf16_bits, variant=0):
    """D = A B^T on one CTA's tensor cores (tcgen05); A (128,64), B (64,64) uint16 BF16 bits."""
    lib = load()
    A = np.ascontiguousarray(A_bf16_bits, dtype=np.uint16)
    B = np.ascontiguousarray(B_bf16_bits, dtype=np.uint16)
    D = np.zeros((128, 64), np.float32)
    rc = lib.chl_tc_selftest(A.ctypes.data_as(C.POINTER(C.c_ushort)), B.ctypes.data_as(C.POINTER(C.c_ushort)),
                             D.ctypes.data_as(_F32P), variant)
    if rc:
        raise ChlError(f"chl_tc_selftest failed ({rc})", rc)
    return D


def sqrt_selftest(a):
    """The library's device square root (the strain magnitudes' root) of a."""
    lib = load()
    a = np.ascontiguousarray(a, dtype=np.float64)
    y = np.empty_like(a)
    rc = lib.chl_sqrt_selftest(a.ctypes.data_as(_F64P), y.ctypes.data_as(_F64P), a.size)
    if rc:
        raise ChlError(f"chl_sqrt_selftest failed ({rc})", rc)
    return y


def fft_pass_table(N):
    """The length-N transform's pass table (chl_fft_pass_table; no GPU needed)."""
    lib = load()
    n = lib.chl_fft_pass_table(int(N), None, 0)
    if n < 0:
        raise ChlError(f"chl_fft_pass_table: no table for length {N} ({n})", n)
    out = np.zeros(n)
    lib.chl_fft_pass_table(int(N), out.ctypes.data_as(_F64P), n)
    return out


def grid_constants(case: Case):
    """Host-side grid constants from the library (no GPU needed)."""
    lib = load()
    keep = []
    d = grid_desc(case, keep)
    n = lib.chl_grid_constants_size(C.byref(d))
    out = np.zeros(n)
    rc = lib.chl_grid_constants(C.byref(d), _ptr(out))
    if rc:
        raise ChlError(f"chl_grid_constants failed ({rc})")
    Nx, Nz, nyg, ny = case.Nx, case.Nz, case.Ny + 2, case.ny
    o = 0
    res = {}
    for name, m in (("kxx", Nx), ("kzz", Nz), ("Dd", nyg - 2), ("Du", nyg - 2), ("Dl", nyg - 2), ("w0", ny)):
        res[name] = out[o:o + m].copy()
        o += m
    res["dxmin"], res["dymin"], res["dzmin"], res["coef_bc_1"], res["coef_bc_2"] = out[o:o + 5]
    return res


class Channel:
    """One or more channel instances resident on the GPU."""

    def __init__(self, cases):
        if isinstance(cases, Case):
            cases = [cases]
        self.cases = list(cases)
        self.lib = load()
        self._keep = []
        descs = (GridDesc * len(self.cases))(*[grid_desc(c, self._keep) for c in self.cases])
        self.h = C.c_void_p()
        rc = self.lib.chl_batch_create(len(self.cases), descs, C.byref(self.h))
        self._check(rc, "chl_batch_create")

    # -- plumbing ------------------------------------------------------------
    def _check(self, rc, what):
        if rc:
            msg = self.lib.chl_last_error(self.h).decode() if self.h else ""
            raise ChlError(f"{what} failed ({rc}): {msg}", rc)

    def close(self):
        if getattr(self, "h", None):
            self.lib.chl_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _shape(self, q, field):
        c = self.cases[q]
        nx, ny, nz = c.nx, c.ny, c.nz
        return {"U": (nx, ny + 1, nz + 1), "V": (nx + 1, ny, nz + 1), "W": (nx + 1, ny + 1, nz),
                "P": (nx + 1, ny + 1, nz + 1)}[field]

    # -- state ---------------------------------------------------------------
    def upload(self, U, V, W, inst=0):
        arrs = [np.asfortranarray(a, dtype=np.float64) for a in (U, V, W)]
        for a, f in zip(arrs, "UVW"):
            if a.shape != self._shape(inst, f):
                raise ValueError(f"{f} has shape {a.shape}, expected {self._shape(inst, f)}")
        rc = self.lib.chl_upload(self.h, inst, *[_ptr(a) for a in arrs])
        self._check(rc, "chl_upload")

    def save_snapshot(self, path, inst=0, with_pressure=True):
        """output_data (input_output.f90:593-730) of one instance: mesh, U, V,
        W and, with the actual pressure computed first, P and nu_t."""
        self._check(self.lib.chl_save_snapshot(self.h, inst, os.fsencode(path), int(bool(with_pressure))),
                    "chl_save_snapshot")

    def load_snapshot(self, path, inst=0):
        """read_input_data (input_output.f90:390-560) into one instance; the
        file's mesh must be the instance's."""
        self._check(self.lib.chl_load_snapshot(self.h, inst, os.fsencode(path)), "chl_load_snapshot")

    def status_flags(self, inst=0):
        """Status word of an instance (1: non-finite velocity, 4: field index
        out of range, bounds-checked build only)."""
        f = C.c_int(0)
        self._check(self.lib.chl_status_flags(self.h, inst, C.byref(f)), "chl_status_flags")
        return f.value

    def agent_observe(self, nagents, y_ind, y_rand, inst=0):
        """States [2][nagents][6] and rewards [2][nagents] of the wall agents
        (send_recv_state_action, smarties_stat.f90:24-176) for given sampling
        rows y_ind (3 or 4) and weights y_rand, both [2][nagents]."""
        yi = np.ascontiguousarray(y_ind, dtype=np.int32).reshape(2, nagents)
        yr = np.ascontiguousarray(y_rand, dtype=np.float64).reshape(2, nagents)
        st = np.zeros((2, nagents, 6))
        rw = np.zeros((2, nagents))
        self._check(self.lib.chl_agent_observe(self.h, inst, nagents, yi.ctypes.data_as(C.POINTER(C.c_int)),
                                               _ptr(yr), _ptr(st), _ptr(rw)), "chl_agent_observe")
        return st, rw

    def agent_act(self, nagents, action, inst=0):
        """Wall stress from the agents' multiplicative actions [2][nagents]
        (smarties_stat.f90:193-256)."""
        a = np.ascontiguousarray(action, dtype=np.float64).reshape(2, nagents)
        self._check(self.lib.chl_agent_act(self.h, inst, nagents, _ptr(a)), "chl_agent_act")

    def download(self, inst=0, fields=("U", "V", "W")):
        out = {}
        args = []
        for f in ("U", "V", "W", "P", "nu_t"):
            if f in fields:
                a = np.zeros(self._shape(inst, "P" if f == "nu_t" else f), order="F")
                out[f] = a
                args.append(_ptr(a))
            else:
                args.append(None)
        rc = self.lib.chl_download(self.h, inst, *args)
        self._check(rc, "chl_download")
        return out

    def pseudo_pressure(self, inst=0):
        a = np.zeros(self._shape(inst, "P"), order="F")
        self._check(self.lib.chl_download_pseudo_pressure(self.h, inst, _ptr(a)), "download p")
        return a

    def set_wall_stress(self, alpha_x, inst=0):
        a = np.asfortranarray(alpha_x, dtype=np.float64)
        c = self.cases[inst]
        if a.shape != (c.nx, 2, c.nz + 1):
            raise ValueError("alpha_x must be (nx, 2, nzg)")
        self._check(self.lib.chl_set_wall_stress(self.h, inst, _ptr(a)), "chl_set_wall_stress")

    def wall_stress(self, inst=0):
        c = self.cases[inst]
        a = np.zeros((c.nx, 2, c.nz + 1), order="F")
        self._check(self.lib.chl_get_wall_stress(self.h, inst, _ptr(a)), "chl_get_wall_stress")
        return a

    def scalars(self, inst=0):
        s = np.zeros(4)
        self._check(self.lib.chl_get_scalars(self.h, inst, _ptr(s)), "chl_get_scalars")
        return dict(dt=s[0], t=s[1], dPdx=s[2], Qflow_x_0=s[3])

    def set_scalars(self, inst=0, **kw):
        cur = self.scalars(inst)
        cur.update(kw)
        s = np.array([cur["dt"], cur["t"], cur["dPdx"], cur["Qflow_x_0"]])
        self._check(self.lib.chl_set_scalars(self.h, inst, _ptr(s)), "chl_set_scalars")

    def set_fields_ptr(self, U, V, W, inst=0):
        """Stream-ordered replacement of U, V, W from host buffers (no sync)."""
        self._check(self.lib.chl_set_fields(self.h, inst, _ptr(U), _ptr(V), _ptr(W)), "chl_set_fields")

    def download_async(self, U, V, W, inst=0):
        self._check(self.lib.chl_download_async(self.h, inst, _ptr(U), _ptr(V), _ptr(W)), "chl_download_async")

    # -- learned wall model -------------------------------------------------------
    def mlp_set_params(self, theta):
        t, p = _f32(theta)
        assert t.size == MLP_NPARAM
        self._check(self.lib.chl_mlp_set_params(self.h, p), "chl_mlp_set_params")

    def mlp_params(self):
        t = np.zeros(MLP_NPARAM, np.float32)
        self._check(self.lib.chl_mlp_get_params(self.h, t.ctypes.data_as(_F32P)), "chl_mlp_get_params")
        return t

    def mlp_configure(self, sigma=0.0, seed=0, train=False):
        self._check(self.lib.chl_mlp_configure(self.h, float(sigma), int(seed), int(bool(train))), "chl_mlp_configure")

    def mlp_trace(self, inst=0, zero=True):
        t = np.zeros(MLP_NPARAM, np.float32)
        self._check(self.lib.chl_mlp_read_trace(self.h, inst, t.ctypes.data_as(_F32P), int(zero)), "chl_mlp_read_trace")
        return t

    def mlp_set_exploration(self, shared=False):
        """One exploration draw per instance and rollout (shared=True) or per
        wall point, stage and step (the default)."""
        self._check(self.lib.chl_mlp_set_exploration(self.h, int(bool(shared))), "chl_mlp_set_exploration")

    def mlp_debug(self, record=False, withhold_polls=0):
        """Checking hooks: per-point record of every evaluation, or MMAs
        withheld so that the completion wait runs out (chl_mlp_debug)."""
        self._check(self.lib.chl_mlp_debug(self.h, int(bool(record)), int(withhold_polls)), "chl_mlp_debug")

    def mlp_record(self, inst=0):
        """(3, 2, Nz, Nx, 8) float32: per RK stage, wall, z, x point the
        normalised features x0..x3, mu, the action a and the trust flag."""
        c = self.cases[inst]
        r = np.zeros((3, 2, c.Nz, c.Nx, 8), np.float32)
        self._check(self.lib.chl_mlp_read_record(self.h, inst, r.ctypes.data_as(_F32P)), "chl_mlp_read_record")
        return r

    def mlp_eval(self, x, g):
        """mu and sum_p g_p dmu_p/dtheta of the network on given features (tensor-core kernel)."""
        xx, px = _f32(x)
        gg, pg = _f32(g)
        P = gg.size
        mu = np.zeros(P, np.float32)
        tr = np.zeros(MLP_NPARAM, np.float32)
        self._check(self.lib.chl_mlp_eval(self.h, px, pg, P, mu.ctypes.data_as(_F32P), tr.ctypes.data_as(_F32P)),
                    "chl_mlp_eval")
        return mu, tr

    # -- measurement -------------------------------------------------------------
    def time_steps(self, nsteps):
        """Device milliseconds of nsteps graph replays (events on the library stream)."""
        ms = C.c_double()
        self._check(self.lib.chl_time_steps(self.h, nsteps, C.byref(ms)), "chl_time_steps")
        return ms.value

    def graph_kernel_count(self):
        n = C.c_int()
        self._check(self.lib.chl_graph_kernel_count(self.h, C.byref(n)), "chl_graph_kernel_count")
        return n.value

    def profile_step(self, reps=3, maxk=64):
        """{kernel: (ms per step, launches per step)} from event-bracketed steps."""
        names = C.create_string_buffer(32 * maxk)
        ms = np.zeros(maxk)
        cnt = (C.c_int * maxk)()
        n = self.lib.chl_profile_step(self.h, reps, maxk, names, _ptr(ms), cnt)
        if n < 0:
            self._check(-n, "chl_profile_step")
        raw = names.raw
        out = {}
        for i in range(n):
            nm = raw[32 * i:32 * i + 32].split(b"\0", 1)[0].decode()
            out[nm] = (float(ms[i]), int(cnt[i]))
        return out

    # -- tile-shape tuner ------------------------------------------------------
    def autotune(self, reps=10):
        """Time the Poisson solve's tile-shape candidates on the uploaded fields
        and keep the fastest (chl_autotune); returns the one-line report.
        Results are bit-identical whatever is chosen."""
        buf = C.create_string_buffer(512)
        self._check(self.lib.chl_autotune(self.h, int(reps), buf, 512), "chl_autotune")
        return buf.value.decode()

    def tile_shapes(self):
        """{x_min_blocks, z_min_blocks, tri_mode, point_threads, z_cols, tri_form, x_threads};
        tri_form 0 row-batched, 1 staged, 2 lane-split, 3 fused z solve."""
        v = (C.c_int * 7)()
        self._check(self.lib.chl_get_tile_shapes(self.h, v), "chl_get_tile_shapes")
        keys = ("x_min_blocks", "z_min_blocks", "tri_mode", "point_threads", "z_cols", "tri_form", "x_threads")
        return dict(zip(keys, (int(x) for x in v)))

    def set_tile_shapes(self, x_min_blocks, z_min_blocks, tri_mode, point_threads=256):
        self._check(self.lib.chl_set_tile_shapes(self.h, int(x_min_blocks), int(z_min_blocks), int(tri_mode),
                                                 int(point_threads)), "chl_set_tile_shapes")

    # -- reference subroutines -------------------------------------------------
    def compute_dt(self):
        self._check(self.lib.chl_compute_dt(self.h), "compute_dt")

    def compute_time_step_RK3(self):
        self._check(self.lib.chl_compute_time_step_RK3(self.h), "compute_time_step_RK3")

    def step(self, nsteps=1):
        """nsteps x (compute_dt; compute_time_step_RK3), graph-replayed, async."""
        self._check(self.lib.chl_rk3_step(self.h, nsteps), "chl_rk3_step")

    def synchronize(self):
        self._check(self.lib.chl_synchronize(self.h), "synchronize")

    def compute_eddy_viscosity(self):
        self._check(self.lib.chl_compute_eddy_viscosity(self.h), "compute_eddy_viscosity")

    def compute_wall_model(self):
        self._check(self.lib.chl_compute_wall_model(self.h), "compute_wall_model")

    def compute_rhs(self, inst=0):
        """(Fu, Fv, Fw) on the unique points: (Nx,Ny,Nz), (Nx,Ny-1,Nz), (Nx,Ny,Nz)."""
        c = self.cases[inst]
        Fu = np.zeros((c.Nx, c.Ny, c.Nz), order="F")
        Fv = np.zeros((c.Nx, c.Ny - 1, c.Nz), order="F")
        Fw = np.zeros((c.Nx, c.Ny, c.Nz), order="F")
        self._check(self.lib.chl_compute_rhs(self.h, inst, _ptr(Fu), _ptr(Fv), _ptr(Fw)), "compute_rhs")
        return Fu, Fv, Fw

    def compute_projection_step(self):
        self._check(self.lib.chl_compute_projection_step(self.h), "compute_projection_step")

    def compute_dPx_for_constant_mass_flow(self, inst=0):
        d = C.c_double()
        self._check(self.lib.chl_compute_dPx_for_constant_mass_flow(self.h, inst, C.byref(d)),
                    "compute_dPx_for_constant_mass_flow")
        return d.value

    def compute_pressure(self):
        self._check(self.lib.chl_compute_pressure(self.h), "compute_pressure")

    def check_divergence(self, inst=0):
        a, b = C.c_double(), C.c_double()
        self._check(self.lib.chl_check_divergence(self.h, inst, C.byref(a), C.byref(b)), "check_divergence")
        return a.value, b.value

    def compute_statistics(self, inst=0):
        s = StatsOut()
        self._check(self.lib.chl_stats(self.h, inst, C.byref(s)), "chl_stats")
        out = {n: getattr(s, n) for n, _ in StatsOut._fields_}
        ny = self.cases[inst].ny
        prof = [np.zeros(ny) for _ in range(7)]
        self._check(self.lib.chl_stats_profiles(self.h, inst, *[_ptr(p) for p in prof]), "chl_stats_profiles")
        for n, p in zip(("Umean", "Vmean", "Wmean", "U2mean", "V2mean", "W2mean", "UVmean"), prof):
            out[n] = p
        return out
