"""C ABI checks that need no GPU: the library loads, exports every symbol
include/chl.h declares, derives the reference's grid constants on the host
and rejects invalid grids before touching CUDA."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from channel_rl_gb300 import cases as CS
from channel_rl_gb300.host import EXPORTS, GridDesc, grid_constants, grid_desc
from oracle.channel_ref import Grid

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "chl.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(chl_[A-Za-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported(lib):
    syms = header_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert set(syms) == set(EXPORTS)


@pytest.mark.parametrize("case", [CS.c1_small(), CS.c2_wm64(), CS.c3_roofline(),
                                  CS.smaller(CS.c1_small(), 48, 20, 96)])
def test_host_grid_constants_match_oracle(lib, case):
    g = Grid(*CS.faces(case))
    gc = grid_constants(case)
    assert np.array_equal(gc["kxx"], g.kxx)
    assert np.array_equal(gc["kzz"], g.kzz)
    assert np.array_equal(gc["Dd"], g.Dd[2:g.nyg])
    assert np.array_equal(gc["Du"][:-1], g.Du[2:g.nyg - 1])
    assert np.array_equal(gc["Dl"][1:], g.Dl[3:g.nyg])
    assert np.array_equal(gc["w0"], g.w0[1:])
    assert (gc["dxmin"], gc["dymin"], gc["dzmin"]) == (g.dxmin, g.dymin, g.dzmin)
    assert (gc["coef_bc_1"], gc["coef_bc_2"]) == (g.coef_bc_1, g.coef_bc_2)


def _create(lib, case, mutate=None):
    keep = []
    d = grid_desc(case, keep)
    if mutate:
        mutate(d)
    h = C.c_void_p()
    rc = lib.chl_create(C.byref(d), C.byref(h))
    msg = lib.chl_last_error(h).decode() if h else ""
    if h:
        lib.chl_destroy(h)
    return rc, msg


@pytest.mark.parametrize("mutate,needle", [
    (lambda d: setattr(d, "nx", 35), "even"),
    (lambda d: setattr(d, "nz", 4), "even"),
    (lambda d: setattr(d, "LES_model", 7), "LES_model"),
    (lambda d: setattr(d, "LES_model", 5), "LES_model"),
    (lambda d: setattr(d, "Dirichlet_nu_t", 3), "Dirichlet_nu_t"),
])
def test_invalid_grid_rejected_without_gpu(lib, mutate, needle):
    rc, msg = _create(lib, CS.c1_small(), mutate)
    assert rc == 1 and needle in msg


def test_fft_length_rule(lib):
    # Nx = 2^a 3^b only (radix-4/3/2 transforms)
    case = CS.smaller(CS.c1_small(), 40, 12, 16)
    rc, msg = _create(lib, case)
    assert rc == 1 and "2^a 3^b" in msg


@pytest.mark.parametrize("axis", ["x", "z"])
def test_nonuniform_periodic_spacing_rejected(lib, axis):
    """The Fourier solve assumes uniform x and z (one spacing in the modified
    wavenumbers, as the reference's initialisation); a stretched periodic
    axis is refused at creation rather than solved wrongly."""
    case = CS.c1_small()
    keep = []
    d = grid_desc(case, keep)
    a = np.array(getattr(keep[0], axis), dtype=np.float64)
    a[3] += 0.1 * (a[4] - a[3])          # one face moved off the uniform mesh
    keep.append(a)
    setattr(d, axis, a.ctypes.data_as(C.POINTER(C.c_double)))
    h = C.c_void_p()
    rc = lib.chl_create(C.byref(d), C.byref(h))
    assert rc == 1 and "uniformly spaced" in lib.chl_last_error(h).decode()
    lib.chl_destroy(h)


def test_decreasing_coordinates_rejected(lib):
    case = CS.c1_small()
    keep = []
    d = grid_desc(case, keep)
    y = np.array(keep[0].y[::-1])
    keep.append(y)
    d.y = y.ctypes.data_as(C.POINTER(C.c_double))
    h = C.c_void_p()
    rc = lib.chl_create(C.byref(d), C.byref(h))
    assert rc == 1 and "increasing" in lib.chl_last_error(h).decode()
    lib.chl_destroy(h)
