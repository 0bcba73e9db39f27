"""Snapshot and parameter files in the reference's formats (host only).

The snapshot layout is the stream of output_data / read_input_data
(input_output.f90:390-730) that scripts/check_file.m reads; the checks below
parse it with an independent NumPy reader written from that layout."""
import numpy as np
import pytest

from channel_rl_gb300 import cases as C


def _check_file_reader(path):
    """check_file.m's reads: int32 n + float64[n] for x, y, z, xm, ym, zm,
    then int32[3] + float64 array per field, little-endian, until EOF."""
    raw = open(path, "rb").read()
    off = 0

    def i32(n):
        nonlocal off
        v = np.frombuffer(raw, "<i4", n, off)
        off += 4 * n
        return v

    def f64(n):
        nonlocal off
        v = np.frombuffer(raw, "<f8", n, off)
        off += 8 * n
        return v

    out = {}
    for name in ("x", "y", "z", "xm", "ym", "zm"):
        n = int(i32(1)[0])
        out[name] = f64(n)
    fields = []
    while off < len(raw):
        d = i32(3)
        fields.append(f64(int(np.prod(d))).reshape(tuple(d), order="F"))
    return out, fields


def _fields(case, seed=3):
    rng = np.random.default_rng(seed)
    nx, ny, nz = case.nx, case.ny, case.nz
    return [np.asfortranarray(rng.standard_normal(s)) for s in
            ((nx, ny + 1, nz + 1), (nx + 1, ny, nz + 1), (nx + 1, ny + 1, nz),
             (nx + 1, ny + 1, nz + 1), (nx + 1, ny + 1, nz + 1))]


def test_snapshot_layout_matches_check_file(tmp_path):
    from channel_rl_gb300.host import write_snapshot
    case = C.smaller(C.c1_small(), 16, 12, 8)
    x, y, z = C.faces(case)
    U, V, W, P, nt = _fields(case)
    path = str(tmp_path / "snap.1000")
    write_snapshot(path, x, y, z, U, V, W, P, nt)
    mesh, fields = _check_file_reader(path)
    assert np.array_equal(mesh["x"], x) and np.array_equal(mesh["y"], y) and np.array_equal(mesh["z"], z)
    assert np.array_equal(mesh["xm"], 0.5 * (x[:-1] + x[1:]))
    assert np.array_equal(mesh["ym"], 0.5 * (y[:-1] + y[1:]))
    assert len(fields) == 5
    for a, b in zip(fields, (U, V, W, P, nt)):
        assert a.shape == b.shape and np.array_equal(a, b)
    # an initial-field file (.init) holds U, V, W only
    write_snapshot(path, x, y, z, U, V, W)
    assert len(_check_file_reader(path)[1]) == 3


def test_snapshot_round_trip(tmp_path):
    from channel_rl_gb300.host import read_snapshot, snapshot_dims, write_snapshot
    case = C.smaller(C.c2_wm64(), 24, 16, 12)
    x, y, z = C.faces(case)
    U, V, W, P, nt = _fields(case, 5)
    path = str(tmp_path / "r.init")
    write_snapshot(path, x, y, z, U, V, W, P, nt)
    assert snapshot_dims(path) == (case.nx, case.ny, case.nz)
    s = read_snapshot(path)
    for k, a in (("x", x), ("y", y), ("z", z), ("U", U), ("V", V), ("W", W)):
        assert np.array_equal(s[k], a), k


def test_snapshot_errors(tmp_path):
    from channel_rl_gb300.host import ChlError, read_snapshot, write_snapshot
    case = C.smaller(C.c1_small(), 16, 12, 8)
    x, y, z = C.faces(case)
    U, V, W, _, _ = _fields(case)
    path = tmp_path / "bad.init"
    write_snapshot(str(path), x, y, z, U, V, W)
    raw = bytearray(path.read_bytes())
    # U's first extent sits right after the mesh block
    off = sum(4 + 8 * n for n in (case.nx, case.ny, case.nz, case.nx - 1, case.ny - 1, case.nz - 1))
    raw[off:off + 4] = np.int32(case.nx + 2).tobytes()
    path.write_bytes(bytes(raw))
    with pytest.raises(ChlError, match="wrong size"):
        read_snapshot(str(path))
    path.write_bytes(bytes(raw[: off - 10]))
    with pytest.raises(ChlError):
        read_snapshot(str(path))
    with pytest.raises(ChlError, match="cannot open"):
        read_snapshot(str(tmp_path / "missing.init"))
    with pytest.raises(ValueError):
        write_snapshot(str(path), x, y, z, V, U, W)


PARAMS = """! domain size nx ny nz
 34 25 18
! CFL (or fixed dT if negative)
 -2.5d-3
! viscosity
  1.0e-4
! Pressure gradient dPdx, x_mass_cte (0->use dPdx, 1->constant mass flow)
 0.0017 0
! LES model (0: no model 1: constant smagorinsky 2: DSM 3: AMD 4: Vreman)
 3
! nsteps, nsave, nstats, nmonitor
 200   101   50   10
! input flow field file
 'start.init'
! output flow field file
 'out/channel_run'
! first number for output flow field
 7
! random initial condition 0->no (reads previous file), 1->yes
 0
! (SGS) BC for eddy vicosity: 1->Dirichlet, 0->Neumann
 1
"""


def test_parameter_file(tmp_path):
    from channel_rl_gb300.host import ChlError, read_parameters
    path = tmp_path / "input_parameters"
    path.write_text(PARAMS)
    p = read_parameters(str(path))
    assert (p["nx"], p["ny"], p["nz"]) == (34, 25, 18)
    assert p["CFL"] == -2.5e-3 and p["nu"] == 1.0e-4 and p["dPdx"] == 0.0017
    assert p["x_mass_cte"] == 0 and p["LES_model"] == 3
    assert (p["nsteps"], p["nsave"], p["nstats"], p["nmonitor"]) == (200, 101, 50, 10)
    assert p["filein"] == "start.init" and p["fileout"] == "out/channel_run"
    assert (p["nstep_init"], p["random_init"], p["Dirichlet_nu_t"]) == (7, 0, 1)
    path.write_text("\n".join(PARAMS.splitlines()[:9]))
    with pytest.raises(ChlError, match="value lines"):
        read_parameters(str(path))


def test_case_from_reference_files(tmp_path):
    """A parameter file plus the snapshot it names become a case with the
    file's mesh, physics and fields (stretched y mesh kept exactly)."""
    from channel_rl_gb300.host import grid_constants, write_snapshot
    base = C.Case(name="b", Nx=32, Ny=24, Nz=16, stretch=1.5)
    x, y, z = C.faces(base)
    U, V, W, _, _ = _fields(base, 9)
    write_snapshot(str(tmp_path / "start.init"), x, y, z, U, V, W)
    (tmp_path / "input_parameters").write_text(PARAMS)
    case, (U2, V2, W2), p = C.case_from_files(str(tmp_path / "input_parameters"), wall_model=C.WM_EQLOG)
    assert (case.Nx, case.Ny, case.Nz) == (32, 24, 16)
    assert case.LES_model == C.LES_AMD and case.CFL == -2.5e-3 and case.Dirichlet_nu_t == 1
    xf, yf, zf = C.faces(case)
    assert np.array_equal(yf, y) and np.array_equal(xf, x) and np.array_equal(zf, z)
    assert np.array_equal(U2, U) and np.array_equal(W2, W)
    g = grid_constants(case)
    assert np.isfinite(g["Dd"]).all()
