"""The library from a plain C caller (channel_rl_gb300/examples/chl_run.c):
snapshot in, solver loop, snapshot out with P and nu_t, bit for bit what
the Python mirror computes from the same file."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from channel_rl_gb300 import cases as C

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_c_caller_matches_python(tmp_path):
    from channel_rl_gb300 import build
    from channel_rl_gb300.host import Channel, write_snapshot
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = build.build()
    exe = str(tmp_path / "chl_run")
    subprocess.run([cc, "-O2", "-Wall", os.path.join(ROOT, "channel_rl_gb300", "examples", "chl_run.c"),
                    "-I", os.path.join(ROOT, "include"), "-L", os.path.dirname(lib), "-lchl",
                    f"-Wl,-rpath,{os.path.dirname(lib)}", "-o", exe], check=True)
    case = C.smaller(C.c2_wm64(), 32, 24, 16)
    x, y, z = C.faces(case)
    U, V, W = C.initial_fields(case)
    src, dst = str(tmp_path / "start.init"), str(tmp_path / "channel.20")
    write_snapshot(src, x, y, z, U, V, W)
    nsteps = 20
    args = [exe, src, dst, str(nsteps), repr(case.nu), repr(case.CFL), repr(case.dPdx), str(case.x_mass_cte),
            str(case.LES_model), str(case.Dirichlet_nu_t), str(case.wall_model)]
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    assert "max|div|" in r.stdout
    ch = Channel(case)
    ch.upload(U, V, W)
    ch.step(nsteps)
    ch.compute_pressure()
    d = ch.download(fields=("U", "V", "W", "P", "nu_t"))
    ch.close()
    raw = open(dst, "rb").read()
    mesh = sum(4 + 8 * n for n in (case.nx, case.ny, case.nz, case.nx - 1, case.ny - 1, case.nz - 1))
    off = mesh
    for f in ("U", "V", "W", "P", "nu_t"):
        dims = np.frombuffer(raw, "<i4", 3, off)
        off += 12
        n = int(np.prod(dims))
        a = np.frombuffer(raw, "<f8", n, off).reshape(tuple(dims), order="F")
        off += 8 * n
        assert np.array_equal(a, d[f]), f
    assert off == len(raw)
