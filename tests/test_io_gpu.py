"""Snapshots of device state in the reference's format: what output_data
writes (mesh, U, V, W, P, nu_t) and a restart from it through
read_input_data's layout (input_output.f90:390-730)."""
from dataclasses import replace

import numpy as np
import pytest

from channel_rl_gb300 import cases as C

pytestmark = pytest.mark.gpu


def test_save_matches_device_state_and_restart_continues_exactly(tmp_path):
    from channel_rl_gb300.host import Channel, read_snapshot
    case = replace(C.smaller(C.c1_small(), 32, 24, 16), x_mass_cte=0, dPdx=2e-3)
    ch = Channel(case)
    ch.upload(*C.initial_fields(case))
    ch.step(3)
    path = str(tmp_path / "channel.3")
    ch.save_snapshot(path, with_pressure=True)
    d = ch.download(fields=("U", "V", "W", "P", "nu_t"))
    raw = open(path, "rb").read()
    s = read_snapshot(path)
    for f in "UVW":
        assert np.array_equal(s[f], d[f]), f
    # P and nu_t follow W in the file
    n = d["P"].size
    tail = np.frombuffer(raw, "<f8", count=n, offset=len(raw) - 8 * n).reshape(d["nu_t"].shape, order="F")
    assert np.array_equal(tail, d["nu_t"])
    Pf = np.frombuffer(raw, "<f8", count=n, offset=len(raw) - 8 * n - 12 - 8 * n).reshape(d["P"].shape, order="F")
    assert np.array_equal(Pf, d["P"])
    # restart: a fresh channel from the file advances exactly like the original
    ch2 = Channel(case)
    ch2.load_snapshot(path)
    ch.step(2)
    ch2.step(2)
    a, b = ch.download(), ch2.download()
    for f in "UVW":
        assert np.array_equal(a[f], b[f]), f
    ch.close()
    ch2.close()


def test_load_rejects_other_mesh(tmp_path):
    from channel_rl_gb300.host import Channel, ChlError
    a = C.smaller(C.c1_small(), 16, 12, 16)
    ch = Channel(a)
    ch.upload(*C.initial_fields(a))
    path = str(tmp_path / "a.init")
    ch.save_snapshot(path, with_pressure=False)
    other = replace(a, stretch=1.0)             # same extents, other y mesh
    ch2 = Channel(other)
    with pytest.raises(ChlError, match="mesh differs"):
        ch2.load_snapshot(path)
    ch.close()
    ch2.close()
