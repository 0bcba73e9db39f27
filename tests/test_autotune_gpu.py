"""The tile-shape tuner (chl_autotune): every candidate regroups independent
points, rows, columns and modes, so a tuned run, and runs forced to the
extreme shapes, must be bit-identical to the default run; and tuning must
leave every array a caller can read as it found it."""
from dataclasses import replace

import numpy as np
import pytest

from channel_rl_gb300 import cases as C

pytestmark = pytest.mark.gpu

WORKLOADS = {
    "rl_case_sized": lambda: [replace(C.smaller(C.rl_case(), 64, 40, 32), name="rl")],
    "vreman_rule2": lambda: [replace(C.smaller(C.rl_case(), 48, 24, 36), name="vr", LES_model=C.LES_VREMAN)],
    "c2_64cubed": lambda: [C.c2_wm64()],
    "uneven_batch": lambda: [C.smaller(C.c2_wm64(), 32, 16, 16), C.smaller(C.c3_roofline(les=C.LES_DSM), 48, 24, 36),
                             replace(C.smaller(C.rl_case(), 24, 10, 12), name="b2", LES_model=C.LES_DSM)],
}
FORCED = ((1, 1, 0, 64), (1, 1, 1, 128), (16 * 152, 16 * 152, 1, 256), (16 * 152, 1, 0, 64), (152, 152, 3, 128))
STEPS = 3


def _readable(ch, n):
    out = []
    for q in range(n):
        d = ch.download(inst=q, fields=("U", "V", "W", "nu_t"))
        d["p"] = ch.pseudo_pressure(inst=q)
        d["alpha"] = ch.wall_stress(inst=q)
        out.append(d)
    return out


def _run(cases_, shapes=None, tune=False):
    from channel_rl_gb300.host import Channel
    ch = Channel(cases_)
    for q, c in enumerate(cases_):
        ch.upload(*C.initial_fields(c), inst=q)
    ch.step(1)
    before = _readable(ch, len(cases_))
    report = None
    if tune:
        report = ch.autotune(reps=2)
    elif shapes is not None:
        ch.set_tile_shapes(*shapes)
    after = _readable(ch, len(cases_))
    for q in range(len(cases_)):
        for k in before[q]:
            assert np.array_equal(before[q][k], after[q][k]), ("tuning changed", q, k)
    info = ch.tile_shapes()
    # rebuilds nu_t from the strain / model nu_t and row coefficients the
    # last stage left, which the tuner's timing runs must not have replaced
    ch.compute_wall_model()
    wm_nut = [ch.download(inst=q, fields=("nu_t",))["nu_t"] for q in range(len(cases_))]
    ch.step(STEPS - 1)
    ch.compute_pressure()            # the same transforms in their pressure mode
    out = [ch.download(inst=q, fields=("U", "V", "W", "P", "nu_t")) for q in range(len(cases_))]
    for q in range(len(cases_)):
        out[q]["wm_nut"] = wm_nut[q]
    ch.close()
    return out, info, report


@pytest.mark.parametrize("name", sorted(WORKLOADS))
def test_tuned_and_forced_shapes_are_bit_identical(name):
    cases_ = WORKLOADS[name]()
    ref, info0, _ = _run(cases_)
    runs = {"tuned": _run(cases_, tune=True)}
    for shapes in FORCED:
        runs[shapes] = _run(cases_, shapes=shapes)
    for key, (out, info, report) in runs.items():
        for q in range(len(cases_)):
            for f in ("U", "V", "W", "P", "nu_t", "wm_nut"):
                assert np.array_equal(out[q][f], ref[q][f]), (key, info, q, f)
    # the forced shapes did change the partition
    assert runs[FORCED[0]][1]["tri_form"] != 1 and runs[FORCED[0]][1]["point_threads"] == 64
    assert runs[FORCED[0]][1]["z_cols"] >= runs[FORCED[2]][1]["z_cols"]
    out, info, report = runs["tuned"]
    assert "point_threads" in report and "x_min_blocks" in report and "tridiag" in report
    assert info["x_min_blocks"] in (1, 152, 304, 608, 1216, 2432)
    assert info["point_threads"] in (64, 128, 256) and info["tri_mode"] in (0, 1, 3)


def test_autotune_needs_fields():
    from channel_rl_gb300.host import Channel, ChlError
    ch = Channel(C.smaller(C.c2_wm64(), 16, 12, 16))
    with pytest.raises(ChlError, match="not uploaded"):
        ch.autotune()
    with pytest.raises(ChlError):
        ch.set_tile_shapes(0, 608, 2)
    with pytest.raises(ChlError):
        ch.set_tile_shapes(608, 608, 2, point_threads=96)
    ch.close()
