"""The tridiagonal forms (row-batched, staged in shared memory, lane split
with an affine scan, and the fused z solve that runs the z transforms and
the lane-split sweeps of one kx in one thread-block cluster) inside
batches: an instance with many modes keeps one lane per mode and the serial
sweep's exact arithmetic even when a small instance in the same launch
splits its columns, so every batched instance equals its own single run bit
for bit; the fused z solve equals the separate launches bit for bit; the
lane-split instances agree with the oracle at the parity tolerance (covered
on small grids by the parity tests)."""
from dataclasses import replace

import numpy as np
import pytest

from channel_rl_gb300 import cases as C

pytestmark = pytest.mark.gpu
C_MIN = 4 * 152          # the default block-count target of the transforms


def _steps(cases_, n=3, tri_mode=None):
    from channel_rl_gb300.host import Channel
    ch = Channel(cases_)
    for q, c in enumerate(cases_):
        ch.upload(*C.initial_fields(c), inst=q)
    if tri_mode is not None:
        ch.set_tile_shapes(C_MIN, C_MIN, tri_mode, 256)
    form = ch.tile_shapes()["tri_form"]
    ch.step(n)
    ch.compute_pressure()
    out = [ch.download(inst=q, fields=("U", "V", "W", "P")) for q in range(len(cases_))]
    ch.close()
    return out, form


def test_mixed_lane_counts_in_one_batch_match_single_runs():
    big = replace(C.smaller(C.c3_roofline(les=C.LES_DSM), 256, 16, 192), name="big")   # 24768 modes: one lane
    small = replace(C.smaller(C.c2_wm64(), 32, 24, 16), name="small")                  # 544 modes: split
    mid = replace(C.smaller(C.c2_wm64(), 32, 13, 48), name="mid")                      # 816 modes, 4 lanes of 4,4,4,1 rows
    batch, form_b = _steps([big, small, mid])
    assert form_b == 2
    for q, c in enumerate((big, small, mid)):
        alone, form = _steps([c])
        # alone, the split instances take the fused z solve (one lane count each)
        assert (form in (0, 1)) if c is big else form == 3, (c.name, form)
        for f in ("U", "V", "W", "P"):
            assert np.array_equal(batch[q][f], alone[0][f]), (c.name, f)


FUSED_CASES = {
    "c1_32x48x32_8_lanes": lambda: [C.c1_small()],
    "wm_32x12x16_4_lanes": lambda: [C.smaller(C.c2_wm64(), 32, 12, 16)],
    "ragged_6x9x12_empty_lane": lambda: [C.smaller(C.c1_small(), 6, 9, 12)],
    "c2_64cubed_1_lane": lambda: [C.c2_wm64()],
    "batch_same_lanes": lambda: [C.smaller(C.c1_small(), 32, 32, 32), C.c1_small()],
}


@pytest.mark.parametrize("name", sorted(FUSED_CASES))
def test_fused_z_solve_is_bit_identical(name):
    """Forced fused z solve (tri_mode 3) against the separate z transforms and
    tridiagonal launches (tri_mode 0): three steps and the actual pressure."""
    cases_ = FUSED_CASES[name]()
    fused, form_f = _steps(cases_, tri_mode=3)
    plain, form_p = _steps(cases_, tri_mode=0)
    assert form_f == 3 and form_p in (0, 2), (form_f, form_p)
    for q in range(len(cases_)):
        for f in ("U", "V", "W", "P"):
            assert np.array_equal(fused[q][f], plain[q][f]), (name, q, f)
