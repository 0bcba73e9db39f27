"""The three tridiagonal forms (row-batched, staged in shared memory, lane
split with an affine scan) inside batches: an instance with many modes keeps
one lane per mode and the serial sweep's exact arithmetic even when a small
instance in the same launch splits its columns, so every batched instance
equals its own single run bit for bit; the lane-split instances agree with
the oracle at the parity tolerance (covered on small grids by the parity
tests)."""
from dataclasses import replace

import numpy as np
import pytest

from channel_rl_gb300 import cases as C

pytestmark = pytest.mark.gpu


def _steps(cases_, n=3):
    from channel_rl_gb300.host import Channel
    ch = Channel(cases_)
    for q, c in enumerate(cases_):
        ch.upload(*C.initial_fields(c), inst=q)
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
        assert (form in (0, 1)) if c is big else form == 2, (c.name, form)
        for f in ("U", "V", "W", "P"):
            assert np.array_equal(batch[q][f], alone[0][f]), (c.name, f)
