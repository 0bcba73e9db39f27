"""The host-buffer path a caller with its own copy of the fields uses every
step (chl_set_fields, chl_rk3_step, chl_download_async; the bench's e2e
loop): from pinned and from pageable buffers it must move exactly what
chl_upload and chl_download move, for every field layout and in a batch.
chl_set_fields replaces the fields only (the bulk-flow target Q0 stays the
one chl_upload computed), so the scalars are carried over explicitly."""
from dataclasses import replace

import numpy as np
import pytest

from channel_rl_gb300 import cases as C

pytestmark = pytest.mark.gpu


def _pinned_like(a):
    import torch
    t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
    v = t.numpy().reshape(a.shape, order="F")
    v[...] = a
    return t, v


@pytest.mark.parametrize("pinned", [True, False], ids=["pinned", "pageable"])
def test_set_fields_and_download_async_match_upload_and_download(pinned):
    from channel_rl_gb300.host import Channel
    batch = [C.smaller(C.c2_wm64(), 32, 16, 16), replace(C.smaller(C.c2_wm64(), 18, 13, 12), name="b")]
    ref = Channel(batch)
    got = Channel(batch)
    keep = []
    for q, c in enumerate(batch):
        U, V, W = C.initial_fields(c)
        ref.upload(U, V, W, inst=q)
        # set_fields needs an uploaded instance; upload something else first
        got.upload(np.zeros_like(U), np.zeros_like(V), np.zeros_like(W), inst=q)
        if pinned:
            bufs = [_pinned_like(a) for a in (U, V, W)]
            keep.append(bufs)
            got.set_fields_ptr(*(b[1] for b in bufs), inst=q)
        else:
            got.set_fields_ptr(np.asfortranarray(U), np.asfortranarray(V), np.asfortranarray(W), inst=q)
        got.set_scalars(inst=q, **ref.scalars(inst=q))
    ref.step(2)
    got.step(2)
    for q, c in enumerate(batch):
        want = ref.download(inst=q)
        if pinned:
            held = [_pinned_like(np.zeros_like(want[f])) for f in "UVW"]
            keep.append(held)
            outs = [h[1] for h in held]
        else:
            outs = [np.zeros_like(want[f], order="F") for f in "UVW"]
        got.download_async(*outs, inst=q)
        got.synchronize()
        for f, o in zip("UVW", outs):
            assert np.array_equal(o, want[f]), (q, f)
    ref.close()
    got.close()
