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


def _round_trips(ch, inputs, scalars, pinned_out):
    """Two phases of set_fields / step / download: the first restores the
    scalars before each step (a synchronising call), the second runs the
    steps back to back.  pinned_out: pinned buffers (one set per step and
    phase) for chl_download_async with one chl_synchronize at the end of
    each phase, or None for the synchronous chl_download after every step."""
    out = []
    for phase in range(2):
        if phase == 1:
            ch.set_scalars(**scalars[0])
        for n, f in enumerate(inputs):
            ch.set_fields_ptr(*f)
            if phase == 0:
                ch.set_scalars(**scalars[n])
            ch.step(1)
            if pinned_out is None:
                d = ch.download()
                out.append([d[k] for k in "UVW"])
            else:
                bufs = pinned_out[phase * len(inputs) + n]
                ch.download_async(*(b[1] for b in bufs))
                out.append([b[1] for b in bufs])
        if pinned_out is not None:
            ch.synchronize()
    return out


def test_pipelined_round_trips_match_synchronous_steps():
    """The round trip queued step after step without waiting for it (the
    copies of one step overlap the computation of its neighbours) gives, step
    by step, exactly what the synchronous path gives, with different inputs
    every step: no copy reads or writes a staging area that a neighbouring
    step still uses.  Checked with a synchronising call between the steps
    and with none; the first phase also against chl_upload + chl_download."""
    from channel_rl_gb300.host import Channel
    base = C.smaller(C.c2_wm64(), 32, 24, 16)
    seeds = (11, 12, 13, 14, 15)
    fields = [C.initial_fields(replace(base, seed=s)) for s in seeds]
    ref = Channel(base)
    scalars, want = [], []
    for U, V, W in fields:
        ref.upload(U, V, W)
        scalars.append(ref.scalars())
        ref.step(1)
        want.append(ref.download())
    ref.close()
    pin_in = [[_pinned_like(a) for a in f] for f in fields]
    pin_out = [[_pinned_like(np.zeros_like(want[0][k])) for k in "UVW"] for _ in range(2 * len(seeds))]
    got = Channel(base)
    got.upload(*fields[0])
    queued = _round_trips(got, [[b[1] for b in f] for f in pin_in], scalars, pin_out)
    got.close()
    chk = Channel(base)
    chk.upload(*fields[0])
    synced = _round_trips(chk, [[np.asfortranarray(a) for a in f] for f in fields], scalars, None)
    chk.close()
    for n in range(len(seeds)):
        for j, k in enumerate("UVW"):
            assert np.array_equal(queued[n][j], want[n][k]), ("upload path", n, k)
    for n in range(2 * len(seeds)):
        for j, k in enumerate("UVW"):
            assert np.array_equal(queued[n][j], synced[n][j]), ("synchronous path", n, k)
