"""The learned wall model inside the channel, against the oracle's restatement
of its stage (oracle/mlp_wm_ref.py), with the trained network.

Per RK3 stage and wall point the GPU records its normalised features, mu,
the action and the trust flag (chl_mlp_debug).  The oracle runs the same
steps from the same state and is given the GPU's actions, so the BF16
rounding of the network drops out of the field comparison; the network
itself is bounded against the BF16 oracle separately.

Tolerances:
  features        |x_gpu - x_oracle| <= 1e-6 (FP32 values of O(1); the FP64
                  inputs agree to ~1e-12, so at most an FP32 rounding flip)
  trust flags     identical
  mu              <= 1e-3 (BF16 activations: a last-bit flip of one hidden
                  unit moves mu by up to ~1e-4, tests/test_mlp_gpu.py)
  alpha_x, U, V, W  <= FIELD_RTOL (1e-12) relative, after each of 3 steps
"""
import os
from dataclasses import replace

import numpy as np
import pytest

from channel_rl_gb300 import cases as C
from tests.helpers import FIELD_RTOL, oracle_for, regions, rel

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FEATURE_ATOL = 1e-6
MU_ATOL = 1e-3


def _theta():
    return np.load(os.path.join(ROOT, "channel_rl_gb300", "data", "mlp_wm.npy")).astype(np.float32)


def _channel(cases_):
    from channel_rl_gb300.host import Channel
    return Channel(cases_)


def test_learned_stage_and_fields_match_oracle():
    case = replace(C.smaller(C.c2_wm64(), 32, 32, 32), wall_model=C.WM_MLP)
    theta = _theta()
    U, V, W = C.initial_fields(case)
    ch = _channel(case)
    ch.upload(U, V, W)
    ch.mlp_set_params(theta)
    ch.mlp_debug(record=True)
    o = oracle_for(case)
    o.set_fields(U, V, W)
    o.mlp_theta = theta
    acts = {}
    o.mlp_actions = lambda s: acts[s]
    g = o.g
    reg = regions(g)
    moved = 0.0
    for step in range(3):
        ch.step(1)
        ch.synchronize()
        rec = ch.mlp_record().transpose(0, 3, 1, 2, 4)          # (stage, Nx, wall, Nz, 8)
        for s in range(3):
            acts[s] = rec[s, ..., 5].copy()
        o.step()
        assert ch.scalars()["dt"] == o.dt, step
        for s in range(3):
            info, r = o.mlp_info[s], rec[s]
            assert np.abs(info["x"] - r[..., :4]).max() <= FEATURE_ATOL, (step, s)
            assert np.array_equal(info["trusted"], r[..., 6] == 1.0), (step, s)
            t = info["trusted"]
            if t.any():
                assert np.abs(info["mu"][t] - r[..., 4][t]).max() <= MU_ATOL, (step, s)
                moved = max(moved, float(np.abs(r[..., 5][t]).max()))
        a = ch.wall_stress()
        assert rel(a[1:-1, :, 1:-2], o.alpha_x[2:g.nx, 1:3, 2:g.nzg - 1]) < FIELD_RTOL, step
        d = ch.download(fields=("U", "V", "W"))
        src = {"U": o.U, "V": o.V, "W": o.W}
        for f in "UVW":
            e = rel(d[f][reg[f]], src[f][1:, 1:, 1:][reg[f]])
            assert e < FIELD_RTOL, (step, f, e)
    assert moved > 1e-3          # the trained network does correct the stress
    ch.close()


def test_batched_learned_instances_equal_their_single_runs():
    """Three learned-wall-model channels of different sizes and Re_tau in one
    handle: every instance bit-identical to its own single run (the network
    is evaluated per 128-point tile of one instance, so the batch does not
    change any point's arithmetic; deterministic policy)."""
    src = C.c5_learned()
    batch = [C.smaller(src[0], 32, 32, 32), C.smaller(src[1], 48, 32, 32), C.smaller(src[2], 32, 40, 48)]
    theta = _theta()
    fields = [C.initial_fields(c) for c in batch]
    b = _channel(batch)
    for q, f in enumerate(fields):
        b.upload(*f, inst=q)
    b.mlp_set_params(theta)
    b.step(4)
    for q, c in enumerate(batch):
        s = _channel(c)
        s.upload(*fields[q])
        s.mlp_set_params(theta)
        s.step(4)
        ds, db = s.download(), b.download(inst=q)
        for f in ("U", "V", "W"):
            assert np.array_equal(ds[f], db[f]), (q, f)
        assert np.array_equal(s.wall_stress(), b.wall_stress(inst=q)), q
        s.close()
    b.close()


def test_tensor_core_wait_runs_out_then_next_launch_is_clean():
    """chl_tc_selftest variant 2 waits at most 64 polls on a completion
    barrier that no MMA commits to: CHL_E_TIMEOUT, TMEM freed.  The next
    launch (variant 0) computes the product correctly."""
    from channel_rl_gb300.host import ChlError, E_TIMEOUT, tc_selftest
    from oracle import mlp_ref as M
    rng = np.random.default_rng(3)
    A = M.bf16(rng.standard_normal((128, 64)).astype(np.float32))
    B = M.bf16(rng.standard_normal((64, 64)).astype(np.float32))
    bits = lambda a: (M.bf16(a).view(np.uint32) >> 16).astype(np.uint16)   # noqa: E731
    with pytest.raises(ChlError) as ei:
        tc_selftest(bits(A), bits(B), variant=2)
    assert ei.value.rc == E_TIMEOUT
    D = tc_selftest(bits(A), bits(B), variant=0)
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    assert np.abs(D - ref).max() <= 1e-5 * np.abs(ref).max()


def test_wall_model_wait_timeout_is_reported_and_cleared():
    """With the MMAs withheld every wall-model CTA's completion wait gives up
    after 16 polls: the stress stays the equilibrium one (the step equals the
    equilibrium model's bit for bit), chl_synchronize reports CHL_E_TIMEOUT
    once, and the next step with the hook off is clean and learned."""
    from channel_rl_gb300.host import ChlError, E_TIMEOUT
    ml = replace(C.smaller(C.c2_wm64(), 32, 32, 32), wall_model=C.WM_MLP)
    eq = replace(ml, wall_model=C.WM_EQLOG)
    U, V, W = C.initial_fields(ml)
    a, b = _channel(eq), _channel(ml)
    a.upload(U, V, W)
    b.upload(U, V, W)
    b.mlp_set_params(_theta())
    b.mlp_debug(record=True, withhold_polls=16)
    a.step(2)
    b.step(2)
    with pytest.raises(ChlError) as ei:
        b.synchronize()
    assert ei.value.rc == E_TIMEOUT
    b.synchronize()                              # reported once, then cleared
    assert np.isnan(b.mlp_record()[..., 4]).all()
    da, db = a.download(), b.download()
    for f in ("U", "V", "W"):
        assert np.array_equal(da[f], db[f]), f
    b.mlp_debug(record=True, withhold_polls=0)
    b.step(1)
    b.synchronize()
    r = b.mlp_record()
    assert np.isfinite(r[..., 4]).all()
    assert (r[..., 6] == 1.0).any()
    a.close()
    b.close()


def _exploration(rec, sigma):
    """(eps of the trusted points whose action is not clipped, per stage)."""
    out = []
    for s in range(3):
        r = rec[s]
        m = (r[..., 6] == 1.0) & (np.abs(r[..., 5]) < 0.5)
        out.append((r[..., 5][m].astype(np.float64) - r[..., 4][m]) / sigma)
    return out


def test_shared_exploration_is_one_draw_per_instance():
    """chl_mlp_set_exploration(1): every unclipped trusted wall point of an
    instance, every stage and every step, explores with the same eps (action
    minus mu, over sigma, to FP32 rounding); the two instances draw different
    eps; a new seed draws a new one.  With the default per-point draws the
    same points carry unit-variance noise."""
    src = C.c5_learned()
    batch = [C.smaller(src[0], 32, 32, 32), C.smaller(src[1], 48, 32, 32)]
    sigma = 0.1
    b = _channel(batch)
    for q, c in enumerate(batch):
        b.upload(*C.initial_fields(c), inst=q)
    b.mlp_set_params(_theta())
    b.mlp_debug(record=True)
    b.step(1)                                   # nu + nu_t of a finished stage
    b.mlp_configure(sigma=sigma, seed=21, train=True)
    b.mlp_set_exploration(True)
    draws = {}
    for seed in (21, 22):
        b.mlp_configure(sigma=sigma, seed=seed, train=True)
        for step in range(2):
            b.step(1)
            b.synchronize()
            for q in range(len(batch)):
                for s, e in enumerate(_exploration(b.mlp_record(inst=q), sigma)):
                    assert e.size > 100, (seed, step, q, s)
                    assert np.ptp(e) <= 1e-5, (seed, step, q, s, np.ptp(e))
                    draws.setdefault((seed, q), []).append(float(e.mean()))
    for key, d in draws.items():
        assert max(d) - min(d) <= 1e-5, key   # the same draw for every stage and step
    assert abs(draws[(21, 0)][0] - draws[(21, 1)][0]) > 1e-3
    assert abs(draws[(21, 0)][0] - draws[(22, 0)][0]) > 1e-3
    b.mlp_set_exploration(False)
    b.step(1)
    b.synchronize()
    e = _exploration(b.mlp_record(inst=0), sigma)[0]
    assert e.size > 100 and 0.8 < e.std() < 1.2
    for q in range(len(batch)):
        assert np.any(b.mlp_trace(q, zero=True) != 0)
    b.mlp_configure(sigma=0.0, seed=0, train=False)
    b.close()
