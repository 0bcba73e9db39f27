"""Wall agents of the reference's RL protocol on the GPU against the oracle:
states and rewards (smarties_stat.f90:38-176), the wall stress after the
agents act (:193-256), the step after it, and the protocol schedule."""
import numpy as np
import pytest

from channel_rl_gb300 import cases as C
from oracle.agents_ref import alpha_from_actions, observe
from tests.helpers import FIELD_RTOL, oracle_for, regions, rel

pytestmark = pytest.mark.gpu


def _shifted(case0):
    """The same channel on the reference's mesh convention, walls at y = 0
    and y = 2 (the agents' wall distance is the raw y coordinate)."""
    from dataclasses import replace
    x, y, z = C.faces(case0)
    return replace(case0, xf=tuple(x), yf=tuple(y + 1.0), zf=tuple(z)), C.initial_fields(case0)


def _pair(case0, alpha):
    from channel_rl_gb300.host import Channel
    case, (U, V, W) = _shifted(case0)
    o = oracle_for(case)
    o.set_fields(U, V, W)
    o.set_wall_stress(alpha)
    ch = Channel(case)
    ch.upload(U, V, W)
    full = np.zeros((case.nx, 2, case.nz + 1), order="F")
    full[1:-1, :, 1:-2] = alpha
    full[0], full[-1] = full[-2], full[1]
    full[:, :, 0], full[:, :, -2], full[:, :, -1] = full[:, :, -3], full[:, :, 1], full[:, :, 2]
    ch.set_wall_stress(full)
    return o, ch, case


def test_observe_act_and_step_match_oracle():
    case = C.wallmodelled("ag", 32, 24, 16, 2000.0, wall_model=C.WM_STRESS)
    rng = np.random.default_rng(4)
    alpha = case.dPdx * (1.0 + 0.2 * rng.standard_normal((case.Nx, 2, case.Nz)))
    o, ch, case = _pair(case, alpha)
    for _ in range(3):
        o.step()
    ch.step(3)
    n = 8
    y_ind = np.where(rng.random((2, n)) < 0.5, 3, 4)
    y_rand = rng.random((2, n))
    st, rw = ch.agent_observe(n, y_ind, y_rand)
    so, ro = observe(o, n, y_ind, y_rand, case.dPdx)
    assert np.isfinite(st).all() and np.isfinite(rw).all()
    for c in range(6):
        assert rel(st[:, :, c], so[:, :, c]) < 1e-12, c
    assert np.abs(rw - ro).max() < 1e-9 * np.abs(ro).max()
    act = rng.uniform(0.9, 1.1, (2, n))
    ch.agent_act(n, act)
    new = alpha_from_actions(o, n, act)
    got = ch.wall_stress()[1:-1, :, 1:-2]
    assert np.array_equal(got, np.transpose(new, (2, 0, 1)))
    o.set_wall_stress(np.transpose(new, (2, 0, 1)))
    o.step()
    ch.step(1)
    d = ch.download()
    reg = regions(o.g)
    for f in "UVW":
        assert rel(d[f][reg[f]], getattr(o, f)[1:, 1:, 1:][reg[f]]) < FIELD_RTOL, f
    ch.close()


def test_protocol_schedule():
    """The reference's schedule on a short run: first message at step 1000,
    then every 200 steps, the last one at nsteps; constant unit actions keep
    the wall stress at its initial random level."""
    from channel_rl_gb300.agents import WallAgentEnv
    from channel_rl_gb300.host import Channel
    case, fields = _shifted(C.wallmodelled("env", 32, 16, 16, 2000.0, wall_model=C.WM_STRESS))
    ch = Channel(case)
    ch.upload(*fields)
    env = WallAgentEnv(ch, case, nagents=8, seed=11)
    sent = []
    env.run(1401, lambda s, r: np.ones((2, 8)),
            on_send=lambda i, s, r, last: sent.append((i, r is None, last, np.isfinite(s).all())))
    assert [s[0] for s in sent] == [1000, 1200, 1400, 1401]
    assert sent[0][1] and not sent[1][1] and sent[-1][2] and all(s[3] for s in sent)
    assert env.decisions == 3
    a = ch.wall_stress()[1:-1, :, 1:-2]
    assert np.allclose(a, a[0, 0, 0], rtol=1e-14)
    ch.close()
