"""Wall agents of the reference's RL protocol (smarties_stat.f90:24-260):
the oracle's action-to-wall-stress map and the reward shaping, on CPU."""
import numpy as np

from channel_rl_gb300 import cases as C
from oracle.agents_ref import alpha_from_actions
from tests.helpers import oracle_for


def _oracle_with_alpha(value, Nx=32, Nz=12):
    case = C.wallmodelled("a", Nx, 16, Nz, 2000.0, wall_model=C.WM_STRESS)
    o = oracle_for(case)
    o.set_wall_stress(np.full((case.Nx, 2, case.Nz), value))
    return o, case


def test_unit_actions_keep_a_uniform_wall_stress():
    o, case = _oracle_with_alpha(3.7e-3)
    new = alpha_from_actions(o, 8, np.ones((2, 8)))
    assert np.abs(new / 3.7e-3 - 1.0).max() <= 4e-16


def test_actions_interpolate_linearly_between_agents():
    o, case = _oracle_with_alpha(1.0)
    n, nxa = 8, case.Nx // 8
    act = np.vstack([np.linspace(0.9, 1.1, n), np.full(n, 1.05)])
    new = alpha_from_actions(o, n, act)
    for w in range(2):
        for na in range(n):
            a0, a1 = act[w, na], act[w, (na + 1) % n]      # the last agent leans on the first
            for j in range(nxa):
                expect = a0 + (a1 - a0) * j / nxa
                assert np.allclose(new[w, :, na * nxa + j], expect, rtol=1e-15, atol=0)


def test_reward_shaping():
    from channel_rl_gb300.agents import WallAgentEnv

    class _Ch:
        pass
    env = WallAgentEnv.__new__(WallAgentEnv)
    env.rewards_old = np.array([[10.0, -5.0], [0.0, 2.0]])
    r = np.array([[12.0, -7.0], [-1.0, 3.0]])
    # r - r_old, plus r where r > 0 (smarties_stat.f90:205-209)
    assert np.array_equal(env.shaped_reward(r), np.array([[14.0, -2.0], [-1.0, 4.0]]))
