"""Known answers of the oracle's learned-wall-model stage (oracle/mlp_wm_ref.py)
in the channel, before it is used as the checker of the GPU's stage."""
from dataclasses import replace

import numpy as np

from channel_rl_gb300 import cases as C
from oracle import mlp_ref
from oracle import mlp_wm_ref
from tests.helpers import oracle_for


def _case():
    return replace(C.smaller(C.c2_wm64(), 16, 16, 16), wall_model=C.WM_MLP)


def test_zero_network_is_the_equilibrium_model():
    """mu = 0 gives a = 0 and tau_eq exp(0) = tau_eq: two steps bit for bit
    equal to the equilibrium wall model's."""
    ml = _case()
    eq = replace(ml, wall_model=C.WM_EQLOG)
    U, V, W = C.initial_fields(ml)
    a, b = oracle_for(eq), oracle_for(ml)
    a.set_fields(U, V, W)
    b.set_fields(U, V, W)
    for _ in range(2):
        a.step()
        b.step()
    for f in ("U", "V", "W"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f


def test_first_stage_is_untrusted_then_features_follow_their_formulas():
    """Before any wall-model pass nu + nu_t is zero, so f3 = ln(1e-300) lies
    outside the trust range and every point keeps tau_eq.  At the next stage
    f1 = ln(h Re_tau) exactly, f0 is the velocity at the third cell, f3 the
    face average of ln((nu + nu_t)/nu) from the previous stage."""
    case = _case()
    o = oracle_for(case)
    o.set_fields(*C.initial_fields(case))
    o.mlp_theta = mlp_ref.xavier_init(3)
    o.compute_dt()
    o.compute_time_step_RK3()
    g = o.g
    i0 = o.mlp_info[0]
    assert not i0["trusted"].any()
    assert np.all(i0["a"] == 0)
    i1 = o.mlp_info[1]
    hb = g.yg[4] - g.y[1]
    ht = g.y[g.ny] - g.yg[g.nyg - 3]
    assert np.all(i1["x"][:, 0, :, 1] == np.float32((np.log(hb * case.Retau) - 6.0) / 2.0))
    assert np.all(i1["x"][:, 1, :, 1] == np.float32((np.log(ht * case.Retau) - 6.0) / 2.0))
    assert i1["trusted"].mean() > 0.9           # a developed near-wall state is inside the range


def test_constant_action_scales_the_stress():
    """Given actions a, every trusted point's stress is tau_eq exp(a) and an
    untrusted point's is tau_eq."""
    case = _case()
    o = oracle_for(case)
    o.set_fields(*C.initial_fields(case))
    o.step()                                    # nu + nu_t of a finished stage
    o.dt = o.compute_dt()
    eq = o.compute_wall_stress_eqlog()
    act = np.full(eq.shape, 0.25, np.float32)
    alpha, info = mlp_wm_ref.wall_stress(o, eq, o.mlp_nutot, theta=None, actions=act)
    t = info["trusted"]
    assert t.any()
    assert np.array_equal(alpha[t], eq[t] * np.exp(0.25))
    assert np.array_equal(alpha[~t], eq[~t])


def test_network_actions_are_the_clipped_mu():
    """Without given actions, a = clip(mu, -0.5, 0.5) of the BF16 network
    on the features (a large output bias saturates mu at 0.5)."""
    case = _case()
    o = oracle_for(case)
    o.set_fields(*C.initial_fields(case))
    o.step()
    o.dt = o.compute_dt()
    theta = mlp_ref.xavier_init(5)
    theta[-1] = 40.0                            # b3: tanh(o) -> 1, mu -> 0.5
    eq = o.compute_wall_stress_eqlog()
    alpha, info = mlp_wm_ref.wall_stress(o, eq, o.mlp_nutot, theta=theta)
    t = info["trusted"]
    assert np.all(info["mu"] == np.float32(0.5))
    assert np.array_equal(alpha[t], eq[t] * np.exp(np.float64(np.float32(0.5))))
