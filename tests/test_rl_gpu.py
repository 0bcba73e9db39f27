"""On-policy training of the learned wall model, and what it gains over the
equilibrium model it corrects (same start, same horizon, deterministic policy)."""
import json
import os

import numpy as np
import pytest

from channel_rl_gb300 import cases as C

pytestmark = pytest.mark.gpu

DATA = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "channel_rl_gb300", "data")


def _checkpoint(name):
    return np.load(os.path.join(DATA, name)).astype(np.float32)


def _held_out():
    """Re_tau 3000 and 7000 (training used 2000, 5200, 10000), other grids and seeds."""
    spec = [(64, 48, 64, 3000.0), (96, 64, 96, 3000.0), (64, 48, 64, 7000.0), (96, 64, 96, 7000.0)]
    return [C.wallmodelled(f"held_out_{m}", Nx, Ny, Nz, rt, seed=9000 + 37 * m, wall_model=C.WM_MLP)
            for m, (Nx, Ny, Nz, rt) in enumerate(spec)]


def test_training_improves_on_equilibrium_model():
    from channel_rl_gb300.rl import Trainer
    batch = [C.wallmodelled(f"t{m}", 32, 32, 32, retau, seed=100 + m)
             for m, retau in enumerate((2000.0, 5200.0, 10000.0, 3000.0))]
    tr = Trainer(batch, seed=3, sigma=0.1, lr=3e-3, spinup=150)
    eq_err, eq_ut = tr.evaluate(None, steps=120)
    first = tr.update(steps=60, it=0)
    for it in range(1, 16):
        tr.update(steps=60, it=it)
    ml_err, ml_ut = tr.evaluate(tr.theta, steps=120)
    report = {"equilibrium_profile_err": eq_err.tolist(), "trained_profile_err": ml_err.tolist(),
              "equilibrium_utau_err": eq_ut.tolist(), "trained_utau_err": ml_ut.tolist(),
              "training_history": tr.history}
    print(json.dumps(report))
    out = os.environ.get("CHL_RL_REPORT")
    if out:
        with open(out, "w") as f:
            json.dump(report, f, indent=1)
    tr.close()
    assert np.all(np.isfinite(ml_err)) and np.all(np.isfinite(ml_ut))
    # the trained correction keeps the mean profile of the model it corrects
    # and lowers the u_tau error (time-averaged wall stress vs the target)
    assert ml_err.mean() <= 1.001 * eq_err.mean()
    assert ml_ut.mean() <= 0.95 * eq_ut.mean()
    assert ml_ut.max() <= 0.02


def test_shipped_checkpoint_beats_equilibrium_model():
    """The parameters trained on the 16-channel learned-wall-model batch
    (channel_rl_gb300/data/mlp_wm.npy, Re_tau 2000/5200/10000) against the
    equilibrium model, same spun-up start, deterministic policy."""
    from channel_rl_gb300.rl import Trainer
    path = os.path.join(os.path.dirname(__file__), "..", "channel_rl_gb300", "data", "mlp_wm.npy")
    theta = np.load(path).astype(np.float32)
    tr = Trainer(C.c5_learned(), seed=7, spinup=300)
    eq_err, eq_ut = tr.evaluate(None, steps=120)
    ml_err, ml_ut = tr.evaluate(theta, steps=120)
    tr.close()
    print(json.dumps({"equilibrium_utau_err": float(eq_ut.mean()), "learned_utau_err": float(ml_ut.mean()),
                      "equilibrium_profile_err": float(eq_err.mean()), "learned_profile_err": float(ml_err.mean())}))
    assert ml_err.mean() <= 1.001 * eq_err.mean()
    assert ml_ut.mean() <= 0.9 * eq_ut.mean()
    assert ml_ut.max() <= 0.02                   # the 2% u_tau gate at every Re_tau


def test_shipped_checkpoint_held_out():
    """The shipped network on channels it never saw: Re_tau 3000 and 7000
    (training used 2000, 5200, 10000), other grids and seeds.  Spin-up of
    1000 steps with the equilibrium model (the reference's agents first act
    at step 1000), then the deterministic policy with statistics every 200
    steps (its decision interval), over 1200 steps and over 7600 steps (3-4
    near-wall response times h/u_tau).

    Measured: the profile error (the reward) is lower on every held-out
    channel; the u_tau error is not lower (0.44 % -> 0.51 % mean at 1200
    steps).  Asserted: profile error lower on every channel at both
    horizons, u_tau within the 2 % gate at 1200 steps for both models, and
    the learned u_tau error at most 0.2 points above the equilibrium
    model's."""
    from channel_rl_gb300.rl import Trainer
    theta = _checkpoint("mlp_wm.npy")
    tr = Trainer(_held_out(), seed=11, spinup=1000)
    res = {}
    for steps in (1200, 7600):
        eq_err, eq_ut = tr.evaluate(None, steps=steps, chunks=steps // 200)
        ml_err, ml_ut = tr.evaluate(theta, steps=steps, chunks=steps // 200)
        res[steps] = (eq_err, eq_ut, ml_err, ml_ut)
        print(json.dumps({"steps": steps, "equilibrium_profile_err": eq_err.tolist(),
                          "learned_profile_err": ml_err.tolist(), "equilibrium_utau_err": eq_ut.tolist(),
                          "learned_utau_err": ml_ut.tolist()}))
    tr.close()
    for steps, (eq_err, eq_ut, ml_err, ml_ut) in res.items():
        assert np.all(ml_err < eq_err), steps
        assert ml_ut.mean() <= eq_ut.mean() + 0.002, steps
    eq_err, eq_ut, ml_err, ml_ut = res[1200]
    assert eq_ut.max() <= 0.02 and ml_ut.max() <= 0.02


def test_reward_checkpoint_held_out():
    """The reward-only network (data/mlp_wm_profile.npy: shared exploration,
    parameters kept on the profile error alone) on the held-out channels,
    same protocol as above over 1200 steps.

    Measured: profile error 0.00831 -> 0.00664 (-20 %), u_tau error 0.44 % ->
    22 %.  Asserted: the profile error (the reward) at least 10 % lower on
    average and lower on every channel; and the price, a u_tau error outside
    the 2 % gate, which is why this network is not the default."""
    from channel_rl_gb300.rl import Trainer
    theta = _checkpoint("mlp_wm_profile.npy")
    tr = Trainer(_held_out(), seed=11, spinup=1000)
    eq_err, eq_ut = tr.evaluate(None, steps=1200, chunks=6)
    ml_err, ml_ut = tr.evaluate(theta, steps=1200, chunks=6)
    tr.close()
    print(json.dumps({"equilibrium_profile_err": eq_err.tolist(), "reward_profile_err": ml_err.tolist(),
                      "equilibrium_utau_err": eq_ut.tolist(), "reward_utau_err": ml_ut.tolist()}))
    assert np.all(ml_err < eq_err)
    assert ml_err.mean() <= 0.9 * eq_err.mean()
    assert eq_ut.max() <= 0.02 and ml_ut.mean() > 0.02
