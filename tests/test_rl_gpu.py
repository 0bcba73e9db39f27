"""On-policy training of the learned wall model, and what it gains over the
equilibrium model it corrects (same start, same horizon, deterministic policy)."""
import json
import os

import numpy as np
import pytest

from channel_rl_gb300 import cases as C

pytestmark = pytest.mark.gpu


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
