"""On-policy training of the learned wall model from the solver's own rollouts.

The reference trains its wall model with the external smarties engine:
states and rewards go out and wall-stress actions come back every 200
steps (smarties_stat.f90:24-260; reward 100 - 5000 |sqrt(tau_w) - u_tau|/u_tau).
Here the policy is the GPU network of chl_mlp.cu. All channels of a batch
share it, and every wall point of every stage is an action:

  a = clip(mu_theta(s) + sigma*eps, -0.5, 0.5),   tau_w = tau_eq exp(a),

with eps ~ N(0,1) drawn on the device. The kernels accumulate, per
instance, the policy-gradient trace sum_t eps/sigma * dmu/dtheta over the
rollout (REINFORCE with a Gaussian policy). The reward of an instance is the
negative L1 deviation of its plane-averaged mean profile from the log law
u+ = ln(y+)/kappa + B over the log region (30 <= y+, y <= 0.3 h), in units
of the bulk velocity. The update is Adam ascent on
sum_i (R_i - b) trace_i with a running-mean baseline b.

The equilibrium wall model (mu = 0) is both the fallback outside the trust
range (in the kernel) and the reference point of `evaluate`.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, replace

import numpy as np

from . import cases as C
from .host import MLP_NPARAM, Channel

KAPPA, B_LOG = C.KAPPA, C.B_LOG
H, NIN = 64, 4


def init_params(seed, out_scale=0.01):
    """Xavier-uniform weights from the seed, zero biases; the output layer is
    scaled down so that the untrained policy starts at the equilibrium model."""
    rng = np.random.default_rng(seed)

    def xa(fo, fi):
        lim = math.sqrt(6.0 / (fi + fo))
        return rng.uniform(-lim, lim, size=(fo, fi)).astype(np.float32)

    th = np.concatenate([xa(H, NIN).ravel(), np.zeros(H, np.float32), xa(H, H).ravel(),
                         np.zeros(H, np.float32), out_scale * xa(1, H).ravel(), np.zeros(1, np.float32)])
    assert th.size == MLP_NPARAM
    return th


def loglaw_rows(case):
    """Rows (Fortran j of U, 1-based) in the log region and their log-law velocity."""
    x, y, z = C.faces(case)
    yg = C.centres_y(y)
    ut = math.sqrt(case.dPdx)
    rows, target = [], []
    for j in range(1, yg.size - 1):          # interior centre rows (Fortran j = 2..nyg-1)
        d = 1.0 - abs(yg[j])
        yp = d * ut / case.nu
        if yp >= 30.0 and d <= 0.3:
            rows.append(j)
            target.append(ut * (math.log(yp) / KAPPA + B_LOG))
    return np.array(rows), np.array(target)


def profile_error(Umean, case):
    """L1 deviation of the mean profile from the log law (bulk-velocity units)."""
    rows, target = loglaw_rows(case)
    if rows.size == 0:
        return 0.0
    return float(np.mean(np.abs(Umean[rows] - target)))


@dataclass
class Adam:
    lr: float = 3e-3
    b1: float = 0.9
    b2: float = 0.999
    eps: float = 1e-8
    m: np.ndarray = field(default_factory=lambda: np.zeros(MLP_NPARAM))
    v: np.ndarray = field(default_factory=lambda: np.zeros(MLP_NPARAM))
    t: int = 0

    def ascend(self, theta, grad):
        self.t += 1
        self.m = self.b1 * self.m + (1 - self.b1) * grad
        self.v = self.b2 * self.v + (1 - self.b2) * grad * grad
        mh = self.m / (1 - self.b1 ** self.t)
        vh = self.v / (1 - self.b2 ** self.t)
        return (theta + self.lr * mh / (np.sqrt(vh) + self.eps)).astype(np.float32)


class Trainer:
    """Batched channels with the learned wall model and its REINFORCE loop."""

    def __init__(self, cases_, seed=0, sigma=0.1, lr=3e-3, spinup=200, shared_noise=False):
        self.cases = [replace(c, wall_model=C.WM_MLP) for c in cases_]
        self.ch = Channel(self.cases)
        self.sigma = sigma
        # shared_noise: one exploration draw per channel and rollout
        # (chl_mlp_set_exploration), so that the per-channel reward sees it
        self.shared_noise = shared_noise
        self.seed = seed
        self.theta = init_params(seed)
        self.opt = Adam(lr=lr)
        self.baseline = None
        self.history = []
        self.reset()
        self.ch.mlp_configure(sigma=0.0, seed=seed, train=False)
        self.ch.step(spinup)
        self.ch.synchronize()
        self.state0 = [self.ch.download(inst=q) for q in range(len(self.cases))]

    def reset(self):
        for q, c in enumerate(self.cases):
            self.ch.upload(*C.initial_fields(c), inst=q)
        self.ch.mlp_set_params(self.theta)

    def restore(self):
        """Back to the spun-up state (same start for every rollout)."""
        for q, s in enumerate(self.state0):
            self.ch.set_fields_ptr(*(np.asfortranarray(s[f]) for f in "UVW"), inst=q)
        self.ch.synchronize()

    def rollout(self, steps, chunks=4):
        """(profile error, mean wall stress) per instance: the mean profile
        and the plane-averaged wall stress sampled `chunks` times over the
        rollout and averaged."""
        acc = [np.zeros(c.ny) for c in self.cases]
        tau = np.zeros(len(self.cases))
        for _ in range(chunks):
            self.ch.step(max(1, steps // chunks))
            for q in range(len(self.cases)):
                st = self.ch.compute_statistics(q)
                acc[q] += st["Umean"]
                tau[q] += st["tau_wall"]
        err = np.array([profile_error(a / chunks, c) for a, c in zip(acc, self.cases)])
        return err, tau / chunks

    def rollout_reward(self, steps, chunks=4):
        """Mean profile error per instance, profiles averaged over the rollout."""
        return self.rollout(steps, chunks)[0]

    def update(self, steps=100, it=0):
        self.restore()
        self.ch.mlp_set_params(self.theta)
        self.ch.mlp_configure(sigma=self.sigma, seed=self.seed * 1000003 + it, train=True)
        self.ch.mlp_set_exploration(self.shared_noise)
        for q in range(len(self.cases)):
            self.ch.mlp_trace(q, zero=True)
        err = self.rollout_reward(steps)
        R = -err
        if self.baseline is None:
            self.baseline = R.copy()
        adv = R - self.baseline
        grad = np.zeros(MLP_NPARAM)
        for q in range(len(self.cases)):
            tr = self.ch.mlp_trace(q, zero=True).astype(np.float64)
            c = self.cases[q]
            n_eval = 3.0 * steps * 2 * c.Nx * c.Nz
            grad += adv[q] * tr / n_eval
        grad /= len(self.cases)
        self.theta = self.opt.ascend(self.theta, grad)
        self.baseline = 0.8 * self.baseline + 0.2 * R
        self.history.append(float(err.mean()))
        self.ch.mlp_configure(sigma=0.0, seed=0, train=False)
        self.ch.mlp_set_exploration(False)
        return float(err.mean())

    def evaluate(self, theta, steps=200, chunks=4):
        """(profile error, u_tau error) per instance of a deterministic policy
        from the spun-up state; theta=None is the equilibrium model (mu = 0).
        u_tau comes from the wall stress averaged over the rollout,
        u_tau = sqrt(2 <tau_w> / L_y) as statistics.f90:108-116 forms it."""
        self.restore()
        self.ch.mlp_set_params(np.zeros(MLP_NPARAM, np.float32) if theta is None else theta)
        self.ch.mlp_configure(sigma=0.0, seed=0, train=False)
        err, tau = self.rollout(steps, chunks)
        ut = []
        for q, c in enumerate(self.cases):
            u = math.sqrt(max(tau[q], 0.0) * 2.0 / 2.0)
            ut.append(abs(u - math.sqrt(c.dPdx)) / math.sqrt(c.dPdx))
        self.ch.mlp_set_params(self.theta)
        return err, np.array(ut)

    def close(self):
        self.ch.close()
