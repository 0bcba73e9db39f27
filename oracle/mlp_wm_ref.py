"""CPU restatement of the learned wall model's stage in the channel — TEST
INFRASTRUCTURE ONLY (only ``tests/`` import it, through oracle/channel_ref.py).

The reference's counterpart is the smarties policy: send_recv_state_action
assembles per-agent states from the near-wall flow (smarties_stat.f90:60-176)
and turns the returned actions into the wall stress alpha_x
(smarties_stat.f90:193-256).  The network and its coupling are the build's
own design (channel_rl_gb300/csrc/chl_mlp.cu: k_mlp); this module restates
that coupling statement by statement in the oracle's Fortran index
convention, so that the GPU's stage can be checked point by point:

Per U wall point (face i = a+2, centre k = c+2, wall w; a in [0,Nx), c in
[0,Nz)), with j = 4 at the bottom wall and nyg-3 at the top (the third
off-wall cell, the matching height of the equilibrium model) and
h = yg(4) - y(1) or y(ny) - yg(nyg-3):

  tau_eq  = the equilibrium log-law stress of this stage (alpha_eq)
  f0      = U(i, j, k)                                   (U_b = 1)
  f1      = ln(h Re_tau)
  dpdx    = (p(i+1, j, k) - p(i, j, k)) / (xg(i+1) - xg(i)) / dt,
            p the pseudo-pressure of the previous projection (0 if dt <= 0)
  f2      = clip(dpdx h / |tau_eq|, -10, 10)               (0 if tau_eq = 0)
  f3      = ln(max(nut_f / nu, 1e-300)),  nut_f = (n(i, j, k) + n(i+1, j, k)) / 2,
            n = nu + nu_t as left by the previous stage's wall-model pass
  x       = float32(f0 - 1, (f1 - 6)/2, f2/5, f3/3 - 1)
  trusted = 0.05 <= f0 <= 3, 2 <= f1 <= 11, 0 <= f3 <= 8, tau_eq != 0
  mu      = network(x)                                    (oracle/mlp_ref.py)
  a       = clip(mu + sigma eps, -0.5, 0.5)  (float32; eps: the GPU's counter noise)
  alpha   = tau_eq exp(a) where trusted, else tau_eq.

The exploration noise eps is not restated (its draw uses the GPU's own
transcendental functions); with sigma > 0, or to take the network's BF16
rounding out of a field comparison, a caller supplies the actions.
"""
from __future__ import annotations

import numpy as np

from . import mlp_ref


def features(o, alpha_eq, nutot):
    """Features of every wall point of oracle `o` for the current velocity.

    alpha_eq: (Nx, 2, Nz) equilibrium stress of this stage.  nutot: the
    nu + nu_t field (Fortran-padded like o.nu_t) left by the previous stage.
    Returns x (Nx, 2, Nz, 4) float32 and trusted (Nx, 2, Nz) bool.
    """
    g, p = o.g, o.p
    nx, nyg, nzg = g.nx, g.nyg, g.nzg
    nu = p.nu
    rdxf = 1.0 / (g.xg[3:nx + 1] - g.xg[2:nx])               # 1/(xg(i+1) - xg(i)), i = 2..nx-1
    x = np.zeros((g.Nx, 2, g.Nz, 4), np.float32)
    trusted = np.zeros((g.Nx, 2, g.Nz), bool)
    for w, (j, h) in enumerate(((4, g.yg[4] - g.y[1]), (nyg - 3, g.y[g.ny] - g.yg[nyg - 3]))):
        u = o.U[2:nx, j, 2:nzg - 1]
        taueq = alpha_eq[:, w, :]
        ap = np.abs(taueq)
        p0 = o.rhs_p[2:nx, j, 2:nzg - 1]
        p1 = np.roll(p0, -1, axis=0)                          # i + 1, periodic
        if o.dt > 0.0:
            dpdx = (p1 - p0) * rdxf[:, None] / o.dt
        else:
            dpdx = np.zeros_like(p0)
        with np.errstate(divide="ignore", invalid="ignore"):
            f2 = np.where(ap > 0.0, dpdx * h / np.where(ap > 0.0, ap, 1.0), 0.0)
        f2 = np.minimum(10.0, np.maximum(-10.0, f2))
        n0 = nutot[2:nx, j, 2:nzg - 1]
        ntf = 0.5 * (n0 + np.roll(n0, -1, axis=0))
        f0 = u
        f1 = np.log(h * p.Re_tau)
        with np.errstate(divide="ignore"):
            f3 = np.log(np.maximum(ntf / nu, 1e-300))
        trusted[:, w, :] = ((f0 >= 0.05) & (f0 <= 3.0) & (f1 >= 2.0) & (f1 <= 11.0)
                            & (f3 >= 0.0) & (f3 <= 8.0) & (ap > 0.0))
        x[:, w, :, 0] = (f0 - 1.0).astype(np.float32)
        x[:, w, :, 1] = np.float32((f1 - 6.0) / 2.0)
        x[:, w, :, 2] = (f2 / 5.0).astype(np.float32)
        x[:, w, :, 3] = (f3 / 3.0 - 1.0).astype(np.float32)
    return x, trusted


def wall_stress(o, alpha_eq, nutot, theta=None, actions=None):
    """The learned stress of every wall point.

    theta: network parameters (4545 float32; None is the zero network).
    actions: (Nx, 2, Nz) float32 actions a to apply in place of
    clip(mu, -0.5, 0.5) (deterministic policy), e.g. the GPU's own.
    Returns (alpha (Nx, 2, Nz) float64, info dict with x, trusted, mu, a).
    """
    x, trusted = features(o, alpha_eq, nutot)
    if theta is None:
        mu = np.zeros(trusted.shape, np.float32)
    else:
        mu = mlp_ref.forward(theta, x.reshape(-1, 4))["mu"].reshape(trusted.shape)
    a = np.clip(mu, np.float32(-0.5), np.float32(0.5)).astype(np.float32) if actions is None \
        else np.asarray(actions, np.float32)
    a = np.where(trusted, a, np.float32(0.0)).astype(np.float32)
    alpha = np.where(trusted, alpha_eq * np.exp(a.astype(np.float64)), alpha_eq)
    return alpha, {"x": x, "trusted": trusted, "mu": mu, "a": a}
