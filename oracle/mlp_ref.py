"""CPU reference of the learned wall-model network — TEST INFRASTRUCTURE ONLY.

The reference's learned part is an external smarties policy fed with
per-agent states by send_recv_state_action (smarties_stat.f90:24-260); its
network is not in the reference, so this restates the network the build
defines (channel_rl_gb300/csrc/chl_mlp.cu), with the GPU's roundings:

  x  = normalised features (4)                           FP32
  h1 = tanh(W1 x + b1)            W1: 64x4  (BF16)        FP32 math, h1 rounded to BF16
  h2 = tanh(W2 h1 + b2)           W2: 64x64 (BF16)        BF16 x BF16 products, FP32 sums
  o  = w3 . h2 + b3               w3: 64    (BF16)        FP32
  mu = 0.5 tanh(o)                (log-scale correction in [-0.5, 0.5])
  a  = clip(mu + sigma*eps, -0.5, 0.5)
  tau_w = tau_eq * exp(a)

Policy-gradient trace of one evaluation, for upstream weights g_p (g_p =
eps_p / sigma for REINFORCE with Gaussian exploration):
  d_o = g * 0.5 (1 - tanh(o)^2);   d_h2 = d_o w3 (1 - h2^2)  (rounded to BF16)
  d_h1 = (d_h2 W2)(1 - h1^2)        (BF16 x BF16 products, FP32 sums)
  dW2 = sum_p d_h2 h1^T, dW1 = sum_p d_h1 x^T, db1 = sum d_h1, db2 = sum d_h2,
  dw3 = sum d_o h2, db3 = sum d_o.
Parameter vector order (FP32 master): W1 (64x4, row major), b1, W2 (64x64,
row major: W2[out, in]), b2, w3, b3 -> 64*4 + 64 + 64*64 + 64 + 64 + 1 = 4545.
"""
from __future__ import annotations

import numpy as np

H = 64
NIN = 4
NPARAM = H * NIN + H + H * H + H + H + 1


def bf16(a):
    """Round float32 to bfloat16 (round to nearest, ties to even), as float32."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rnd = ((u >> 16) & 1) + 0x7FFF
    r = ((u + rnd) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out).astype(np.float32)


def unpack(theta):
    t = np.asarray(theta, dtype=np.float32)
    o = 0
    W1 = t[o:o + H * NIN].reshape(H, NIN); o += H * NIN
    b1 = t[o:o + H]; o += H
    W2 = t[o:o + H * H].reshape(H, H); o += H * H
    b2 = t[o:o + H]; o += H
    w3 = t[o:o + H]; o += H
    b3 = t[o]
    return W1, b1, W2, b2, w3, b3


def xavier_init(seed):
    """Xavier-uniform weights, zero biases (FP32 master)."""
    rng = np.random.default_rng(seed)
    def xa(fo, fi):
        lim = np.sqrt(6.0 / (fi + fo))
        return rng.uniform(-lim, lim, size=(fo, fi)).astype(np.float32)
    return np.concatenate([xa(H, NIN).ravel(), np.zeros(H, np.float32), xa(H, H).ravel(),
                           np.zeros(H, np.float32), xa(1, H).ravel(), np.zeros(1, np.float32)])


def forward(theta, x):
    """x: (P, 4) float32 -> dict of activations (float32)."""
    W1, b1, W2, b2, w3, b3 = unpack(theta)
    W1, W2, w3 = bf16(W1), bf16(W2), bf16(w3)
    x = np.asarray(x, dtype=np.float32)
    z1 = x @ W1.T.astype(np.float64)
    h1 = bf16(np.tanh((z1 + b1).astype(np.float32)))
    z2 = (h1.astype(np.float64) @ W2.T.astype(np.float64)).astype(np.float32) + b2
    h2 = np.tanh(z2).astype(np.float32)
    o = (h2.astype(np.float64) @ w3.astype(np.float64)).astype(np.float32) + b3
    mu = (0.5 * np.tanh(o)).astype(np.float32)
    return {"x": x, "h1": h1, "h2": h2, "o": o, "mu": mu, "W2": W2, "w3": w3}


def trace_grad(theta, x, g):
    """Sum over points of g_p * d mu_p / d theta (4545 float64)."""
    f = forward(theta, x)
    h1, h2, o = f["h1"], f["h2"], f["o"]
    W2, w3 = f["W2"], f["w3"]
    g = np.asarray(g, dtype=np.float64)
    d_o = g * 0.5 * (1.0 - np.tanh(o.astype(np.float64)) ** 2)
    d_h2 = bf16((d_o[:, None] * w3[None, :] * (1.0 - h2.astype(np.float64) ** 2)).astype(np.float32))
    d_h1 = (d_h2.astype(np.float64) @ W2.astype(np.float64)) * (1.0 - h1.astype(np.float64) ** 2)
    dW1 = d_h1.T @ f["x"].astype(np.float64)
    db1 = d_h1.sum(0)
    dW2 = d_h2.astype(np.float64).T @ h1.astype(np.float64)
    db2 = d_h2.astype(np.float64).sum(0)
    dw3 = (d_o[:, None] * h2.astype(np.float64)).sum(0)
    db3 = d_o.sum()
    return np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dw3, [db3]])


def trace_grad_fd(theta, x, g, eps=1e-3):
    """Finite-difference check of trace_grad in float64 without BF16 rounding."""
    theta = np.asarray(theta, dtype=np.float64)

    def mu_sum(t):
        W1, b1, W2, b2, w3, b3 = unpack_f64(t)
        h1 = np.tanh(x @ W1.T + b1)
        h2 = np.tanh(h1 @ W2.T + b2)
        return float((g * 0.5 * np.tanh(h2 @ w3 + b3)).sum())

    out = np.zeros_like(theta)
    for i in range(theta.size):
        tp, tm = theta.copy(), theta.copy()
        tp[i] += eps
        tm[i] -= eps
        out[i] = (mu_sum(tp) - mu_sum(tm)) / (2 * eps)
    return out


def trace_grad_f64(theta, x, g):
    """trace_grad in float64 without BF16 rounding (for the FD check)."""
    W1, b1, W2, b2, w3, b3 = unpack_f64(theta)
    h1 = np.tanh(x @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    o = h2 @ w3 + b3
    d_o = g * 0.5 * (1.0 - np.tanh(o) ** 2)
    d_h2 = d_o[:, None] * w3[None, :] * (1.0 - h2 ** 2)
    d_h1 = (d_h2 @ W2) * (1.0 - h1 ** 2)
    return np.concatenate([(d_h1.T @ x).ravel(), d_h1.sum(0), (d_h2.T @ h1).ravel(), d_h2.sum(0),
                           (d_o[:, None] * h2).sum(0), [d_o.sum()]])


def unpack_f64(theta):
    t = np.asarray(theta, dtype=np.float64)
    o = 0
    W1 = t[o:o + H * NIN].reshape(H, NIN); o += H * NIN
    b1 = t[o:o + H]; o += H
    W2 = t[o:o + H * H].reshape(H, H); o += H * H
    b2 = t[o:o + H]; o += H
    w3 = t[o:o + H]; o += H
    return W1, b1, W2, b2, w3, t[o]
