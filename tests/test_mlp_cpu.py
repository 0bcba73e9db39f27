"""CPU checks of the learned wall-model reference network (oracle/mlp_ref.py)."""
import numpy as np
import torch

from oracle import mlp_ref as M


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(0)
    a = (rng.standard_normal(10000) * 10.0 ** rng.uniform(-5, 5, 10000)).astype(np.float32)
    ref = torch.from_numpy(a).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(M.bf16(a), ref)


def test_trace_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    theta = M.xavier_init(3).astype(np.float64)
    theta[M.H * M.NIN:M.H * M.NIN + M.H] = rng.standard_normal(M.H) * 0.1
    x = rng.standard_normal((7, 4))
    g = rng.standard_normal(7)
    ga = M.trace_grad_f64(theta, x, g)
    idx = rng.choice(theta.size, 60, replace=False)
    fd = M.trace_grad_fd(theta, x, g, eps=1e-5)
    assert np.abs(ga[idx] - fd[idx]).max() < 1e-7
    assert np.abs(ga - fd).max() < 1e-7


def test_bf16_network_close_to_exact():
    rng = np.random.default_rng(2)
    theta = M.xavier_init(5)
    x = rng.standard_normal((512, 4)).astype(np.float32)
    g = rng.standard_normal(512).astype(np.float32)
    mu = M.forward(theta, x)["mu"]
    W1, b1, W2, b2, w3, b3 = M.unpack_f64(theta)
    mu64 = 0.5 * np.tanh(np.tanh(np.tanh(x @ W1.T + b1) @ W2.T + b2) @ w3 + b3)
    assert np.abs(mu - mu64).max() < 2e-2
    t = M.trace_grad(theta, x, g)
    t64 = M.trace_grad_f64(theta, x, g)
    assert np.linalg.norm(t - t64) / np.linalg.norm(t64) < 2e-2
