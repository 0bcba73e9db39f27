"""Train the learned wall model on the GPU from the solver's own rollouts.

    python -m channel_rl_gb300.train --iters 120 --out mlp_wm.npy --report report.json

The batch is the 16-channel learned-wall-model ensemble (Re_tau 2000, 5200,
10000; grids 48^3 .. 96x64x96), all channels advancing in one launch per
kernel with the network on the tensor cores.  Every iteration is one
on-policy rollout from the same spun-up state with Gaussian exploration
(REINFORCE, rl.Trainer.update).  Every `--eval-every` iterations the
deterministic policy is evaluated against the equilibrium wall model from
the same state; the parameters with the lowest mean profile error among
those that do not raise the u_tau error are kept (`--keep reward` drops
the u_tau condition).

The reward-only network shipped as data/mlp_wm_profile.npy came from

    python -m channel_rl_gb300.train --shared-noise --keep reward --iters 40 --steps 400 \
        --eval-steps 400 --out mlp_wm_profile.npy --report mlp_wm_profile_report.json
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import cases as C
from .rl import Trainer


def summarise(cases_, eq, ml):
    """Per-Re_tau means of (profile error, u_tau error), equilibrium vs learned."""
    out = {}
    for rt in sorted({c.Retau for c in cases_}):
        idx = [q for q, c in enumerate(cases_) if c.Retau == rt]
        out[f"{rt:g}"] = {"equilibrium_profile_err": float(np.mean(eq[0][idx])),
                          "learned_profile_err": float(np.mean(ml[0][idx])),
                          "equilibrium_utau_err": float(np.mean(eq[1][idx])),
                          "learned_utau_err": float(np.mean(ml[1][idx]))}
    return out


def train(cases_, iters=120, steps=60, spinup=300, sigma=0.1, lr=3e-3, seed=7, eval_steps=120,
          eval_every=10, shared_noise=False, keep="gated", log=print):
    tr = Trainer(cases_, seed=seed, sigma=sigma, lr=lr, spinup=spinup, shared_noise=shared_noise)
    eq = tr.evaluate(None, steps=eval_steps)
    best = (float(eq[0].mean()), tr.theta.copy(), eq, 0)
    log(f"equilibrium: profile err {eq[0].mean():.5f}, u_tau err {eq[1].mean():.5f}")
    t0 = time.perf_counter()
    for it in range(iters):
        tr.update(steps=steps, it=it)
        if (it + 1) % eval_every == 0 or it + 1 == iters:
            ml = tr.evaluate(tr.theta, steps=eval_steps)
            log(f"iter {it + 1:4d}  rollout err {tr.history[-1]:.5f}  eval profile err {ml[0].mean():.5f}"
                f"  u_tau err {ml[1].mean():.5f}  ({time.perf_counter() - t0:.0f} s)")
            if ml[0].mean() < best[0] and (keep == "reward" or ml[1].mean() <= eq[1].mean()):
                best = (float(ml[0].mean()), tr.theta.copy(), ml, it + 1)
    theta, ml, it_best = best[1], best[2], best[3]
    report = {"instances": [c.name for c in cases_], "iterations": iters, "rollout_steps": steps,
              "spinup_steps": spinup, "sigma": sigma, "lr": lr, "seed": seed, "eval_steps": eval_steps,
              "shared_noise": shared_noise, "keep": keep,
              "best_iteration": it_best, "train_seconds": time.perf_counter() - t0,
              "equilibrium": {"profile_err": eq[0].tolist(), "utau_err": eq[1].tolist()},
              "learned": {"profile_err": ml[0].tolist(), "utau_err": ml[1].tolist()},
              "by_retau": summarise(cases_, eq, ml), "history": tr.history}
    tr.close()
    return theta, report


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--iters", type=int, default=120)
    ap.add_argument("--steps", type=int, default=60, help="RK3 steps per rollout")
    ap.add_argument("--spinup", type=int, default=300)
    ap.add_argument("--sigma", type=float, default=0.1)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--eval-steps", type=int, default=120)
    ap.add_argument("--eval-every", type=int, default=10)
    ap.add_argument("--shared-noise", action="store_true",
                    help="one exploration draw per channel and rollout instead of one per wall point and step")
    ap.add_argument("--keep", choices=("gated", "reward"), default="gated",
                    help="gated: lowest profile error among parameters that do not raise the u_tau error; "
                         "reward: lowest profile error")
    ap.add_argument("--out", default=None, help="where to write the kept parameters (.npy, float32)")
    ap.add_argument("--report", default=None, help="where to write the JSON report")
    args = ap.parse_args()
    theta, report = train(C.c5_learned(), iters=args.iters, steps=args.steps, spinup=args.spinup,
                          sigma=args.sigma, lr=args.lr, seed=args.seed, eval_steps=args.eval_steps,
                          eval_every=args.eval_every, shared_noise=args.shared_noise,
                          keep=args.keep)
    if args.out:
        np.save(args.out, theta.astype(np.float32))
    if args.report:
        with open(args.report, "w") as f:
            json.dump(report, f, indent=1)
    print(json.dumps(report["by_retau"], indent=1))


if __name__ == "__main__":
    main()
