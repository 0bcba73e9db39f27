"""Regenerate tests/golden/golden.npz from the oracle.

Two tiny seeded channels (cases.c1_small and cases.c2_wm64 physics on
16x12x16 / 16x16x16 grids) are advanced three solver steps (compute_dt +
compute_time_step_RK3); after each step the script stores U, V, W and the
actual pressure P at 256 fixed sample positions per field, plus each
field's sum and sum of squares over the unique points, and dt.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from channel_rl_gb300 import cases as C            # noqa: E402
from tests.helpers import oracle_for, regions      # noqa: E402

NSTEP = 3
NSAMPLE = 256


def golden_cases():
    return {"c1": C.smaller(C.c1_small(), 16, 12, 16),
            "c2": C.smaller(C.c2_wm64(), 16, 16, 16)}


def sample_positions(shape, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.integers(0, n, NSAMPLE) for n in shape], axis=1)


def summarise(fields, g):
    reg = regions(g)
    out = {}
    for name, arr in fields.items():
        r = reg["C" if name == "P" else name]
        a = arr[r]
        pos = sample_positions(a.shape, ord(name[0]))
        out[name + "_samples"] = a[tuple(pos.T)]
        out[name + "_sum"] = np.array([a.sum(), (a * a).sum()])
    return out


def main():
    data = {}
    for tag, case in golden_cases().items():
        o = oracle_for(case)
        o.set_fields(*C.initial_fields(case))
        for s in range(1, NSTEP + 1):
            o.step()
            P = o.compute_pressure()
            f = {"U": o.U[1:, 1:, 1:], "V": o.V[1:, 1:, 1:], "W": o.W[1:, 1:, 1:], "P": P[1:, 1:, 1:]}
            for k, v in summarise(f, o.g).items():
                data[f"{tag}_s{s}_{k}"] = v
            data[f"{tag}_s{s}_dt"] = np.array([o.dt])
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz")
    np.savez(out, **data)
    print(out, len(data), "arrays")


if __name__ == "__main__":
    main()
