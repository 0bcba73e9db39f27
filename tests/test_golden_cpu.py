"""The oracle reproduces its frozen golden fixtures (tests/golden/golden.npz,
written by tests/golden/make_golden.py): guards the checker against drift."""
import os

import numpy as np
import pytest

from channel_rl_gb300 import cases as C
from tests.golden.make_golden import NSTEP, golden_cases, summarise
from tests.helpers import oracle_for

GOLD = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.npz"))


@pytest.mark.parametrize("tag", ["c1", "c2"])
def test_oracle_reproduces_golden(tag):
    case = golden_cases()[tag]
    o = oracle_for(case)
    o.set_fields(*C.initial_fields(case))
    for s in range(1, NSTEP + 1):
        o.step()
        P = o.compute_pressure()
        f = {"U": o.U[1:, 1:, 1:], "V": o.V[1:, 1:, 1:], "W": o.W[1:, 1:, 1:], "P": P[1:, 1:, 1:]}
        got = summarise(f, o.g)
        for k, v in got.items():
            ref = GOLD[f"{tag}_s{s}_{k}"]
            scale = np.abs(ref).max()
            assert np.abs(v - ref).max() <= 1e-12 * scale, (tag, s, k)
        assert GOLD[f"{tag}_s{s}_dt"][0] == o.dt
