"""The multi-core C++ restatement (oracle/refcpu.cpp, the host-core baseline)
against the NumPy oracle: same step, same inputs, every physics switch."""
from dataclasses import replace

import numpy as np
import pytest

from channel_rl_gb300 import cases as C
from helpers import oracle_for, regions, rel

# Both restatements are FP64 with different summation orders (OpenMP plane
# sums, FFT factorisation); after a few steps they agree far below this.
REFCPU_RTOL = 1e-13

CASES = {
    "dsm_massflow": lambda: C.smaller(C.c1_small(), 16, 12, 16),
    "dsm_eqwm": lambda: C.smaller(C.c3_roofline(C.LES_DSM), 16, 12, 24),
    "smag_eqwm": lambda: C.smaller(C.c3_roofline(C.LES_SMAG), 24, 16, 16),
    "dsm_eqwm_massflow_ragged": lambda: C.smaller(C.c2_wm64(), 18, 10, 12),
    # the reference's RL cases: AMD, ghost rule 2, fixed dt (as rl_case)
    "amd_eqwm_rule2_fixed_dt": lambda: replace(C.smaller(C.rl_case(), 16, 10, 12), Dirichlet_nu_t=2),
    "amd_rule1_massflow": lambda: replace(C.smaller(C.c1_small(), 18, 12, 12), LES_model=C.LES_AMD),
    "vreman_eqwm_rule0": lambda: replace(C.smaller(C.c3_roofline(C.LES_DSM), 12, 14, 18),
                                         LES_model=C.LES_VREMAN, Dirichlet_nu_t=0),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_refcpu_matches_oracle(name):
    from oracle.refcpu import RefCPU
    case = CASES[name]()
    U, V, W = C.initial_fields(case)
    r = RefCPU(case)
    r.upload(U, V, W)
    o = oracle_for(case)
    o.set_fields(U, V, W)
    for _ in range(4):
        o.step()
    r.step(4)
    d = r.download()
    r.close()
    reg = regions(o.g)
    for f in "UVW":
        assert rel(d[f][reg[f]], getattr(o, f)[1:, 1:, 1:][reg[f]]) <= REFCPU_RTOL, f
    assert d["dt"] == pytest.approx(o.dt, rel=1e-14)


def test_refcpu_rejects_learned_wall_model():
    from oracle.refcpu import RefCPU
    case = replace(C.smaller(C.c1_small(), 16, 12, 16), wall_model=C.WM_MLP)
    with pytest.raises(ValueError):
        RefCPU(case)
