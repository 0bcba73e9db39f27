"""The bench configurations at their full sizes, tuned as the bench runs
them: 256x96x192 with the dynamic Smagorinsky model (the default line), with
static Smagorinsky and with AMD, and the reference's RL-case size
(128x40x64, AMD, ghost rule 2, fixed dt).  Ten steps against the C++
restatement of the reference step on the host cores, U, V and W within the
FP64 parity tolerance after every step, and the size-independent property
of the projection: max|div u| <= 1e-12 after every step."""
from dataclasses import replace

import numpy as np
import pytest

from channel_rl_gb300 import cases as C
from tests.helpers import FIELD_RTOL

pytestmark = pytest.mark.gpu

NSTEPS = 10

CASES = {
    "c3_dsm_256x96x192": lambda: C.c3_roofline(les=C.LES_DSM),
    "c3_smag_256x96x192": lambda: C.c3_roofline(les=C.LES_SMAG),
    "c3_amd_256x96x192": lambda: replace(C.c3_roofline(les=C.LES_DSM), LES_model=C.LES_AMD),
    "rl_case_128x40x64": lambda: C.rl_case(),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_full_size_ten_steps_against_host_restatement(name):
    from channel_rl_gb300.host import Channel
    from oracle.refcpu import RefCPU
    case = CASES[name]()
    U, V, W = C.initial_fields(case)
    ch = Channel(case)
    ch.upload(U, V, W)
    ch.autotune(reps=2)
    r = RefCPU(case)
    r.upload(U, V, W)
    worst = 0.0
    for step in range(1, NSTEPS + 1):
        ch.step(1)
        d = ch.download()
        assert ch.check_divergence()[1] <= 1e-12, step
        r.step(1)
        h = r.download()
        for f in "UVW":
            e = np.abs(d[f] - h[f]).max() / np.abs(h[f]).max()
            worst = max(worst, e)
            assert e < FIELD_RTOL, (name, step, f, e)
    print(f"{name}: {NSTEPS} steps, worst relative field error {worst:.2e}")
    ch.close()
    r.close()
