"""The bench configurations at their full sizes, tuned as the bench runs
them: 256x96x192 with the dynamic Smagorinsky model (the default line) and
with AMD, and the reference's RL-case size (128x40x64, AMD, ghost rule 2,
fixed dt).  Two steps against the C++ restatement of the reference step on
the host cores, at the FP64 parity tolerance, and the size-independent
property of the projection: max|div u| <= 1e-12."""
from dataclasses import replace

import numpy as np
import pytest

from channel_rl_gb300 import cases as C
from tests.helpers import FIELD_RTOL

pytestmark = pytest.mark.gpu

CASES = {
    "c3_dsm_256x96x192": lambda: C.c3_roofline(les=C.LES_DSM),
    "c3_amd_256x96x192": lambda: replace(C.c3_roofline(les=C.LES_DSM), LES_model=C.LES_AMD),
    "rl_case_128x40x64": lambda: C.rl_case(),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_full_size_two_steps_against_host_restatement(name):
    from channel_rl_gb300.host import Channel
    from oracle.refcpu import RefCPU
    case = CASES[name]()
    U, V, W = C.initial_fields(case)
    ch = Channel(case)
    ch.upload(U, V, W)
    ch.autotune(reps=2)
    ch.step(2)
    d = ch.download()
    assert ch.check_divergence()[1] <= 1e-12
    ch.close()
    r = RefCPU(case)
    r.upload(U, V, W)
    r.step(2)
    h = r.download()
    r.close()
    for f in "UVW":
        e = np.abs(d[f] - h[f]).max() / np.abs(h[f]).max()
        assert e < FIELD_RTOL, (name, f, e)
