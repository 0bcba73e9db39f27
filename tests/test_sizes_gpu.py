"""Grid sizes at the edges of what the solver accepts: the smallest and
ragged FFT lengths (2^a 3^b, odd wall-normal counts) against the oracle, and
long x and z lines (where the z transform stages fewer columns per block)
against the C++ restatement."""
from dataclasses import replace

import numpy as np
import pytest

from channel_rl_gb300 import cases as C
from tests.helpers import FIELD_RTOL, oracle_for, regions, rel

pytestmark = pytest.mark.gpu

RAGGED = {
    "6x9x12_dsm_massflow": C.smaller(C.c1_small(), 6, 9, 12),
    "18x13x6_smag_eqwm": C.smaller(C.c3_roofline(les=C.LES_SMAG), 18, 13, 6),
    "54x10x36_amd_eqwm_rule2": replace(C.smaller(C.c3_roofline(les=C.LES_DSM), 54, 10, 36),
                                       LES_model=C.LES_AMD, Dirichlet_nu_t=2),
    "4x8x4_vreman_eqwm": replace(C.smaller(C.c2_wm64(), 4, 8, 4), LES_model=C.LES_VREMAN),
}


@pytest.mark.parametrize("name", sorted(RAGGED))
def test_ragged_grids_match_oracle(name):
    from channel_rl_gb300.host import Channel
    case = RAGGED[name]
    U, V, W = C.initial_fields(case)
    o = oracle_for(case)
    o.set_fields(U, V, W)
    ch = Channel(case)
    ch.upload(U, V, W)
    for _ in range(5):
        o.step()
    ch.step(5)
    d = ch.download()
    reg = regions(o.g)
    for f in "UVW":
        assert rel(d[f][reg[f]], getattr(o, f)[1:, 1:, 1:][reg[f]]) < FIELD_RTOL, f
    assert ch.check_divergence()[1] < 1e-12
    ch.close()


def test_long_lines_against_host_restatement():
    """1536 x 16 x 576: a 1536-point x transform and a 576-point z transform
    (8 kx columns per block instead of 16), two steps against oracle/refcpu.cpp."""
    from channel_rl_gb300.host import Channel
    from oracle.refcpu import RefCPU
    case = C.smaller(C.c3_roofline(les=C.LES_DSM), 1536, 16, 576)
    U, V, W = C.initial_fields(case)
    ch = Channel(case)
    ch.upload(U, V, W)
    ch.step(2)
    d = ch.download()
    assert ch.check_divergence()[1] < 1e-12
    ch.close()
    r = RefCPU(case)
    r.upload(U, V, W)
    r.step(2)
    h = r.download()
    r.close()
    for f in "UVW":
        e = np.abs(d[f] - h[f]).max() / np.abs(h[f]).max()
        assert e < FIELD_RTOL, (f, e)
