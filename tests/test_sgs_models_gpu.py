"""The anisotropic minimum-dissipation (AMD) and Vreman eddy viscosities
(subgrid.f90:632-874, 897-1004) on the GPU against the oracle: nu_t of one
evaluation, then U, V, W after 5 RK3 steps, for each ghost-row rule
(Dirichlet_nu_t 0, 1, 2) with and without the wall model."""
from dataclasses import replace

import numpy as np
import pytest

from channel_rl_gb300 import cases as C
from tests.helpers import FIELD_RTOL, NUT_RTOL, oracle_for, regions, rel

pytestmark = pytest.mark.gpu

CASES = {
    "amd_dir1_nowm_massflow": replace(C.smaller(C.c1_small(), 32, 24, 16), LES_model=C.LES_AMD),
    "amd_rule2_eqwm": replace(C.smaller(C.c3_roofline(les=C.LES_DSM), 48, 24, 32), LES_model=C.LES_AMD,
                              Dirichlet_nu_t=2),
    "amd_neumann_eqwm_massflow": replace(C.smaller(C.c2_wm64(), 32, 32, 24), LES_model=C.LES_AMD,
                                         Dirichlet_nu_t=0),
    "vreman_dir1_nowm_massflow": replace(C.smaller(C.c1_small(), 24, 24, 32), LES_model=C.LES_VREMAN),
    "vreman_rule2_eqwm": replace(C.smaller(C.c3_roofline(les=C.LES_DSM), 32, 16, 48), LES_model=C.LES_VREMAN,
                                 Dirichlet_nu_t=2),
    "vreman_neumann_eqwm": replace(C.smaller(C.c2_wm64(), 32, 32, 32), LES_model=C.LES_VREMAN,
                                   Dirichlet_nu_t=0, x_mass_cte=0, dPdx=C.c2_wm64().dPdx or 1e-3),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_amd_vreman_match_oracle(name):
    from channel_rl_gb300.host import Channel
    case = CASES[name]
    U, V, W = C.initial_fields(case)
    o = oracle_for(case)
    o.set_fields(U, V, W)
    ch = Channel(case)
    ch.upload(U, V, W)
    reg = regions(o.g)
    o.compute_eddy_viscosity()
    ch.compute_eddy_viscosity()
    nt = ch.download(fields=("nu_t",))["nu_t"]
    assert np.isfinite(nt[reg["C"]]).all()
    assert (nt[reg["C"]][:, 1:-1, :] >= 0.0).all()
    assert rel(nt[reg["C"]], o.nu_t[1:, 1:, 1:][reg["C"]]) < NUT_RTOL
    for _ in range(5):
        o.step()
    ch.step(5)
    d = ch.download(fields=("U", "V", "W"))
    src = {"U": o.U, "V": o.V, "W": o.W}
    for f in "UVW":
        e = rel(d[f][reg[f]], src[f][1:, 1:, 1:][reg[f]])
        assert e < FIELD_RTOL, (f, e)
    assert ch.scalars()["dt"] == o.dt
    assert ch.check_divergence()[1] < 1e-12
    ch.close()
