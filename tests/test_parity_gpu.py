"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Tolerance: relative max error <= 1e-12 on every velocity and pressure field
(FIELD_RTOL), <= 1e-10 on nu_t of the dynamic model (NUT_RTOL, see helpers).
"""
import os
from dataclasses import replace

import numpy as np
import pytest

from channel_rl_gb300 import cases as C
from tests.helpers import FIELD_RTOL, NUT_RTOL, oracle_for, regions, rel

pytestmark = pytest.mark.gpu


def _channel(cases_):
    from channel_rl_gb300.host import Channel
    return Channel(cases_)


def _cmp_fields(d, o, fields=("U", "V", "W")):
    reg = regions(o.g)
    src = {"U": o.U, "V": o.V, "W": o.W}
    return {f: rel(d[f][reg[f]], src[f][1:, 1:, 1:][reg[f]]) for f in fields}


SUB_CASES = {
    "c1_dsm_nowm": C.c1_small(),
    "c2_dsm_eqwm": C.smaller(C.c2_wm64(), 32, 32, 32),
    "c3_smag_eqwm": C.smaller(C.c3_roofline(les=C.LES_SMAG), 48, 24, 32),
    "c3_dsm_eqwm_r3": C.smaller(C.c3_roofline(les=C.LES_DSM), 96, 16, 48),
}


@pytest.mark.parametrize("name", list(SUB_CASES))
def test_subroutines_match_oracle(name):
    case = SUB_CASES[name]
    U, V, W = C.initial_fields(case)
    o = oracle_for(case)
    o.set_fields(U, V, W)
    ch = _channel(case)
    ch.upload(U, V, W)
    g = o.g
    reg = regions(g)
    # boundary conditions on upload (apply_boundary_conditions)
    d = ch.download(fields=("U", "V", "W"))
    for f in "UVW":
        assert np.array_equal(d[f], {"U": o.U, "V": o.V, "W": o.W}[f][1:, 1:, 1:]), f
    assert rel(ch.scalars()["Qflow_x_0"], o.Qflow_x_0) < 1e-14
    # compute_dt
    ch.compute_dt()
    assert ch.scalars()["dt"] == o.compute_dt()
    # compute_eddy_viscosity
    o.compute_eddy_viscosity()
    ch.compute_eddy_viscosity()
    nt = ch.download(fields=("nu_t",))["nu_t"]
    assert rel(nt[reg["C"]], o.nu_t[1:, 1:, 1:][reg["C"]]) < (NUT_RTOL if case.LES_model == 2 else FIELD_RTOL)
    # compute_wall_model
    if case.wall_model:
        o.set_wall_stress(o.compute_wall_stress_eqlog())
        o.compute_wall_model()
        ch.compute_wall_model()
        a = ch.wall_stress()
        assert rel(a[1:-1, :, 1:-2], o.alpha_x[2:g.nx, 1:3, 2:g.nzg - 1]) < FIELD_RTOL
        nt = ch.download(fields=("nu_t",))["nu_t"]
        assert rel(nt[reg["C"]], o.nu_t[1:, 1:, 1:][reg["C"]]) < NUT_RTOL
    # compute_rhs_u/v/w
    Fu, Fv, Fw = ch.compute_rhs()
    assert rel(Fu, o.compute_rhs_u(o.U, o.V, o.W, o.nu_t, o.dPdx)[:, :, :g.Nz]) < FIELD_RTOL
    assert rel(Fv, o.compute_rhs_v(o.U, o.V, o.W, o.nu_t)[:g.Nx, :, :g.Nz]) < FIELD_RTOL
    assert rel(Fw, o.compute_rhs_w(o.U, o.V, o.W, o.nu_t)[:g.Nx, :, :]) < FIELD_RTOL
    # compute_pressure on the initial state
    o.compute_pressure()
    ch.compute_pressure()
    P = ch.download(fields=("P",))["P"]
    assert rel(P[reg["C"]], o.P[1:, 1:, 1:][reg["C"]]) < FIELD_RTOL
    # compute_dPx_for_constant_mass_flow
    assert abs(ch.compute_dPx_for_constant_mass_flow() - o.compute_dPx_for_constant_mass_flow()) < 1e-13
    # compute_projection_step (pseudo-pressure and projected velocity)
    o.compute_projection_step()
    o.apply_boundary_conditions()
    ch.compute_projection_step()
    d = ch.download(fields=("U", "V", "W"))
    for f, e in _cmp_fields(d, o).items():
        assert e < FIELD_RTOL, (f, e)
    p = ch.pseudo_pressure()
    Ip = (slice(1, g.nxg - 2), slice(1, g.nyg - 1), slice(1, g.nzg - 2))
    assert rel(p[Ip], o.rhs_p[1:, 1:, 1:][Ip]) < FIELD_RTOL
    assert ch.check_divergence()[1] < 1e-12
    ch.close()


def test_ten_steps_c1_every_field_every_step():
    """The parity bar on the small plain channel (32x48x32, dynamic
    Smagorinsky, no wall model): U, V, W and the actual pressure after each
    of the first 10 RK3 steps, within the FP64 tolerance of the oracle."""
    case = C.c1_small()
    U, V, W = C.initial_fields(case)
    o = oracle_for(case)
    o.set_fields(U, V, W)
    ch = _channel(case)
    ch.upload(U, V, W)
    reg = regions(o.g)
    for s in range(10):
        o.step()
        ch.step(1)
        o.compute_pressure()
        ch.compute_pressure()
        d = ch.download(fields=("U", "V", "W", "P"))
        errs = _cmp_fields(d, o)
        errs["P"] = rel(d["P"][reg["C"]], o.P[1:, 1:, 1:][reg["C"]])
        assert max(errs.values()) < FIELD_RTOL, (s + 1, errs)
        assert ch.scalars()["dt"] == o.dt
        assert ch.check_divergence()[1] < 1e-12
    st, so = ch.compute_statistics(), o.compute_statistics()
    for k in ("Umean", "Vmean", "Wmean", "U2mean", "V2mean", "W2mean", "UVmean"):
        assert rel(st[k], so[k]) < 1e-11, k
    for k in ("utau", "Retau", "Qflow_x"):
        assert abs(st[k] - so[k]) <= 1e-12 * abs(so[k]), k
    ch.close()


def test_rk3_takes_the_dt_set_from_the_host():
    """compute_time_step_RK3 without compute_dt uses the step size set through
    chl_set_scalars (which also forms the stage products dt c / 4 that the
    update kernel reads): a dt that compute_dt would not produce, two steps,
    every velocity field within FIELD_RTOL of the oracle's RK3 with that dt."""
    case = C.c1_small()
    U, V, W = C.initial_fields(case)
    o = oracle_for(case)
    o.set_fields(U, V, W)
    ch = _channel(case)
    ch.upload(U, V, W)
    dt = 0.37 * o.compute_dt()
    for s in range(2):
        o.dt = dt
        ch.set_scalars(dt=dt)
        o.compute_time_step_RK3()
        ch.compute_time_step_RK3()
        d = ch.download(fields=("U", "V", "W"))
        for f, e in _cmp_fields(d, o).items():
            assert e < FIELD_RTOL, (s + 1, f, e)
        assert ch.scalars()["dt"] == dt
    ch.close()


def test_golden_fixtures_on_gpu():
    from tests.golden.make_golden import NSTEP, golden_cases, summarise
    gold = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.npz"))
    for tag, case in golden_cases().items():
        ch = _channel(case)
        ch.upload(*C.initial_fields(case))
        g = oracle_for(case).g
        for s in range(1, NSTEP + 1):
            ch.step(1)
            ch.compute_pressure()
            d = ch.download(fields=("U", "V", "W", "P"))
            got = summarise(d, g)
            for k, v in got.items():
                ref = gold[f"{tag}_s{s}_{k}"]
                assert np.abs(v - ref).max() <= FIELD_RTOL * np.abs(ref).max(), (tag, s, k)
        ch.close()


def test_batched_instances_equal_single_runs():
    """Uneven instances in one launch per kernel advance exactly as they do alone."""
    batch = [C.smaller(C.c2_wm64(), 32, 32, 48), C.smaller(C.c3_roofline(les=C.LES_DSM), 64, 24, 32),
             C.wallmodelled("x", 48, 48, 96, 7000.0, seed=99)]
    chb = _channel(batch)
    for q, c in enumerate(batch):
        chb.upload(*C.initial_fields(c), inst=q)
    chb.step(3)
    chb.synchronize()
    for q, c in enumerate(batch):
        ch = _channel(c)
        ch.upload(*C.initial_fields(c))
        ch.step(3)
        a = chb.download(inst=q)
        b = ch.download()
        for f in "UVW":
            assert np.array_equal(a[f], b[f]), (q, f)
        assert chb.scalars(q)["dt"] == ch.scalars()["dt"]
        ch.close()
    chb.close()


def test_full_size_roofline_channel_properties():
    """256x96x192 at full size: the oracle is too slow for many steps here,
    so check one step against it plus size-independent properties."""
    case = C.c3_roofline(les=C.LES_DSM)
    U, V, W = C.initial_fields(case)
    ch = _channel(case)
    ch.upload(U, V, W)
    ch.step(1)
    ch.synchronize()
    o = oracle_for(case)
    o.set_fields(U, V, W)
    o.step()
    d = ch.download(fields=("U", "V", "W"))
    for f, e in _cmp_fields(d, o).items():
        assert e < FIELD_RTOL, (f, e)
    ch.step(4)
    ch.synchronize()
    assert ch.check_divergence()[1] < 1e-12
    d = ch.download(fields=("U", "V", "W", "nu_t"))
    assert all(np.isfinite(v).all() for v in d.values())
    ch.close()


def test_calls_out_of_order_report_errors():
    from channel_rl_gb300.host import ChlError
    ch = _channel(C.smaller(C.c1_small(), 16, 12, 16))
    with pytest.raises(ChlError, match="not uploaded"):
        ch.step(1)
    with pytest.raises(ValueError):
        ch.upload(np.zeros((3, 3, 3)), np.zeros((3, 3, 3)), np.zeros((3, 3, 3)))
    ch.close()


@pytest.mark.parametrize("cfl", [0.5, -1e-3], ids=["cfl", "fixed_dt"])
def test_non_finite_velocity_is_reported(cfl):
    """A NaN in the uploaded field (made on the host) is found by the next
    step's CFL pass (with a fixed step, by its non-finite check alone) and
    reported as CHL_E_NAN at the synchronising calls, until clean fields are
    uploaded again."""
    from channel_rl_gb300.host import ChlError
    case = replace(C.smaller(C.c1_small(), 16, 12, 16), CFL=cfl)
    U, V, W = C.initial_fields(case)
    ch = _channel(case)
    bad = U.copy()
    bad[5, 6, 7] = np.nan
    ch.upload(bad, V, W)
    ch.step(1)
    with pytest.raises(ChlError, match=r"\(5\).*non-finite"):
        ch.synchronize()
    with pytest.raises(ChlError, match="non-finite"):
        ch.download()
    ch.upload(U, V, W)
    ch.step(1)
    ch.synchronize()
    assert np.isfinite(ch.download()["U"]).all()
    ch.close()


def test_non_finite_instance_is_isolated_in_a_batch():
    """One channel of a batch carries a NaN: the batch-wide check names it,
    the others stay readable and advance exactly as they do alone."""
    from channel_rl_gb300.host import ChlError
    batch = [C.smaller(C.c2_wm64(), 32, 16, 16), C.smaller(C.c1_small(), 16, 12, 16),
             C.smaller(C.c3_roofline(les=C.LES_DSM), 24, 16, 32)]
    batch = [b if q != 1 else replace(b, wall_model=C.WM_EQLOG, Retau=2000.0, x_mass_cte=1)
             for q, b in enumerate(batch)]
    chb = _channel(batch)
    for q, c in enumerate(batch):
        U, V, W = C.initial_fields(c)
        if q == 1:
            U = U.copy()
            U[3, 4, 5] = np.inf
        chb.upload(U, V, W, inst=q)
    chb.step(3)
    with pytest.raises(ChlError, match="instance 1"):
        chb.synchronize()
    with pytest.raises(ChlError, match="non-finite"):
        chb.download(inst=1)
    for q in (0, 2):
        ch = _channel(batch[q])
        ch.upload(*C.initial_fields(batch[q]))
        ch.step(3)
        a, b = chb.download(inst=q), ch.download()
        for f in "UVW":
            assert np.array_equal(a[f], b[f]), (q, f)
        ch.close()
    chb.close()


def test_viscous_limit_of_dt():
    """compute_dt's viscous limit CFL*dymin**2/nu (time_integration.f90:131-137)
    binding: a viscous small channel (nu = 0.2 on a stretched 16x24x16 mesh)
    where it lies below both the convective limit and the 1e-3 cap.  dt equals
    the oracle's bit for bit over three steps."""
    case = replace(C.smaller(C.c1_small(), 16, 24, 16), nu=0.2)
    U, V, W = C.initial_fields(case)
    o = oracle_for(case)
    o.set_fields(U, V, W)
    g = o.g
    vis = min(case.CFL * g.dxmin ** 2.0 / case.nu, case.CFL * g.dymin ** 2.0 / case.nu,
              case.CFL * g.dzmin ** 2.0 / case.nu)
    ch = _channel(case)
    ch.upload(U, V, W)
    for s in range(3):
        o.step()
        ch.step(1)
        assert o.dt == vis < 1e-3, (o.dt, vis)
        assert ch.scalars()["dt"] == o.dt, s
    d = ch.download(fields=("U", "V", "W"))
    for f, e in _cmp_fields(d, o).items():
        assert e < FIELD_RTOL, (f, e)
    ch.close()
