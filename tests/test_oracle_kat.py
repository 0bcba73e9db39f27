"""Known-answer tests of the CPU oracle (no GPU).

The reference ships no tests or golden data, so the oracle is pinned by
properties the discretisation must have and by LAPACK's zgtsv, then frozen
by the fixtures in tests/golden/.
"""
import math

import numpy as np
import pytest
from scipy.linalg import lapack

from channel_rl_gb300 import cases as C
from oracle import channel_ref as R
from tests.helpers import oracle_for, rel


def small(case, nx=16, ny=12, nz=16):
    return C.smaller(case, nx, ny, nz)


def test_rk3_table_consistent():
    for s in range(3):
        assert math.isclose(sum(R.RK_COEF[s]), R.RK_T[s], rel_tol=0, abs_tol=1e-15)


def test_grid_constants_match_reference_formulas():
    case = C.c1_small()
    g = R.Grid(*C.faces(case))
    # modified wavenumbers: 2 (cos(2 pi k/N) - 1)/dx^2, symmetric in k
    k = np.arange(g.Nx)
    ref = 2.0 * (np.cos(2 * np.pi * k / g.Nx) - 1.0) / g.dxmin ** 2
    assert np.abs(g.kxx - ref).max() <= 1e-12 * np.abs(ref).max()
    assert np.array_equal(g.kxx[1:], g.kxx[1:][::-1])
    # Neumann rows of Dyy: row sums vanish at both walls (constant pressure
    # is in the null space before the 00-mode pin)
    j = np.arange(3, g.nyg - 1)
    assert np.abs(g.Dd[2] + g.Du[2]) < 1e-9 * abs(g.Dd[2])
    assert np.abs(g.Dd[g.nyg - 1] + g.Dl[g.nyg - 1]) < 1e-9 * abs(g.Dd[g.nyg - 1])
    assert np.all(np.abs(g.Dd[j] + g.Du[j] + g.Dl[j]) < 1e-9 * np.abs(g.Dd[j]))
    # interpolation weights reproduce linear functions of y
    y, yg = g.y, g.yg
    lin = g.w0[1:] * yg[1:g.nyg] + g.w1[1:] * yg[2:g.nyg + 1]
    assert np.abs(lin - y[1:]).max() < 1e-14


def test_tridiagonal_matches_zgtsv():
    case = C.c1_small()
    o = oracle_for(case)
    g = o.g
    rng = np.random.default_rng(0)
    Ny = g.nyg - 2
    rhs = rng.standard_normal((g.Nx, Ny, g.Nz)) + 1j * rng.standard_normal((g.Nx, Ny, g.Nz))
    sol = o.solve_modes(rhs)
    for (kx, kz) in [(0, 0), (1, 0), (0, 3), (5, 7), (g.Nx // 2, g.Nz // 2), (g.Nx - 1, 1)]:
        d = (g.Dd[2:g.nyg] + g.kxx[kx] + g.kzz[kz]).astype(complex)
        if kx == 0 and kz == 0:
            d[0] *= 1.5
        dl = g.Dl[3:g.nyg].astype(complex)
        du = g.Du[2:g.nyg - 1].astype(complex)
        _, _, _, x, info = lapack.zgtsv(dl.copy(), d.copy(), du.copy(), rhs[kx, :, kz].copy()[:, None])
        assert info == 0
        assert rel(sol[kx, :, kz], x[:, 0]) < 1e-11


def test_poisson_manufactured_solution():
    """solve_poisson_equation inverts the discrete Laplacian of the
    projection (d/dy Dyy + central differences in x, z) up to a constant."""
    case = small(C.c1_small())
    o = oracle_for(case)
    g = o.g
    rng = np.random.default_rng(3)
    p = rng.standard_normal((g.Nx, g.nyg - 2, g.Nz))
    lap = np.zeros_like(p)
    dx2, dz2 = g.dxmin ** 2, g.dzmin ** 2
    lap += (np.roll(p, -1, 0) - 2 * p + np.roll(p, 1, 0)) / dx2
    lap += (np.roll(p, -1, 2) - 2 * p + np.roll(p, 1, 2)) / dz2
    Ny = g.nyg - 2
    for r in range(Ny):
        jf = r + 2
        lap[:, r, :] += g.Dd[jf] * p[:, r, :]
        if r > 0:
            lap[:, r, :] += g.Dl[jf] * p[:, r - 1, :]
        if r < Ny - 1:
            lap[:, r, :] += g.Du[jf] * p[:, r + 1, :]
    div = np.zeros((g.nxg - 2, g.nyg - 2, g.nzg - 2))
    div[:g.Nx, :, :g.Nz] = lap
    # remove the 00-mode pin's effect by comparing gradients (p up to a constant)
    out = o.solve_poisson_equation(div)[2:g.Nx + 2, 2:g.nyg, 2:g.Nz + 2]
    c = (out - p).mean()
    assert rel(out - c, p) < 1e-10


def test_projection_is_divergence_free():
    case = small(C.c1_small())
    o = oracle_for(case)
    o.set_fields(*C.initial_fields(case))
    assert o.check_divergence()[1] > 1e-3
    o.compute_projection_step()
    o.apply_boundary_conditions()
    assert o.check_divergence()[1] < 1e-12


def test_uniform_flow_has_no_advection():
    case = small(C.c1_small())
    o = oracle_for(case)
    g = o.g
    U = np.full((g.nx, g.nyg, g.nzg), 0.7)
    V = np.zeros((g.nxg, g.ny, g.nzg))
    W = np.zeros((g.nxg, g.nyg, g.nz))
    o.set_fields(U, V, W)
    o.nu_t[:] = 0.0
    F = o.compute_rhs_u(o.U, o.V, o.W, o.nu_t, 0.0)
    assert np.abs(F[:, 2:-2, :]).max() < 1e-12      # rows away from the walls


def test_dynamic_smagorinsky_scales_linearly():
    """L and M are both quadratic in the velocity, so <LM>/<MM> is scale
    free and nu_t = -1/2 <LM>/<MM> |S| is linear in the velocity scale."""
    case = small(C.c1_small())
    U, V, W = C.initial_fields(case)
    o1 = oracle_for(case)
    o1.set_fields(U, V, W)
    n1 = o1.compute_eddy_viscosity().copy()
    o2 = oracle_for(case)
    o2.set_fields(3.0 * U, 3.0 * V, 3.0 * W)
    n2 = o2.compute_eddy_viscosity()
    assert np.abs(n1).max() > 0
    assert rel(n2, 3.0 * n1) < 1e-12


def test_equilibrium_wall_stress_satisfies_log_law():
    nu, h = 1e-4, 0.05
    u = np.array([0.3, 1.0, 1.7, -1.2])
    tau = R.eqlog_tau(u, h, nu)
    ut = np.sqrt(np.abs(tau))
    resid = np.abs(u) / ut - (np.log(h * ut / nu) / R.KAPPA + R.B_LOG)
    assert np.abs(resid).max() < 1e-10
    assert np.all(np.sign(tau) == np.sign(u))
    # viscous sublayer: linear law
    t2 = R.eqlog_tau(np.array([1e-3]), 1e-3, 1e-2)
    assert abs(t2[0] - 1e-2 * 1e-3 / 1e-3) < 1e-15


def test_dt_is_viscous_or_capped():
    case = C.c1_small()
    o = oracle_for(case)
    o.set_fields(*C.initial_fields(case))
    dt = o.compute_dt()
    g, p = o.g, o.p
    assert dt == min(p.CFL * min(g.dxmin, g.dymin, g.dzmin) ** 2 / p.nu, 1e-3)


def test_rk3_step_keeps_mass_flow_constant():
    case = small(C.c1_small())
    o = oracle_for(case)
    o.set_fields(*C.initial_fields(case))
    for _ in range(3):
        o.step()
        assert abs(o.compute_dPx_for_constant_mass_flow()) < 1e-12
        assert o.check_divergence()[1] < 1e-12


def _linear_field_oracle(model, a=0.7):
    """Uniform 16x12x8 grid, u = a x, v = -a y, w = 0 (no boundary conditions
    applied: the SGS routines read the arrays as given)."""
    case = C.Case(name="kat", Nx=16, Ny=12, Nz=8, Lx=2.0, Lz=1.0)
    g = R.Grid(*C.faces(case))
    o = R.ChannelOracle(g, R.Params(nu=1e-3, LES_model=model, Dirichlet_nu_t=0))
    o.U[1:, 1:, 1:] = a * g.x[1:, None, None]
    o.V[1:, 1:, 1:] = -a * g.y[None, 1:, None]
    o.W[...] = 0.0
    return o, g, 2.0 / 16, 2.0 / 12


def test_amd_pure_strain_known_answer():
    """AMD on u = a x, v = -a y: N = a^3 (dx^2 - dy^2), D = 2 a^2, so
    nu_t = 0.15 a (dy^2 - dx^2) (subgrid.f90:632-874, C = 0.3)."""
    a = 0.7
    o, g, dx, dy = _linear_field_oracle(R.LES_AMD, a)
    nt = o.compute_eddy_viscosity()[2:g.nxg - 1, 2:g.nyg, 2:g.nzg - 1]
    assert np.allclose(nt, 0.15 * a * (dy * dy - dx * dx), rtol=1e-13, atol=0)


def test_vreman_pure_strain_known_answer():
    """Vreman on u = a x, v = -a y: B_b = dx^2 dy^2 a^4, a_ij a_ij = 2 a^2,
    nu_t = C dx dy |a| / sqrt(2), C = 2.5 * 0.1^2 (subgrid.f90:897-1004)."""
    a = 0.7
    o, g, dx, dy = _linear_field_oracle(R.LES_VREMAN, a)
    nt = o.compute_eddy_viscosity()[2:g.nxg - 1, 2:g.nyg, 2:g.nzg - 1]
    assert np.allclose(nt, 0.025 * dx * dy * a / math.sqrt(2.0), rtol=1e-13, atol=0)


@pytest.mark.parametrize("model", [3, 4])
def test_amd_and_vreman_vanish_in_pure_shear(model):
    """Both models are built to give no eddy viscosity in a pure shear u(y)."""
    o, g, _, _ = _linear_field_oracle(model)
    o.U[1:, 1:, 1:] = 0.3 * g.yg[None, 1:, None]
    o.V[...] = 0.0
    nt = o.compute_eddy_viscosity()[2:g.nxg - 1, 2:g.nyg, 2:g.nzg - 1]
    assert np.abs(nt).max() == 0.0
