"""Channel cases: grids, parameters and seeded initial fields.

A case is what the reference reads from its parameter file
(input_output.f90:20-91) plus the grid and the initial field that it takes
from a ``.init`` snapshot or generates in ``init_flow``
(input_output.f90:99-174).  The reference's own ``.init`` fields are not
available, so the initial fields here are seeded synthetic ones:

* ``laminar``: U = 1.5 (1 - y^2) U_b plus uniform noise of +-amp U_b;
* ``loglaw``:  U = u_tau (ln(y+)/kappa + B) (u_tau y+ in the viscous
  sublayer) of the distance to the nearer wall, plus uniform noise;
V and W are uniform noise of +-amp U_b.  Walls are at y = -1 and y = +1.

Grid convention (matches the reference's parameter files, 130x41x66 faces
for 128x40x64 cells): ``Nx, Ny, Nz`` are unique periodic cells (the FFT
lengths) and wall-normal cells, so the Fortran face counts are
nx = Nx+2, ny = Ny+1, nz = Nz+2 and the centre counts with ghosts
nxg = Nx+3, nyg = Ny+2, nzg = Nz+3.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, replace

import numpy as np

KAPPA = 0.41
B_LOG = 5.2

LES_NONE, LES_SMAG, LES_DSM, LES_AMD, LES_VREMAN = 0, 1, 2, 3, 4
WM_NONE, WM_STRESS, WM_EQLOG, WM_MLP = 0, 1, 2, 3


@dataclass(frozen=True)
class Case:
    name: str
    Nx: int
    Ny: int
    Nz: int
    Lx: float = 2.0 * math.pi
    Lz: float = math.pi
    stretch: float = 0.0          # tanh stretching of the wall-normal faces (0: uniform)
    nu: float = 2.0 / 5600.0
    CFL: float = 0.5
    dPdx: float = 0.0
    x_mass_cte: int = 1
    LES_model: int = LES_DSM
    Dirichlet_nu_t: int = 1
    wall_model: int = WM_NONE
    Cs: float = 0.1
    Retau: float = 180.0
    init: str = "laminar"
    amp: float = 0.1
    seed: int = 1234
    # explicit face coordinates (e.g. from a snapshot file); None: built from Lx, Lz, stretch
    xf: tuple | None = None
    yf: tuple | None = None
    zf: tuple | None = None

    # Fortran extents
    @property
    def nx(self):
        return self.Nx + 2

    @property
    def ny(self):
        return self.Ny + 1

    @property
    def nz(self):
        return self.Nz + 2

    @property
    def points(self):
        return self.Nx * self.Ny * self.Nz


def utau_for_retau(retau, ub=1.0):
    """u_tau whose log-law profile has bulk velocity ub in a channel of
    half-height 1: ub/u_tau = (ln Re_tau - 1)/kappa + B."""
    return ub / ((math.log(retau) - 1.0) / KAPPA + B_LOG)


def wallmodelled(name, Nx, Ny, Nz, retau, *, Lx=2.0 * math.pi, Lz=math.pi, les=LES_DSM,
                 x_mass_cte=0, seed=1234, wall_model=WM_EQLOG):
    ut = utau_for_retau(retau)
    nu = ut / retau
    return Case(name=name, Nx=Nx, Ny=Ny, Nz=Nz, Lx=Lx, Lz=Lz, stretch=0.0, nu=nu, CFL=0.5,
                dPdx=ut * ut, x_mass_cte=x_mass_cte, LES_model=les, Dirichlet_nu_t=1,
                wall_model=wall_model, Retau=retau, init="loglaw", amp=0.1, seed=seed)


def c1_small(seed=1234):
    """Plain method, single small channel: 32x48x32, tanh stretching 2.0,
    Re_bulk 5600 (nu = 2/5600), constant mass flow, DSM, no wall model."""
    return Case(name="c1_32x48x32_dsm_nowm", Nx=32, Ny=48, Nz=32, stretch=2.0,
                nu=2.0 / 5600.0, CFL=0.5, x_mass_cte=1, LES_model=LES_DSM,
                wall_model=WM_NONE, Retau=180.0, init="laminar", seed=seed)


def c2_wm64(seed=1234):
    """Plain method, wall-modelled: 64^3 uniform, Re_tau 2000 via constant
    mass flow, equilibrium log-law wall model, DSM."""
    return wallmodelled("c2_64x64x64_dsm_eqwm", 64, 64, 64, 2000.0, x_mass_cte=1, seed=seed)


def c3_roofline(les=LES_SMAG, seed=1234):
    """Roofline sizing: 8pi x 2 x 3pi, 256x96x192, Re_tau 5200, equilibrium
    wall model, static Smagorinsky Cs=0.1 (or DSM), pressure-gradient forcing."""
    tag = "smag" if les == LES_SMAG else "dsm"
    return wallmodelled(f"c3_256x96x192_{tag}_eqwm", 256, 96, 192, 5200.0,
                        Lx=8.0 * math.pi, Lz=3.0 * math.pi, les=les, x_mass_cte=0, seed=seed)


def c4_ensemble(n=64, seed=4321):
    """Batched ensemble: grids drawn from the seed, Nx,Nz in {32,48,64,96},
    Ny in {32,48,64}, Re_tau log-uniform in [1000, 10000]."""
    rng = np.random.default_rng(seed)
    out = []
    for m in range(n):
        Nx = int(rng.choice([32, 48, 64, 96]))
        Nz = int(rng.choice([32, 48, 64, 96]))
        Ny = int(rng.choice([32, 48, 64]))
        retau = float(math.exp(rng.uniform(math.log(1000.0), math.log(10000.0))))
        out.append(wallmodelled(f"c4_{m:02d}_{Nx}x{Ny}x{Nz}", Nx, Ny, Nz, retau,
                                seed=seed + 17 * m))
    return out


def rl_case(seed=2000):
    """The size and physics of the reference's own RL cases (its parameter
    files for Re_tau 2000: 130x41x66 faces = 128x40x64 cells, 2pi x 2 x pi,
    AMD with Dirichlet nu_t ghosts, pressure-gradient forcing, fixed
    dt = 1e-2), with the equilibrium wall model setting the wall stress
    that the reference's agents set."""
    return replace(wallmodelled("rl_128x40x64_amd", 128, 40, 64, 2000.0, les=LES_AMD, seed=seed), CFL=-1e-2)


def c5_learned(n=16, seed=5555):
    """Learned wall model: 16 channels, Re_tau in {2000, 5200, 10000},
    grids 48x48x48 .. 96x64x96."""
    rng = np.random.default_rng(seed)
    grids = [(48, 48, 48), (64, 48, 64), (64, 64, 64), (96, 48, 96), (96, 64, 96)]
    out = []
    for m in range(n):
        Nx, Ny, Nz = grids[int(rng.integers(len(grids)))]
        retau = float([2000.0, 5200.0, 10000.0][m % 3])
        out.append(wallmodelled(f"c5_{m:02d}_{Nx}x{Ny}x{Nz}", Nx, Ny, Nz, retau,
                                seed=seed + 31 * m, wall_model=WM_MLP))
    return out


def faces(case: Case):
    """Face coordinates x(1:nx), y(1:ny), z(1:nz) as the reference's grid
    arrays (global.f90:63-67): x(i) = (i-1) Lx/Nx so that x(nx-1) = Lx,
    unless the case carries explicit coordinates."""
    if case.xf is not None:
        return (np.array(case.xf, dtype=np.float64), np.array(case.yf, dtype=np.float64),
                np.array(case.zf, dtype=np.float64))
    dx = case.Lx / case.Nx
    dz = case.Lz / case.Nz
    x = np.arange(case.nx, dtype=np.float64) * dx
    z = np.arange(case.nz, dtype=np.float64) * dz
    eta = 2.0 * np.arange(case.ny, dtype=np.float64) / case.Ny - 1.0
    if case.stretch > 0.0:
        y = np.tanh(case.stretch * eta) / math.tanh(case.stretch)
    else:
        y = eta.copy()
    y[0], y[-1] = -1.0, 1.0
    return x, y, z


def centres_y(y):
    """yg(1:nyg) from faces (initialization.f90:197-216)."""
    ny = y.size
    ym = 0.5 * (y[:-1] + y[1:])
    yg = np.empty(ny + 1)
    yg[1:ny] = ym
    yg[0] = ym[0] - 2.0 * (ym[0] - y[0])
    yg[ny] = ym[-1] + 2.0 * (y[-1] - ym[-1])
    return yg


def mean_profile(case: Case, yc):
    if case.init == "laminar":
        return 1.5 * (1.0 - yc * yc)
    ut = case.dPdx ** 0.5 if case.dPdx > 0 else utau_for_retau(case.Retau)
    d = np.clip(1.0 - np.abs(yc), 0.0, None)
    yp = d * ut / case.nu
    with np.errstate(divide="ignore"):
        lg = ut * (np.log(np.maximum(yp, 1e-300)) / KAPPA + B_LOG)
    return np.where(yp > 11.06, lg, ut * yp)


def initial_fields(case: Case):
    """Seeded initial U(nx,nyg,nzg), V(nxg,ny,nzg), W(nxg,nyg,nz), Fortran
    order.  Ghost entries are filled too; the solver re-applies its boundary
    conditions on upload, as the reference's snapshot reader does."""
    x, y, z = faces(case)
    yg = centres_y(y)
    nx, ny, nz = case.nx, case.ny, case.nz
    nxg, nyg, nzg = nx + 1, ny + 1, nz + 1
    rng = np.random.default_rng(case.seed)
    a = case.amp
    ru = rng.random((nzg, nyg, nx))
    rv = rng.random((nzg, ny, nxg))
    rw = rng.random((nz, nyg, nxg))
    prof = mean_profile(case, yg)
    U = prof[None, :, None] + a * (2.0 * ru - 1.0)
    V = a * (2.0 * rv - 1.0)
    W = a * (2.0 * rw - 1.0)
    # (k, j, i) C-order -> (i, j, k) Fortran order
    return (np.asfortranarray(U.transpose(2, 1, 0)),
            np.asfortranarray(V.transpose(2, 1, 0)),
            np.asfortranarray(W.transpose(2, 1, 0)))


def smaller(case: Case, Nx, Ny, Nz):
    """Same physics on another grid (used for quick parity cases)."""
    return replace(case, Nx=Nx, Ny=Ny, Nz=Nz, name=f"{case.name}_as_{Nx}x{Ny}x{Nz}")


def case_from_files(params_path, snapshot_path=None, wall_model=WM_STRESS, Cs=0.1, Retau=0.0):
    """A case and its initial fields from the reference's own files: the
    parameter file (read_input_parameters, input_output.f90:20-91) and the
    snapshot it names (read_input_data, input_output.f90:390-560; resolved
    against the parameter file's folder unless given).  The parameter file
    has no wall-model entry (the reference always calls compute_wall_model
    with the alpha_x its RL driver sets), hence the argument."""
    import os
    from .host import read_parameters, read_snapshot
    p = read_parameters(params_path)
    path = snapshot_path or os.path.join(os.path.dirname(os.path.abspath(params_path)), p["filein"])
    snap = read_snapshot(path)
    if (snap["x"].size, snap["y"].size, snap["z"].size) != (p["nx"], p["ny"], p["nz"]):
        raise ValueError("snapshot extents differ from the parameter file")
    x, y, z = snap["x"], snap["y"], snap["z"]
    case = Case(name=os.path.basename(path), Nx=p["nx"] - 2, Ny=p["ny"] - 1, Nz=p["nz"] - 2,
                Lx=float(x[-2] - x[0]), Lz=float(z[-2] - z[0]), nu=p["nu"], CFL=p["CFL"], dPdx=p["dPdx"],
                x_mass_cte=p["x_mass_cte"], LES_model=p["LES_model"], Dirichlet_nu_t=p["Dirichlet_nu_t"],
                wall_model=wall_model, Cs=Cs, Retau=Retau, init="file",
                xf=tuple(x.tolist()), yf=tuple(y.tolist()), zf=tuple(z.tolist()))
    return case, (snap["U"], snap["V"], snap["W"]), p
