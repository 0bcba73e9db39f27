"""CPU oracle for the channel LES RK3 time step — TEST INFRASTRUCTURE ONLY.

This module is the checker for the GB300 path.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import it;
the product path (``channel_rl_gb300``) never does.

It restates, routine by routine, the Fortran reference of wadaniel/channel_RL
(file:line citations below are into that project's ``code/`` directory) in
NumPy, in the reference's own Fortran index convention: every 3-D array is
stored with one padding slot so that ``A[i, j, k]`` is the Fortran element
``A(i,j,k)`` (index 0 unused) and a Fortran range ``lo:hi`` is the Python
slice ``lo:hi+1``.

Decomposition semantics.  The reference is an MPI z-slab code.  Its
single-rank run is broken (``apply_periodic_bc_z`` self-sendrecv truncates,
boundary_conditions.f90:144-151; the pseudo-pressure z-wrap is skipped,
projection.f90:139-149), so this oracle implements what a P>=2 run computes:
z periodic exactly like x, with the per-rank loop ranges, whose union is the
P=1 range (e.g. the DSM plane sums run over i=2..nxg-1, k=2..nzg-1, which
includes one duplicated periodic column and plane).  ``update_ghost_interior_
planes`` is the identity in this global view.

Known reference quirks reproduced on purpose (each is a switchable oracle
mode where the reference itself cannot run it):
* compute_dt takes max(dx/|u|) (time_integration.f90:117-119);
* the constant-mass-flow control averages planes j=3 and nyg-2 only and
  shifts U by the difference (mass_flow.f90:135-155, time_integration.f90:89-94);
* the wall model overwrites nu_t in rows 1,2,nyg-1,nyg and uses yg(2)-yg(1)
  for both walls (wallmodel.f90:32-42); its x interpolation writes centres
  2..nx (one past the section, wallmodel.f90:37);
* x/z interpolation ignores ``di`` (interpolation.f90:24-40, 88-105); the
  viscous y flux of u and w uses the un-interpolated dU/dy (equations.f90:115,417);
* the 00 Fourier mode is pinned by D(2)*=3/2 (projection.f90:107);
* static Smagorinsky aborts in the reference (subgrid.f90:575); it is written
  from its formula with Cs=0.1 and with periodic nu_t ghosts;
* ``rhs_uf/vf/wf`` are never allocated in the reference (global.f90:96), so
  compute_pressure uses full-extent arrays (intended semantics).
* "no wall model" means skipping compute_wall_model (the reference always
  calls it, time_integration.f90:37,54,71).

Parity status: UNPINNED.  The reference has no tests, fixtures or golden
vectors, its ``.init`` input fields are not in the repository, and it cannot
be built here (Fortran + MPI + FFTW-MPI + LAPACK + smarties; no gfortran).
The oracle is instead checked by known-answer tests (tests/test_oracle_kat.py)
and frozen by golden fixtures it generated (tests/golden/).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# ---------------------------------------------------------------------------
# constants (initialization.f90:413-427)
RK_T = (8.0 / 15.0, 2.0 / 3.0, 1.0)
RK_COEF = ((8.0 / 15.0, 0.0, 0.0),
           (1.0 / 4.0, 5.0 / 12.0, 0.0),
           (1.0 / 4.0, 0.0, 3.0 / 4.0))

# equilibrium wall model (log law)
KAPPA = 0.41
B_LOG = 5.2
EQWM_NEWTON_ITERS = 12

LES_NONE, LES_SMAG, LES_DSM, LES_AMD, LES_VREMAN = 0, 1, 2, 3, 4
WM_NONE, WM_STRESS, WM_EQLOG, WM_MLP = 0, 1, 2, 3


def pad1(a):
    """1-D Fortran-indexed copy: result[i] == a(i) for i=1..n."""
    a = np.asarray(a, dtype=np.float64)
    out = np.zeros(a.size + 1)
    out[1:] = a
    return out


def alloc(n1, n2, n3):
    return np.zeros((n1 + 1, n2 + 1, n3 + 1))


@dataclass
class Params:
    """The reference's input-parameter block (input_output.f90:20-91)."""
    nu: float
    CFL: float = 0.5
    dPdx: float = 0.0
    x_mass_cte: int = 1
    LES_model: int = LES_DSM
    Dirichlet_nu_t: int = 1
    wall_model: int = WM_NONE      # oracle switch (see module doc)
    Cs: float = 0.1                # static Smagorinsky constant
    Re_tau: float = 0.0            # nominal Re_tau (learned wall model feature ln(h Re_tau))


class Grid:
    """Grid constants derived from face coordinates (initialization.f90:187-427)."""

    def __init__(self, xf, yf, zf):
        x, y, z = pad1(xf), pad1(yf), pad1(zf)
        nx, ny, nz = x.size - 1, y.size - 1, z.size - 1
        if nx % 2 or nz % 2:                      # initialization.f90:66-67
            raise ValueError("nx and nz must be even")
        nxm, nym, nzm = nx - 1, ny - 1, nz - 1
        nxg, nyg, nzg = nxm + 2, nym + 2, nzm + 2
        self.nx, self.ny, self.nz = nx, ny, nz
        self.nxg, self.nyg, self.nzg = nxg, nyg, nzg
        self.x, self.y, self.z = x, y, z

        def centres(f, n):                       # initialization.f90:194-220
            m = np.zeros(n)                      # m[i] = fm(i), i = 1..n-1
            m[1:] = 0.5 * (f[1:n] + f[2:n + 1])
            g = np.zeros(n + 2)                  # g[i], i = 1..n+1
            g[2:n + 1] = m[1:]
            g[1] = m[1] - 2.0 * (m[1] - f[1])
            g[n + 1] = m[n - 1] + 2.0 * (f[n] - m[n - 1])
            return m, g

        self.xm, self.xg = centres(x, nx)
        self.ym, self.yg = centres(y, ny)
        self.zm, self.zg = centres(z, nz)
        xg, yg, zg = self.xg, self.yg, self.zg
        # initialization.f90:233-240
        self.dxmin = float(np.min(xg[2:nxg + 1] - xg[1:nxg]))
        self.dymin = float(np.min(yg[2:nyg + 1] - yg[1:nyg]))
        self.dzmin = float(np.min(zg[2:nzg + 1] - zg[1:nzg]))
        self.Lx = x[nx] - x[1]
        self.Ly = y[ny] - y[1]
        self.Lz = z[nz] - z[1]
        # Fourier lengths and modified wavenumbers (initialization.f90:250-308)
        self.Nx = nxm - 1
        self.Nz = nzm - 1
        dx, dz = self.dxmin, self.dzmin
        self.kxx = self._kmod(self.Nx, dx)
        self.kzz = self._kmod(self.Nz, dz)
        # Dyy (initialization.f90:355-385): stored as tridiagonal bands over
        # rows j = 2..nyg-1, Fortran indexed.
        def abc(j):
            a = 1.0 / (y[j] - y[j - 1]) / (yg[j + 1] - yg[j])
            b = 1.0 / (y[j] - y[j - 1]) * (-1.0 / (yg[j + 1] - yg[j]) - 1.0 / (yg[j] - yg[j - 1]))
            c = 1.0 / (y[j] - y[j - 1]) / (yg[j] - yg[j - 1])
            return a, b, c
        self.Dd = np.zeros(nyg + 1)     # Dyy(j,j)
        self.Du = np.zeros(nyg + 1)     # Dyy(j,j+1)
        self.Dl = np.zeros(nyg + 1)     # Dyy(j,j-1)
        for j in range(3, nyg - 1):
            a, b, c = abc(j)
            self.Du[j], self.Dl[j], self.Dd[j] = a, c, b
        a, b, c = abc(2)
        self.Dd[2], self.Du[2], self.coef_bc_1 = b + c, a, c
        a, b, c = abc(nyg - 1)
        self.Dd[nyg - 1], self.Dl[nyg - 1], self.coef_bc_2 = a + b, c, a
        # interpolation weights (initialization.f90:398-400)
        self.w0 = np.zeros(ny + 1)
        self.w0[1:] = (yg[2:nyg + 1] - y[1:ny + 1]) / (yg[2:nyg + 1] - yg[1:nyg])
        self.w1 = 1.0 - self.w0
        self.w1[0] = 0.0

    @staticmethod
    def _kmod(N, d):
        """initialization.f90:296-308 (Ceiling(N/2) split kept as written)."""
        k = np.zeros(N)
        half = int(math.ceil(N / 2.0))
        for i in range(0, half + 1):
            if i < N:
                k[i] = 2.0 * (math.cos(2.0 * math.pi * float(i) / float(N)) - 1.0) / d ** 2.0
        for i in range(half + 1, N):
            k[i] = 2.0 * (math.cos(2.0 * math.pi * float(-N + i) / float(N)) - 1.0) / d ** 2.0
        return k


# ---------------------------------------------------------------------------
# boundary conditions (boundary_conditions.f90), global single-domain view

def per_x(F, g, fid):
    """apply_periodic_bc_x (boundary_conditions.f90:60-79)."""
    if fid == 1:
        F[1] = F[g.nx - 1]
        F[g.nx] = F[2]
    else:
        F[1] = F[g.nxg - 2]
        F[g.nxg - 1] = F[2]
        F[g.nxg] = F[3]


def per_z(F, g, fid):
    """apply_periodic_bc_z (boundary_conditions.f90:84-226), intended P>=2
    semantics: faces (id 3) F(1)=F(nz-1), F(nz)=F(2); centres F(1)=F(nzg-2),
    F(nzg-1)=F(2), F(nzg)=F(3).  Buffers are taken before any write."""
    if fid == 3:
        a, b = F[:, :, g.nz - 1].copy(), F[:, :, 2].copy()
        F[:, :, 1] = a
        F[:, :, g.nz] = b
    else:
        a, b, c = F[:, :, g.nzg - 2].copy(), F[:, :, 2].copy(), F[:, :, 3].copy()
        F[:, :, 1] = a
        F[:, :, g.nzg - 1] = b
        F[:, :, g.nzg] = c


def dir_y(F, g, fid):
    """apply_Dirichlet_bc_y (boundary_conditions.f90:239-254)."""
    if fid == 1:
        F[:, 1, :] = 0.0
        F[:, g.ny, :] = 0.0
    else:
        F[:, 1, :] = -F[:, 2, :]
        F[:, g.nyg, :] = -F[:, g.nyg - 1, :]


def neu_y(F, g, fid):
    """apply_Neumann_bc_y (boundary_conditions.f90:266-281)."""
    if fid == 1:
        F[:, 1, :] = F[:, 2, :]
        F[:, g.ny, :] = F[:, g.ny - 1, :]
    else:
        F[:, 1, :] = F[:, 2, :]
        F[:, g.nyg, :] = F[:, g.nyg - 1, :]


# ---------------------------------------------------------------------------
# filters (subgrid.f90:140-190)
_FIL = {(-1, -1): 1.0 / 36.0, (1, 1): 1.0 / 36.0, (-1, 1): 1.0 / 36.0, (1, -1): 1.0 / 36.0,
        (0, 1): 1.0 / 9.0, (1, 0): 1.0 / 9.0, (0, -1): 1.0 / 9.0, (-1, 0): 1.0 / 9.0,
        (0, 0): 4.0 / 9.0}


def filter_xzy(Uin):
    """filter_xzy(U_, Uf_) of subgrid.f90:140-190 on a 0-based view ``Uin`` of
    shape (n1,n2,n3); returns the (n1-2, n2, n3-2) block written to
    ``Uf_(ii-1, j, kk-1)`` for ii=2..n1-1, kk=2..n3-1."""
    n1, n2, n3 = Uin.shape
    Y = np.empty_like(Uin)
    Y[:, 1:n2 - 1, :] = (1.0 / 6.0 * Uin[:, 0:n2 - 2, :] + 2.0 / 3.0 * Uin[:, 1:n2 - 1, :]
                         + 1.0 / 6.0 * Uin[:, 2:n2, :])
    Y[:, 0, :] = 2.0 / 3.0 * Uin[:, 0, :] + 1.0 / 3.0 * Uin[:, 1, :]
    Y[:, n2 - 1, :] = 1.0 / 3.0 * Uin[:, n2 - 2, :] + 2.0 / 3.0 * Uin[:, n2 - 1, :]
    out = np.zeros((n1 - 2, n2, n3 - 2))
    for i in (-1, 0, 1):
        for k in (-1, 0, 1):
            out += Y[1 + i:n1 - 1 + i, :, 1 + k:n3 - 1 + k] * _FIL[(i, k)]
    return out


def _iavg(u, axis):
    """interpolate_x / interpolate_z (any di) and interpolate_y with di=1
    (interpolation.f90:24-105) of the section ``u`` along ``axis``:
    ui(m) = 0.5 (u(m) + u(m+1)), one point shorter than ``u``."""
    n = u.shape[axis]
    lo = [slice(None)] * 3
    hi = [slice(None)] * 3
    lo[axis] = slice(0, n - 1)
    hi[axis] = slice(1, n)
    return 0.5 * (u[tuple(lo)] + u[tuple(hi)])


# ---------------------------------------------------------------------------
class ChannelOracle:
    """One channel instance; state and subroutines of the reference's hot path."""

    def __init__(self, grid: Grid, params: Params):
        g = self.g = grid
        self.p = params
        self.U = alloc(g.nx, g.nyg, g.nzg)
        self.V = alloc(g.nxg, g.ny, g.nzg)
        self.W = alloc(g.nxg, g.nyg, g.nz)
        self.P = alloc(g.nxg, g.nyg, g.nzg)
        self.nu_t = alloc(g.nxg, g.nyg, g.nzg)
        self.rhs_p = alloc(g.nxg, g.nyg, g.nzg)      # allocated (2:nxg-1,2:nyg-1,2:nzg)
        self.alpha_x = np.zeros((g.nx + 1, 3, g.nzg + 1))
        self.dPdx = params.dPdx
        self.t = 0.0
        self.dt = 0.0
        self.Qflow_x_0 = 0.0
        # learned wall model (WM_MLP, oracle/mlp_wm_ref.py): network
        # parameters (None: zero network), optional per-stage actions
        # callable(stage) -> (Nx, 2, Nz) float32 in place of the network's,
        # the nu + nu_t field of the previous stage's wall-model pass (zero
        # before the first, as a new GPU handle holds it), and the last
        # evaluation's features and actions per stage
        self.mlp_theta = None
        self.mlp_actions = None
        self.mlp_nutot = alloc(g.nxg, g.nyg, g.nzg)
        self.mlp_info = [None, None, None]

    # -- state I/O ---------------------------------------------------------
    def set_fields(self, U, V, W):
        """Load Fortran-shaped (unpadded) fields, apply BCs and set the
        initial bulk flow (initialization.f90:442)."""
        self.U[1:, 1:, 1:] = U
        self.V[1:, 1:, 1:] = V
        self.W[1:, 1:, 1:] = W
        self.apply_boundary_conditions()
        self.Qflow_x_0 = self.compute_mean_mass_flow_U(self.U)

    def fields(self):
        return (self.U[1:, 1:, 1:].copy(), self.V[1:, 1:, 1:].copy(), self.W[1:, 1:, 1:].copy())

    def set_wall_stress(self, alpha_unique):
        """alpha_unique: (Nx, 2, Nz) wall stress at U wall points (faces
        i=2..nx-1, centres k=2..nzg-2); ghosts filled periodically as
        smarties_stat.f90:249-251 does."""
        g = self.g
        a = self.alpha_x
        a[2:g.nx, 1:3, 2:g.nzg - 1] = alpha_unique
        per_x(a, g, 1)
        a2 = a[:, :, :]
        c1, c2, c3 = a2[:, :, g.nzg - 2].copy(), a2[:, :, 2].copy(), a2[:, :, 3].copy()
        a2[:, :, 1], a2[:, :, g.nzg - 1], a2[:, :, g.nzg] = c1, c2, c3

    # -- boundary conditions (boundary_conditions.f90:20-48) ---------------
    def apply_boundary_conditions(self):
        g = self.g
        per_x(self.U, g, 1)
        per_x(self.V, g, 2)
        per_x(self.W, g, 2)
        per_z(self.U, g, 1)
        per_z(self.V, g, 2)
        per_z(self.W, g, 3)
        dir_y(self.U, g, 2)
        dir_y(self.V, g, 1)
        dir_y(self.W, g, 2)

    # -- dt (time_integration.f90:102-150) ----------------------------------
    def compute_dt(self):
        g, p = self.g, self.p
        I, J, K = slice(2, g.nxg), slice(2, g.nyg), slice(2, g.nzg)
        with np.errstate(divide="ignore"):
            dxs = (g.xg[3:g.nxg + 1] - g.xg[2:g.nxg])[:, None, None]
            dys = (g.yg[3:g.nyg + 1] - g.yg[2:g.nyg])[None, :, None]
            dzs = (g.zg[3:g.nzg + 1] - g.zg[2:g.nzg])[None, None, :]
            lU = max(0.0, float(np.max(dxs / np.abs(self.U[I, J, K]))))
            lV = max(0.0, float(np.max(dys / np.abs(self.V[I, J, K]))))
            lW = max(0.0, float(np.max(dzs / np.abs(self.W[I, J, K]))))
        dt_conv = min(p.CFL * lU, p.CFL * lV, p.CFL * lW)
        dt_vis = min(p.CFL * g.dxmin ** 2.0 / p.nu, p.CFL * g.dymin ** 2.0 / p.nu,
                     p.CFL * g.dzmin ** 2.0 / p.nu)
        dt = min(dt_conv, dt_vis)
        dt = min(dt, 1e-3)
        if p.CFL < 0:
            dt = -p.CFL
        self.dt = dt
        return dt

    # -- compute_Sij (subgrid.f90:1014-1072) --------------------------------
    def compute_Sij(self, U, V, W):
        g = self.g
        nxg, nyg, nzg = g.nxg, g.nyg, g.nzg
        x, y, z, xg, yg, zg = g.x, g.y, g.z, g.xg, g.yg, g.zg
        Sij = np.zeros((nxg + 1, nyg + 1, nzg + 1, 7))
        I, J, K = slice(2, nxg), slice(2, nyg), slice(2, nzg)
        Sij[I, J, K, 1] = (U[I, J, K] - U[1:nxg - 1, J, K]) / (x[2:nxg] - x[1:nxg - 1])[:, None, None]
        Sij[I, J, K, 2] = (V[I, J, K] - V[I, 1:nyg - 1, K]) / (y[2:nyg] - y[1:nyg - 1])[None, :, None]
        Sij[I, J, K, 3] = (W[I, J, K] - W[I, J, 1:nzg - 1]) / (z[2:nzg] - z[1:nzg - 1])[None, None, :]
        Ie, Je, Ke = slice(2, nxg + 1), slice(2, nyg + 1), slice(2, nzg + 1)
        Im, Jm, Km = slice(1, nxg), slice(1, nyg), slice(1, nzg)
        dyg = (yg[2:nyg + 1] - yg[1:nyg])[None, :, None]
        dxg = (xg[2:nxg + 1] - xg[1:nxg])[:, None, None]
        dzg = (zg[2:nzg + 1] - zg[1:nzg])[None, None, :]
        Sij[Ie, Je, Ke, 4] = 0.5 * ((U[Im, Je, Ke] - U[Im, Jm, Ke]) / dyg
                                    + (V[Ie, Jm, Ke] - V[Im, Jm, Ke]) / dxg)
        Sij[Ie, Je, Ke, 5] = 0.5 * ((U[Im, Je, Ke] - U[Im, Je, Km]) / dzg
                                    + (W[Ie, Je, Km] - W[Im, Je, Km]) / dxg)
        Sij[Ie, Je, Ke, 6] = 0.5 * ((V[Ie, Jm, Ke] - V[Ie, Jm, Km]) / dzg
                                    + (W[Ie, Je, Km] - W[Ie, Jm, Km]) / dyg)
        # edges -> centres; the in-place Fortran loop only reads points not yet
        # overwritten, so an out-of-place average is identical
        Ip, Jp, Kp = slice(3, nxg + 1), slice(3, nyg + 1), slice(3, nzg + 1)
        s4 = Sij[:, :, :, 4].copy(); s5 = Sij[:, :, :, 5].copy(); s6 = Sij[:, :, :, 6].copy()
        Sij[I, J, K, 4] = 0.25 * (s4[I, J, K] + s4[Ip, J, K] + s4[I, Jp, K] + s4[Ip, Jp, K])
        Sij[I, J, K, 5] = 0.25 * (s5[I, J, K] + s5[Ip, J, K] + s5[I, J, Kp] + s5[Ip, J, Kp])
        Sij[I, J, K, 6] = 0.25 * (s6[I, J, K] + s6[I, Jp, K] + s6[I, J, Kp] + s6[I, Jp, Kp])
        S = np.zeros((nxg + 1, nyg + 1, nzg + 1))
        acc = np.zeros_like(S[I, J, K])
        for m in range(1, 7):
            c = 2.0 if m <= 3 else 4.0
            acc = acc + c * Sij[I, J, K, m] * Sij[I, J, K, m]
        S[I, J, K] = acc ** 0.5
        return Sij, S

    # -- dynamic Smagorinsky (subgrid.f90:379-537) --------------------------
    def sgs_dynamic_Smagorinsky(self):
        g, p = self.g, self.p
        nx, ny, nz, nxg, nyg, nzg = g.nx, g.ny, g.nz, g.nxg, g.nyg, g.nzg
        U, V, W = self.U, self.V, self.W
        term = alloc(nxg, nyg, nzg)
        term_1 = alloc(nxg, nyg, nzg)
        term_2 = alloc(nxg, nyg, nzg)
        # part 1: Leonard term (subgrid.f90:394-432)
        term[2:nxg, 1:, 1:] = 0.5 * (U[1:nx, 1:, 1:] + U[2:nx + 1, 1:, 1:])
        term_1[1:, 2:nyg, 1:] = 0.5 * (V[1:, 1:ny, 1:] + V[1:, 2:ny + 1, 1:])
        term_2[1:, 1:, 2:nz + 1] = 0.5 * (W[1:, 1:, 1:nz] + W[1:, 1:, 2:nz + 1])
        term_2[1:, 1:, nzg] = 0.0
        per_x(term, g, 2)
        per_z(term_2, g, 4)
        uc = (term, term_1, term_2)
        pairs = ((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2))
        ten = np.zeros((nxg + 1, nyg + 1, nzg + 1, 7))
        for m, (a, b) in enumerate(pairs, start=1):
            ten[2:nxg + 1, 2:nyg, 2:nzg + 1, m] = uc[a][2:nxg + 1, 2:nyg, 2:nzg + 1] * uc[b][2:nxg + 1, 2:nyg, 2:nzg + 1]
            per_x(ten[:, :, :, m], g, 2)
            per_z(ten[:, :, :, m], g, 4)
        I, J, K = slice(2, nxg), slice(2, nyg), slice(2, nzg)
        Lij = np.zeros((nxg + 1, nyg + 1, nzg + 1, 7))
        for m in range(1, 7):
            Lij[I, J, K, m] = filter_xzy(ten[1:nxg + 1, 2:nyg, 1:nzg + 1, m])
        fu = [filter_xzy(c[1:nxg + 1, 2:nyg, 1:nzg + 1]) for c in uc]
        for m, (a, b) in enumerate(pairs, start=1):
            Lij[I, J, K, m] = Lij[I, J, K, m] - fu[a] * fu[b]
        # part 2: Mij (subgrid.f90:434-476)
        Uf = alloc(nx, nyg, nzg)
        Vf = alloc(nxg, ny, nzg)
        Wf = alloc(nxg, nyg, nz)
        Uf[2:nx, 1:nyg + 1, 2:nzg] = filter_xzy(U[1:nx + 1, 1:nyg + 1, 1:nzg + 1])
        Vf[2:nxg, 1:ny + 1, 2:nzg] = filter_xzy(V[1:nxg + 1, 1:ny + 1, 1:nzg + 1])
        Wf[2:nxg, 1:nyg + 1, 2:nz] = filter_xzy(W[1:nxg + 1, 1:nyg + 1, 1:nz + 1])
        per_x(Uf, g, 1); per_z(Uf, g, 1)
        per_x(Vf, g, 2); per_z(Vf, g, 2)
        per_x(Wf, g, 2); per_z(Wf, g, 3)
        Sh, Shat = self.compute_Sij(Uf, Vf, Wf)
        Mij = np.zeros((nxg + 1, nyg + 1, nzg + 1, 7))
        for m in range(1, 7):
            Mij[I, J, K, m] = 2.0 ** 2.0 * Shat[I, J, K] * Sh[I, J, K, m]
        Sr, S = self.compute_Sij(U, V, W)
        for m in range(1, 7):
            t = alloc(nxg, nyg, nzg)
            t[I, J, K] = S[I, J, K] * Sr[I, J, K, m]
            per_x(t, g, 2)
            per_z(t, g, 4)
            Mij[I, J, K, m] = Mij[I, J, K, m] - filter_xzy(t[1:nxg + 1, 2:nyg, 1:nzg + 1])
        # part 3 (subgrid.f90:481-535)
        L, M = Lij[I, J, K], Mij[I, J, K]
        LM = (L[..., 1] * M[..., 1] + L[..., 2] * M[..., 2] + L[..., 3] * M[..., 3]
              + 2.0 * (L[..., 4] * M[..., 4] + L[..., 5] * M[..., 5] + L[..., 6] * M[..., 6]))
        MM = (M[..., 1] * M[..., 1] + M[..., 2] * M[..., 2] + M[..., 3] * M[..., 3]
              + 2.0 * (M[..., 4] * M[..., 4] + M[..., 5] * M[..., 5] + M[..., 6] * M[..., 6]))
        LMs = LM.sum(axis=(0, 2))
        MMs = MM.sum(axis=(0, 2))
        ratio = LMs / MMs
        nu_t = alloc(nxg, nyg, nzg)
        nu_t[I, J, K] = -0.5 * ratio[None, :, None] * S[I, J, K]
        per_x(nu_t, g, 2)
        per_z(nu_t, g, 4)
        nu_t = np.maximum(nu_t, 0.0)
        if p.Dirichlet_nu_t == 1:
            dir_y(nu_t, g, 2)
        else:
            neu_y(nu_t, g, 2)
        self.nu_t = nu_t
        self.dsm_planes = (LMs, MMs)
        return nu_t

    # -- static Smagorinsky (subgrid.f90:563-612, written from its formula) --
    def sgs_Smagorinsky(self):
        g, p = self.g, self.p
        nxg, nyg, nzg = g.nxg, g.nyg, g.nzg
        _, S = self.compute_Sij(self.U, self.V, self.W)
        nu_t = self.nu_t.copy()
        utau_t = self.dPdx ** 0.5
        with np.errstate(divide="ignore"):
            ls = p.nu / utau_t if utau_t != 0.0 else math.inf
        for j in range(2, nyg):
            if j < nyg // 2:
                f = 1.0 - math.exp(-(g.yg[j] - g.y[1]) / 25.0 / ls)
            else:
                f = 1.0 - math.exp(-(g.y[g.ny] - g.yg[j]) / 25.0 / ls)
            if p.Dirichlet_nu_t == 0:
                f = 1.0
            Delta = (g.dxmin * g.dzmin * (g.y[j] - g.y[j - 1])) ** (1.0 / 3.0)
            nu_t[2:nxg, j, 2:nzg] = ((p.Cs * Delta * f) ** 2.0) * S[2:nxg, j, 2:nzg]
        per_x(nu_t, g, 2)
        per_z(nu_t, g, 4)
        nu_t = np.maximum(nu_t, 0.0)
        if p.Dirichlet_nu_t == 1:
            dir_y(nu_t, g, 2)
        else:
            neu_y(nu_t, g, 2)
        self.nu_t = nu_t
        return nu_t

    # -- ghost rows of the AMD and Vreman models (subgrid.f90:858-871, 991-1002)
    def _nut_ghost_rows_amd_vreman(self, nu_t):
        g, p = self.g, self.p
        per_x(nu_t, g, 2)
        per_z(nu_t, g, 4)
        if p.Dirichlet_nu_t == 1:
            dir_y(nu_t, g, 2)
        elif p.Dirichlet_nu_t == 0:
            neu_y(nu_t, g, 2)
        elif p.Dirichlet_nu_t == 2:
            c = 2.0 * 0.38 * self.dPdx ** 0.5 * (g.y[2] - g.y[1]) / 2.0
            nu_t[:, 1, :] = -nu_t[:, 2, :] + c
            nu_t[:, g.nyg, :] = -nu_t[:, g.nyg - 1, :] + c
        return nu_t

    # -- anisotropic minimum dissipation (subgrid.f90:632-874) ---------------
    def sgs_AMD(self):
        """nu_t = max(0, -C sum_k (d^_k u_i)(d^_k u_j) S_ij / (d_k u_l)^2), C = 0.3,
        restated statement by statement: d^ are grid-scaled differences
        interpolated to centres in the reference's order; the interior centres
        (the only ones that survive the ghost-row rules) are evaluated."""
        g = self.g
        nx, ny, nz, nxg, nyg, nzg = g.nx, g.ny, g.nz, g.nxg, g.nyg, g.nzg
        x, y, z, xg, yg, zg = g.x, g.y, g.z, g.xg, g.yg, g.zg
        U, V, W = self.U, self.V, self.W
        Cp = 0.3
        Sij, _ = self.compute_Sij(U, V, W)
        S = [None] + [Sij[:, :, :, m] for m in range(1, 7)]
        sh = (nxg + 1, nyg + 1, nzg + 1)
        t, t1, t2, t3, t4 = (np.zeros(sh) for _ in range(5))
        B = (slice(2, nxg), slice(2, nyg), slice(2, nzg))
        nu = np.zeros(sh)
        ax = _iavg
        dyg = (yg[2:nyg + 1] - yg[1:nyg])[None, :, None]
        dzg = (zg[2:nzg + 1] - zg[1:nzg])[None, None, :]
        dxg = (xg[2:nxg + 1] - xg[1:nxg])[:, None, None]
        # (d^ U)^2 S11 and (d U)^2 (subgrid.f90:650-681)
        t2[2:nx + 1] = U[2:nx + 1] - U[1:nx]
        t4[2:nx + 1] = (U[2:nx + 1] - U[1:nx]) ** 2.0 / ((x[2:nx + 1] - x[1:nx]) ** 2.0)[:, None, None]
        nu[B] = t2[B] ** 2.0 * S[1][B]
        t[1:nx + 1, 2:nyg + 1] = U[1:nx + 1, 2:nyg + 1] - U[1:nx + 1, 1:nyg]
        t1[1:nx + 1, 2:nyg + 1] = t[1:nx + 1, 2:nyg + 1] / dyg
        t2[2:nx + 1, 2:nyg + 1] = ax(t1[1:nx + 1, 2:nyg + 1], 0)
        t3[2:nx + 1, 2:nyg] = ax(t2[2:nx + 1, 2:nyg + 1], 1)
        t4 = t4 + t3 ** 2.0
        t1[2:nx + 1, 2:nyg + 1] = ax(t[1:nx + 1, 2:nyg + 1], 0)
        t2[2:nx + 1, 2:nyg] = ax(t1[2:nx + 1, 2:nyg + 1], 1)
        nu[B] = nu[B] + t2[B] ** 2.0 * S[1][B]
        t[1:nx + 1, :, 2:nzg + 1] = U[1:nx + 1, :, 2:nzg + 1] - U[1:nx + 1, :, 1:nzg]
        t1[1:nx + 1, :, 2:nzg + 1] = t[1:nx + 1, :, 2:nzg + 1] / dzg
        t2[2:nx + 1, :, 2:nzg + 1] = ax(t1[1:nx + 1, :, 2:nzg + 1], 0)
        t3[2:nx + 1, :, 2:nzg] = ax(t2[2:nx + 1, :, 2:nzg + 1], 2)
        t4 = t4 + t3 ** 2.0
        t1[2:nx + 1, :, 2:nzg + 1] = ax(t[1:nx + 1, :, 2:nzg + 1], 0)
        t2[2:nx + 1, :, 2:nzg] = ax(t1[2:nx + 1, :, 2:nzg + 1], 2)
        nu[B] = nu[B] + t2[B] ** 2.0 * S[1][B]
        # V (subgrid.f90:683-716)
        t2[:, 2:ny + 1] = V[:, 2:ny + 1] - V[:, 1:ny]
        t4[:, 2:ny + 1] = t4[:, 2:ny + 1] + t2[:, 2:ny + 1] ** 2.0 / ((y[2:ny + 1] - y[1:ny]) ** 2.0)[None, :, None]
        nu[B] = nu[B] + t2[B] ** 2.0 * S[2][B]
        t[2:nxg + 1, 1:ny + 1] = V[2:nxg + 1, 1:ny + 1] - V[1:nxg, 1:ny + 1]
        t1[2:nxg + 1, 1:ny + 1] = t[2:nxg + 1, 1:ny + 1] / dxg
        t2[2:nxg + 1, 2:ny + 1] = ax(t1[2:nxg + 1, 1:ny + 1], 1)
        t3[2:nxg, 2:ny + 1] = ax(t2[2:nxg + 1, 2:ny + 1], 0)
        t4 = t4 + t3 ** 2.0
        t1[2:nxg + 1, 2:ny + 1] = ax(t[2:nxg + 1, 1:ny + 1], 1)
        t2[2:nxg, 2:ny + 1] = ax(t1[2:nxg + 1, 2:ny + 1], 0)
        nu[B] = nu[B] + t2[B] ** 2.0 * S[2][B]
        t[:, 1:ny + 1, 2:nzg + 1] = V[:, 1:ny + 1, 2:nzg + 1] - V[:, 1:ny + 1, 1:nzg]
        t1[:, 1:ny + 1, 2:nzg + 1] = t[:, 1:ny + 1, 2:nzg + 1] / dzg
        t2[:, 2:ny + 1, 2:nzg + 1] = ax(t1[:, 1:ny + 1, 2:nzg + 1], 1)
        t3[:, 2:ny + 1, 2:nzg] = ax(t2[:, 2:ny + 1, 2:nzg + 1], 2)
        t4 = t4 + t3 ** 2.0
        t1[:, 2:ny + 1, 2:nzg + 1] = ax(t[:, 1:ny + 1, 2:nzg + 1], 1)
        t2[:, 2:ny + 1, 2:nzg] = ax(t1[:, 2:ny + 1, 2:nzg + 1], 2)
        nu[B] = nu[B] + t2[B] ** 2.0 * S[2][B]
        # W (subgrid.f90:718-749)
        t2[:, :, 2:nz + 1] = (W[:, :, 2:nz + 1] - W[:, :, 1:nz]) ** 2.0
        t4[:, :, 2:nz + 1] = t4[:, :, 2:nz + 1] + t2[:, :, 2:nz + 1] / ((z[2:nz + 1] - z[1:nz]) ** 2.0)[None, None, :]
        nu[B] = nu[B] + t2[B] * S[3][B]
        t[2:nxg + 1, :, 1:nz + 1] = W[2:nxg + 1, :, 1:nz + 1] - W[1:nxg, :, 1:nz + 1]
        t1[2:nxg + 1, :, 1:nz + 1] = t[2:nxg + 1, :, 1:nz + 1] / dxg
        t2[2:nxg + 1, :, 2:nz + 1] = ax(t1[2:nxg + 1, :, 1:nz + 1], 2)
        t3[2:nxg, :, 2:nz + 1] = ax(t2[2:nxg + 1, :, 2:nz + 1], 0)
        t4 = t4 + t3 ** 2.0
        t1[2:nxg + 1, :, 2:nz + 1] = ax(t[2:nxg + 1, :, 1:nz + 1], 2)
        t2[2:nxg, :, 2:nz + 1] = ax(t1[2:nxg + 1, :, 2:nz + 1], 0)
        nu[B] = nu[B] + t2[B] ** 2.0 * S[3][B]
        t[:, 2:nyg + 1, 1:nz + 1] = W[:, 2:nyg + 1, 1:nz + 1] - W[:, 1:nyg, 1:nz + 1]
        t1[:, 2:nyg + 1, 1:nz + 1] = t[:, 2:nyg + 1, 1:nz + 1] / dyg
        t2[:, 2:nyg + 1, 2:nz + 1] = ax(t1[:, 2:nyg + 1, 1:nz + 1], 2)
        t3[:, 2:nyg, 2:nz + 1] = ax(t2[:, 2:nyg + 1, 2:nz + 1], 1)
        t4 = t4 + t3 ** 2.0
        t1[:, 2:nyg + 1, 2:nz + 1] = ax(t[:, 2:nyg + 1, 1:nz + 1], 2)
        t2[:, 2:nyg, 2:nz + 1] = ax(t1[:, 2:nyg + 1, 2:nz + 1], 1)
        nu[B] = nu[B] + t2[B] ** 2.0 * S[3][B]
        nu = self._amd_cross_terms(nu, S, B)
        with np.errstate(divide="ignore", invalid="ignore"):
            out = alloc(nxg, nyg, nzg)
            out[B] = -Cp * nu[B] / t4[B]
        out = np.maximum(out, 0.0)
        self.nu_t = self._nut_ghost_rows_amd_vreman(out)
        self.amd_terms = (nu, t4)
        return self.nu_t

    def _amd_cross_terms(self, nu, S, B):
        """2 (d^_k u_i)(d^_k u_j) S_ij, i != j (subgrid.f90:751-851)."""
        g = self.g
        nx, ny, nz, nxg, nyg, nzg = g.nx, g.ny, g.nz, g.nxg, g.nyg, g.nzg
        U, V, W = self.U, self.V, self.W
        sh = (nxg + 1, nyg + 1, nzg + 1)
        t, t1, t2 = (np.zeros(sh) for _ in range(3))
        ax = _iavg
        # S12: k = x, y, z
        t[2:nxg + 1, 1:ny + 1] = V[2:nxg + 1, 1:ny + 1] - V[1:nxg, 1:ny + 1]
        t1[2:nxg + 1, 2:ny + 1] = ax(t[2:nxg + 1, 1:ny + 1], 1)
        t2[2:nxg, 2:ny + 1] = ax(t1[2:nxg + 1, 2:ny + 1], 0)
        t1[2:nx + 1, 2:nyg] = t2[2:nx + 1, 2:nyg] * (U[2:nx + 1, 2:nyg] - U[1:nx, 2:nyg])
        nu[B] = nu[B] + 2.0 * t1[B] * S[4][B]
        t[1:nx + 1, 2:nyg + 1] = U[1:nx + 1, 2:nyg + 1] - U[1:nx + 1, 1:nyg]
        t1[2:nx + 1, 2:nyg + 1] = ax(t[1:nx + 1, 2:nyg + 1], 0)
        t2[2:nx + 1, 2:nyg] = ax(t1[2:nx + 1, 2:nyg + 1], 1)
        t1[2:nxg, 2:ny + 1] = t2[2:nxg, 2:ny + 1] * (V[2:nxg, 2:ny + 1] - V[2:nxg, 1:ny])
        nu[B] = nu[B] + 2.0 * t1[B] * S[4][B]
        t[1:nx + 1, :, 2:nzg + 1] = U[1:nx + 1, :, 2:nzg + 1] - U[1:nx + 1, :, 1:nzg]
        t1[2:nx + 1, :, 2:nzg + 1] = ax(t[1:nx + 1, :, 2:nzg + 1], 0)
        t[:, 1:ny + 1, 2:nzg + 1] = V[:, 1:ny + 1, 2:nzg + 1] - V[:, 1:ny + 1, 1:nzg]
        t2[:, 2:ny + 1, 2:nzg + 1] = ax(t[:, 1:ny + 1, 2:nzg + 1], 1)
        t3 = t1 * t2
        t1[2:nxg, 2:nyg, 2:nzg] = ax(t3[2:nxg, 2:nyg, 2:nzg + 1], 2)
        nu[B] = nu[B] + 2.0 * t1[B] * S[4][B]
        # S13: k = x, z, y
        t[2:nxg + 1, :, 1:nz + 1] = W[2:nxg + 1, :, 1:nz + 1] - W[1:nxg, :, 1:nz + 1]
        t1[2:nxg + 1, :, 2:nz + 1] = ax(t[2:nxg + 1, :, 1:nz + 1], 2)
        t2[2:nxg, :, 2:nz + 1] = ax(t1[2:nxg + 1, :, 2:nz + 1], 0)
        t1[2:nx + 1, 2:nyg] = t2[2:nx + 1, 2:nyg] * (U[2:nx + 1, 2:nyg] - U[1:nx, 2:nyg])
        nu[B] = nu[B] + 2.0 * t1[B] * S[5][B]
        t[1:nx + 1, :, 2:nzg + 1] = U[1:nx + 1, :, 2:nzg + 1] - U[1:nx + 1, :, 1:nzg]
        t1[2:nx + 1, :, 2:nzg + 1] = ax(t[1:nx + 1, :, 2:nzg + 1], 0)
        t2[2:nx + 1, :, 2:nzg] = ax(t1[2:nx + 1, :, 2:nzg + 1], 2)
        t1[2:nxg, :, 2:nz + 1] = t2[2:nxg, :, 2:nz + 1] * (W[2:nxg, :, 2:nz + 1] - W[2:nxg, :, 1:nz])
        nu[B] = nu[B] + 2.0 * t1[B] * S[5][B]
        t[1:nx + 1, 2:nyg + 1] = U[1:nx + 1, 2:nyg + 1] - U[1:nx + 1, 1:nyg]
        t1[2:nx + 1, 2:nyg + 1] = ax(t[1:nx + 1, 2:nyg + 1], 0)
        t[:, 2:nyg + 1, 1:nz + 1] = W[:, 2:nyg + 1, 1:nz + 1] - W[:, 1:nyg, 1:nz + 1]
        t2[:, 2:nyg + 1, 2:nz + 1] = ax(t[:, 2:nyg + 1, 1:nz + 1], 2)
        t3 = t1 * t2
        t1[2:nxg, 2:nyg, 2:nzg] = ax(t3[2:nxg, 2:nyg + 1, 2:nzg], 1)
        nu[B] = nu[B] + 2.0 * t1[B] * S[5][B]
        # S23: k = y, z, x
        t[:, 2:nyg + 1, 1:nz + 1] = W[:, 2:nyg + 1, 1:nz + 1] - W[:, 1:nyg, 1:nz + 1]
        t1[:, 2:nyg + 1, 2:nz + 1] = ax(t[:, 2:nyg + 1, 1:nz + 1], 2)
        t2[:, 2:nyg, 2:nz + 1] = ax(t1[:, 2:nyg + 1, 2:nz + 1], 1)
        t1[2:nxg, 2:ny + 1] = t2[2:nxg, 2:ny + 1] * (V[2:nxg, 2:ny + 1] - V[2:nxg, 1:ny])
        nu[B] = nu[B] + 2.0 * t1[B] * S[6][B]
        t[:, 1:ny + 1, 2:nzg + 1] = V[:, 1:ny + 1, 2:nzg + 1] - V[:, 1:ny + 1, 1:nzg]
        t1[:, 2:ny + 1, 2:nzg + 1] = ax(t[:, 1:ny + 1, 2:nzg + 1], 1)
        t2[:, 2:ny + 1, 2:nzg] = ax(t1[:, 2:ny + 1, 2:nzg + 1], 2)
        t1[:, 2:nyg, 2:nz + 1] = t2[:, 2:nyg, 2:nz + 1] * (W[:, 2:nyg, 2:nz + 1] - W[:, 2:nyg, 1:nz])
        nu[B] = nu[B] + 2.0 * t1[B] * S[6][B]
        t[2:nxg + 1, 1:ny + 1] = V[2:nxg + 1, 1:ny + 1] - V[1:nxg, 1:ny + 1]
        t1[2:nxg + 1, 2:ny + 1] = ax(t[2:nxg + 1, 1:ny + 1], 1)
        t[2:nxg + 1, :, 1:nz + 1] = W[2:nxg + 1, :, 1:nz + 1] - W[1:nxg, :, 1:nz + 1]
        t2[2:nxg + 1, :, 2:nz + 1] = ax(t[2:nxg + 1, :, 1:nz + 1], 2)
        t3 = t1 * t2
        t1[2:nxg, 2:nyg, 2:nzg] = ax(t3[2:nxg + 1, 2:nyg, 2:nzg], 0)
        nu[B] = nu[B] + 2.0 * t1[B] * S[6][B]
        return nu

    # -- Vreman (subgrid.f90:897-1004) ---------------------------------------
    def sgs_Vreman(self):
        """nu_t = C sqrt(B_b / a_ij a_ij), C = 2.5 (0.1)^2, b_ij = sum_m d_m^2
        a_mi a_mj with a_ij = du_j/dx_i at centres (off-diagonals: mean of the
        four surrounding edge derivatives).  The U sections written 2:ny and
        1:ny-1 where 2:nx and 1:nx-1 are meant (subgrid.f90:930-931,946-947)
        start at the same index, so element-wise they read the intended U
        values; that reading is restated here.  No clipping, as written."""
        g = self.g
        nxg, nyg, nzg = g.nxg, g.nyg, g.nzg
        x, y, z, xg, yg, zg = g.x, g.y, g.z, g.xg, g.yg, g.zg
        U, V, W = self.U, self.V, self.W
        C = 2.5 * (0.1 ** 2.0)
        I, J, K = slice(2, nxg), slice(2, nyg), slice(2, nzg)      # 2..n?g-1
        Ip, Jp, Kp = slice(3, nxg + 1), slice(3, nyg + 1), slice(3, nzg + 1)
        Im, Jm, Km = slice(1, nxg - 1), slice(1, nyg - 1), slice(1, nzg - 1)
        dxl = (xg[2:nxg] - xg[1:nxg - 1])[:, None, None]            # xg(i)-xg(i-1)
        dxr = (xg[3:nxg + 1] - xg[2:nxg])[:, None, None]            # xg(i+1)-xg(i)
        dyl = (yg[2:nyg] - yg[1:nyg - 1])[None, :, None]
        dyr = (yg[3:nyg + 1] - yg[2:nyg])[None, :, None]
        dzl = (zg[2:nzg] - zg[1:nzg - 1])[None, None, :]
        dzr = (zg[3:nzg + 1] - zg[2:nzg])[None, None, :]
        a = [None] * 10
        a[1] = (U[I, J, K] - U[Im, J, K]) / (x[2:nxg] - x[1:nxg - 1])[:, None, None]
        a[4] = (0.25 * (V[I, J, K] - V[Im, J, K]) / dxl + 0.25 * (V[I, Jm, K] - V[Im, Jm, K]) / dxl
                + 0.25 * (V[Ip, J, K] - V[I, J, K]) / dxr + 0.25 * (V[Ip, Jm, K] - V[I, Jm, K]) / dxr)
        a[5] = (0.25 * (W[I, J, K] - W[Im, J, K]) / dxl + 0.25 * (W[I, J, Km] - W[Im, J, Km]) / dxl
                + 0.25 * (W[Ip, J, K] - W[I, J, K]) / dxr + 0.25 * (W[Ip, J, Km] - W[I, J, Km]) / dxr)
        a[2] = (V[I, J, K] - V[I, Jm, K]) / (y[2:nyg] - y[1:nyg - 1])[None, :, None]
        a[7] = (0.25 * (U[I, J, K] - U[I, Jm, K]) / dyl + 0.25 * (U[Im, J, K] - U[Im, Jm, K]) / dyl
                + 0.25 * (U[I, Jp, K] - U[I, J, K]) / dyr + 0.25 * (U[Im, Jp, K] - U[Im, J, K]) / dyr)
        a[6] = (0.25 * (W[I, J, K] - W[I, Jm, K]) / dyl + 0.25 * (W[I, J, Km] - W[I, Jm, Km]) / dyl
                + 0.25 * (W[I, Jp, K] - W[I, J, K]) / dyr + 0.25 * (W[I, Jp, Km] - W[I, J, Km]) / dyr)
        a[3] = (W[I, J, K] - W[I, J, Km]) / (z[2:nzg] - z[1:nzg - 1])[None, None, :]
        a[8] = (0.25 * (U[I, J, K] - U[I, J, Km]) / dzl + 0.25 * (U[Im, J, K] - U[Im, J, Km]) / dzl
                + 0.25 * (U[I, J, Kp] - U[I, J, K]) / dzr + 0.25 * (U[Im, J, Kp] - U[Im, J, K]) / dzr)
        a[9] = (0.25 * (V[I, J, K] - V[I, J, Km]) / dzl + 0.25 * (V[I, Jm, K] - V[I, Jm, Km]) / dzl
                + 0.25 * (V[I, J, Kp] - V[I, J, K]) / dzr + 0.25 * (V[I, Jm, Kp] - V[I, Jm, K]) / dzr)
        ddx = ((x[2:nxg] - x[1:nxg - 1]) ** 2.0)[:, None, None]
        ddy = ((y[2:nyg] - y[1:nyg - 1]) ** 2.0)[None, :, None]
        ddz = ((z[2:nzg] - z[1:nzg - 1]) ** 2.0)[None, None, :]
        # b_ij components 1..6 = (11, 22, 33, 12, 13, 23); a layout (1 4 5; 7 2 6; 8 9 3)
        px = {1: (1, 1), 2: (4, 4), 3: (5, 5), 4: (1, 4), 5: (1, 5), 6: (4, 5)}
        py = {1: (7, 7), 2: (2, 2), 3: (6, 6), 4: (7, 2), 5: (7, 6), 6: (2, 6)}
        pz = {1: (8, 8), 2: (9, 9), 3: (3, 3), 4: (8, 9), 5: (8, 3), 6: (9, 3)}
        b = {}
        for m in range(1, 7):
            b[m] = 0.0 + ddx * a[px[m][0]] * a[px[m][1]]
            b[m] = b[m] + ddy * a[py[m][0]] * a[py[m][1]]
            b[m] = b[m] + ddz * a[pz[m][0]] * a[pz[m][1]]
        Bb = (b[1] * b[2] - b[4] ** 2.0 + b[1] * b[3] - b[5] ** 2.0 + b[2] * b[3] - b[6] ** 2.0)
        Ab = a[1] ** 2.0
        for m in range(2, 10):
            Ab = Ab + a[m] ** 2.0
        out = alloc(nxg, nyg, nzg)
        with np.errstate(divide="ignore", invalid="ignore"):
            out[I, J, K] = C * (Bb / Ab) ** 0.5
        self.vreman_terms = (Bb, Ab)
        self.nu_t = self._nut_ghost_rows_amd_vreman(out)
        return self.nu_t

    def compute_eddy_viscosity(self):
        """subgrid.f90:23-47."""
        if self.p.LES_model == LES_SMAG:
            return self.sgs_Smagorinsky()
        if self.p.LES_model == LES_DSM:
            return self.sgs_dynamic_Smagorinsky()
        if self.p.LES_model == LES_AMD:
            return self.sgs_AMD()
        if self.p.LES_model == LES_VREMAN:
            return self.sgs_Vreman()
        self.nu_t = alloc(self.g.nxg, self.g.nyg, self.g.nzg)
        return self.nu_t

    # -- equilibrium log-law wall stress (new; writes alpha_x) --------------
    def compute_wall_stress_eqlog(self):
        """tau_w per wall point from u/u_tau = ln(h u_tau/nu)/kappa + B matched
        at the third off-wall cell (rows 4 and nyg-3), Newton from the
        laminar estimate, viscous sublayer (u+=y+) where the log law is not
        above it.  Result (Nx,2,Nz) goes to set_wall_stress."""
        g, p = self.g, self.p
        Ub = self.U[2:g.nx, 4, 2:g.nzg - 1]
        Ut = self.U[2:g.nx, g.nyg - 3, 2:g.nzg - 1]
        hb = g.yg[4] - g.y[1]
        ht = g.y[g.ny] - g.yg[g.nyg - 3]
        alpha = np.zeros((g.Nx, 2, g.Nz))
        alpha[:, 0, :] = eqlog_tau(Ub, hb, p.nu)
        alpha[:, 1, :] = eqlog_tau(Ut, ht, p.nu)
        return alpha

    # -- wall model (wallmodel.f90:23-46) -----------------------------------
    def compute_wall_model(self):
        g, p = self.g, self.p
        nx, nyg, nxg = g.nx, g.nyg, g.nxg
        U, a = self.U, self.alpha_x
        dyw = g.yg[2] - g.yg[1]
        with np.errstate(divide="ignore", invalid="ignore"):
            tb = a[1:nx + 1, 1, 1:] / ((U[1:nx + 1, 2, 1:] - U[1:nx + 1, 1, 1:]) / dyw) - p.nu
            tt = a[1:nx + 1, 2, 1:] / ((U[1:nx + 1, nyg - 1, 1:] - U[1:nx + 1, nyg, 1:]) / dyw) - p.nu
        # interpolate_x over the section term(2:nx-1) writes centres 2..nx
        cb = 0.5 * (tb[0:nx - 1] + tb[1:nx])
        ct = 0.5 * (tt[0:nx - 1] + tt[1:nx])
        nu_t = self.nu_t
        nu_t[2:nx + 1, 1, 1:] = cb
        nu_t[2:nx + 1, 2, 1:] = cb
        nu_t[2:nx + 1, nyg - 1, 1:] = ct
        nu_t[2:nx + 1, nyg, 1:] = ct
        per_x(nu_t, g, 2)

    # -- RHS (equations.f90) -------------------------------------------------
    def compute_rhs_u(self, U, V, W, nu_t, dPdx):
        """equations.f90:24-167 -> F(2:nx-1, 2:nyg-1, 2:nzg-1)."""
        g, p = self.g, self.p
        nx, nyg, nzg, nz = g.nx, g.nyg, g.nzg, g.nz
        x, y, z, xg, yg, zg, w0, w1 = g.x, g.y, g.z, g.xg, g.yg, g.zg, g.w0, g.w1
        nu = p.nu
        I, J, K = slice(2, nx), slice(2, nyg), slice(2, nzg)
        Im, Jm, Km = slice(1, nx - 1), slice(1, nyg - 1), slice(1, nzg - 1)
        Ip, Jp, Kp = slice(3, nx + 1), slice(3, nyg + 1), slice(3, nzg + 1)
        # 1) -du^2/dx : term_1(i) = 0.5(U(i)+U(i+1))^2, i = 1..nx-1
        t1 = np.zeros((nx + 1, nyg + 1, nzg + 1))
        t1[1:nx] = (0.5 * (U[1:nx] + U[2:nx + 1])) ** 2.0
        rhs = -(t1[I, J, K] - t1[Im, J, K]) / (xg[3:nx + 1] - xg[2:nx])[:, None, None]
        # 2) -duv/dy
        uy = w0[None, 1:nyg, None] * U[1:nx + 1, 1:nyg, :] + w1[None, 1:nyg, None] * U[1:nx + 1, 2:nyg + 1, :]
        vx = 0.5 * (V[1:nx + 1, 1:, :] + V[2:nx + 2, 1:, :])        # i = 1..nx, j = 1..ny
        t1 = np.zeros((nx + 1, nyg + 1, nzg + 1))
        t1[1:nx + 1, 1:nyg, :] = uy[:, :, :] * vx[:, :, :]
        rhs = rhs + (-(t1[I, J, K] - t1[I, Jm, K]) / (y[2:nyg] - y[1:nyg - 1])[None, :, None])
        # 3) -duw/dz
        t1 = np.zeros((nx + 1, nyg + 1, nzg + 1))
        uz = 0.5 * (U[1:nx + 1, :, 1:nzg] + U[1:nx + 1, :, 2:nzg + 1])      # k = 1..nzg-1
        wx = 0.5 * (W[1:nx + 1, :, 1:nz + 1] + W[2:nx + 2, :, 1:nz + 1])    # k = 1..nz
        t1[1:nx + 1, :, 1:nzg] = uz * wx[:, :, 0:nzg - 1]
        rhs = rhs + (-(t1[I, J, K] - t1[I, J, Km]) / (z[2:nzg] - z[1:nzg - 1])[None, None, :])
        # 4) viscous term
        t2 = np.zeros((nx + 1, nyg + 1, nzg + 1))
        t2[1:nx + 1, 1:nyg, 1:] = (U[1:nx + 1, 2:nyg + 1, 1:] - U[1:nx + 1, 1:nyg, 1:]) / (yg[2:nyg + 1] - yg[1:nyg])[None, :, None]
        dz1 = (zg[2:nzg] - zg[1:nzg - 1])[None, None, :]
        dz2 = (zg[3:nzg + 1] - zg[2:nzg])[None, None, :]
        dz3 = (z[2:nzg] - z[1:nzg - 1])[None, None, :]
        dy3 = (y[2:nyg] - y[1:nyg - 1])[None, :, None]
        dx1 = (x[2:nx] - x[1:nx - 1])[:, None, None]
        dx2 = (x[3:nx + 1] - x[2:nx])[:, None, None]
        dx3 = (xg[3:nx + 1] - xg[2:nx])[:, None, None]
        nt = nu_t
        Ix1 = slice(3, nx + 1)
        nu_x1 = nu + nt[I, J, K]
        nu_x2 = nu + nt[Ix1, J, K]
        w0m, w1m = w0[None, 1:nyg - 1, None], w1[None, 1:nyg - 1, None]
        w0j, w1j = w0[None, 2:nyg, None], w1[None, 2:nyg, None]
        nu_y1 = nu + 0.5 * (w0m * nt[I, Jm, K] + w1m * nt[I, J, K] + w0m * nt[Ix1, Jm, K] + w1m * nt[Ix1, J, K])
        nu_y2 = nu + 0.5 * (w0j * nt[I, J, K] + w1j * nt[I, Jp, K] + w0j * nt[Ix1, J, K] + w1j * nt[Ix1, Jp, K])
        nu_z1 = nu + 0.25 * (nt[I, J, K] + nt[I, J, Km] + nt[Ix1, J, K] + nt[Ix1, J, Km])
        nu_z2 = nu + 0.25 * (nt[I, J, K] + nt[I, J, Kp] + nt[Ix1, J, K] + nt[Ix1, J, Kp])
        visc = (1.0 / dx3 * (nu_x2 * 1.0 / dx2 * (U[Ip, J, K] - U[I, J, K]) - nu_x1 * 1.0 / dx1 * (U[I, J, K] - U[Im, J, K]))
                + 1.0 / dy3 * (nu_y2 * t2[I, J, K] - nu_y1 * t2[I, Jm, K])
                + 1.0 / dz3 * (nu_z2 * 1.0 / dz2 * (U[I, J, Kp] - U[I, J, K]) - nu_z1 * 1.0 / dz1 * (U[I, J, K] - U[I, J, Km])))
        rhs = rhs + visc
        rhs = rhs + dPdx
        return rhs

    def compute_rhs_v(self, U, V, W, nu_t):
        """equations.f90:174-320 -> F(2:nxg-1, 2:ny-1, 2:nzg-1)."""
        g, p = self.g, self.p
        nx, ny, nxg, nyg, nzg, nz = g.nx, g.ny, g.nxg, g.nyg, g.nzg, g.nz
        x, y, z, xg, yg, zg, w0, w1 = g.x, g.y, g.z, g.xg, g.yg, g.zg, g.w0, g.w1
        nu = p.nu
        I, J, K = slice(2, nxg), slice(2, ny), slice(2, nzg)
        Im, Jm, Km = slice(1, nxg - 1), slice(1, ny - 1), slice(1, nzg - 1)
        Ip, Jp, Kp = slice(3, nxg + 1), slice(3, ny + 1), slice(3, nzg + 1)
        # 1) -dv^2/dy: term_1(j) = 0.5(V(j)+V(j+1))^2, j = 1..ny-1
        t1 = np.zeros((nxg + 1, nyg + 1, nzg + 1))
        t1[:, 1:ny, :] = (0.5 * (V[:, 1:ny, :] + V[:, 2:ny + 1, :])) ** 2.0
        rhs = -(t1[I, J, K] - t1[I, Jm, K]) / (yg[3:ny + 1] - yg[2:ny])[None, :, None]
        # 2) -duv/dx: term_1 = interp_y(U) (i=1..nx, j=1..ny), term_2 = interp_x(V) (i=1..nx)
        t1 = np.zeros((nxg + 1, nyg + 1, nzg + 1))
        uy = w0[None, 1:ny + 1, None] * U[1:nx + 1, 1:ny + 1, :] + w1[None, 1:ny + 1, None] * U[1:nx + 1, 2:ny + 2, :]
        vx = 0.5 * (V[1:nx + 1, 1:ny + 1, :] + V[2:nx + 2, 1:ny + 1, :])
        t1[1:nx + 1, 1:ny + 1, :] = uy * vx
        rhs = rhs + (-(t1[I, J, K] - t1[Im, J, K]) / (x[2:nxg] - x[1:nxg - 1])[:, None, None])
        # 3) -dvw/dz: term_1 = interp_z(V) (k = 1..nzg-1), term_2 = interp_y(W) (j=1..ny, k=1..nz)
        t1 = np.zeros((nxg + 1, nyg + 1, nzg + 1))
        vz = 0.5 * (V[:, 1:ny + 1, 1:nzg] + V[:, 1:ny + 1, 2:nzg + 1])
        wy = w0[None, 1:ny + 1, None] * W[:, 1:ny + 1, 1:nz + 1] + w1[None, 1:ny + 1, None] * W[:, 2:ny + 2, 1:nz + 1]
        t1[:, 1:ny + 1, 1:nzg] = vz * wy[:, :, 0:nzg - 1]
        rhs = rhs + (-(t1[I, J, K] - t1[I, J, Km]) / (z[2:nzg] - z[1:nzg - 1])[None, None, :])
        # 4) viscous
        nt = nu_t
        dz1 = (zg[2:nzg] - zg[1:nzg - 1])[None, None, :]
        dz2 = (zg[3:nzg + 1] - zg[2:nzg])[None, None, :]
        dz3 = (z[2:nzg] - z[1:nzg - 1])[None, None, :]
        dy1 = (y[2:ny] - y[1:ny - 1])[None, :, None]
        dy2 = (y[3:ny + 1] - y[2:ny])[None, :, None]
        dy3 = (yg[3:ny + 1] - yg[2:ny])[None, :, None]
        dx1 = (xg[2:nxg] - xg[1:nxg - 1])[:, None, None]
        dx2 = (xg[3:nxg + 1] - xg[2:nxg])[:, None, None]
        dx3 = (x[2:nxg] - x[1:nxg - 1])[:, None, None]
        w0j, w1j = w0[None, 2:ny, None], w1[None, 2:ny, None]
        Jn = slice(3, ny + 1)   # j+1 of nu_t (nyg extent)
        nu_x1 = nu + 0.5 * (w0j * nt[Im, J, K] + w1j * nt[Im, Jn, K] + w0j * nt[I, J, K] + w1j * nt[I, Jn, K])
        nu_x2 = nu + 0.5 * (w0j * nt[I, J, K] + w1j * nt[I, Jn, K] + w0j * nt[Ip, J, K] + w1j * nt[Ip, Jn, K])
        nu_y1 = nu + nt[I, J, K]
        nu_y2 = nu + nt[I, Jn, K]
        nu_z1 = nu + 0.5 * (w0j * nt[I, J, Km] + w1j * nt[I, Jn, Km] + w0j * nt[I, J, K] + w1j * nt[I, Jn, K])
        nu_z2 = nu + 0.5 * (w0j * nt[I, J, K] + w1j * nt[I, Jn, K] + w0j * nt[I, J, Kp] + w1j * nt[I, Jn, Kp])
        visc = (1.0 / dx3 * (nu_x2 * 1.0 / dx2 * (V[Ip, J, K] - V[I, J, K]) - nu_x1 * 1.0 / dx1 * (V[I, J, K] - V[Im, J, K]))
                + 1.0 / dy3 * (nu_y2 * 1.0 / dy2 * (V[I, Jp, K] - V[I, J, K]) - nu_y1 * 1.0 / dy1 * (V[I, J, K] - V[I, Jm, K]))
                + 1.0 / dz3 * (nu_z2 * 1.0 / dz2 * (V[I, J, Kp] - V[I, J, K]) - nu_z1 * 1.0 / dz1 * (V[I, J, K] - V[I, J, Km])))
        return rhs + visc

    def compute_rhs_w(self, U, V, W, nu_t):
        """equations.f90:327-468 -> F(2:nxg-1, 2:nyg-1, 2:nz-1)."""
        g, p = self.g, self.p
        nx, ny, nxg, nyg, nzg, nz = g.nx, g.ny, g.nxg, g.nyg, g.nzg, g.nz
        x, y, z, xg, yg, zg, w0, w1 = g.x, g.y, g.z, g.xg, g.yg, g.zg, g.w0, g.w1
        nu = p.nu
        I, J, K = slice(2, nxg), slice(2, nyg), slice(2, nz)
        Im, Jm, Km = slice(1, nxg - 1), slice(1, nyg - 1), slice(1, nz - 1)
        Ip, Jp, Kp = slice(3, nxg + 1), slice(3, nyg + 1), slice(3, nz + 1)
        # 1) -dw^2/dz: term_1(k) = 0.5(W(k)+W(k+1))^2, k=1..nz-1
        t1 = np.zeros((nxg + 1, nyg + 1, nzg + 1))
        t1[:, :, 1:nz] = (0.5 * (W[:, :, 1:nz] + W[:, :, 2:nz + 1])) ** 2.0
        rhs = -(t1[I, J, K] - t1[I, J, Km]) / (zg[3:nz + 1] - zg[2:nz])[None, None, :]
        # 2) -duw/dx: term_1 = interp_z(U) (i=1..nx, k=1..nzg-1), term_2 = interp_x(W) (i=1..nxg-1)
        t1 = np.zeros((nxg + 1, nyg + 1, nzg + 1))
        uz = 0.5 * (U[1:nx + 1, :, 1:nzg] + U[1:nx + 1, :, 2:nzg + 1])
        wx = 0.5 * (W[1:nx + 1, :, 1:nz + 1] + W[2:nx + 2, :, 1:nz + 1])
        t1[1:nx + 1, :, 1:nzg] = uz * wx[:, :, 0:nzg - 1]
        rhs = rhs + (-(t1[I, J, K] - t1[Im, J, K]) / (x[2:nxg] - x[1:nxg - 1])[:, None, None])
        # 3) -dvw/dy: term_1 = interp_z(V) (j=1..ny, k=1..nzg-1), term_2 = interp_y(W) (j=1..ny, k=1..nz)
        t1 = np.zeros((nxg + 1, nyg + 1, nzg + 1))
        vz = 0.5 * (V[:, 1:ny + 1, 1:nzg] + V[:, 1:ny + 1, 2:nzg + 1])
        wy = w0[None, 1:ny + 1, None] * W[:, 1:ny + 1, 1:nz + 1] + w1[None, 1:ny + 1, None] * W[:, 2:ny + 2, 1:nz + 1]
        t1[:, 1:ny + 1, 1:nzg] = vz * wy[:, :, 0:nzg - 1]
        rhs = rhs + (-(t1[I, J, K] - t1[I, Jm, K]) / (y[2:nyg] - y[1:nyg - 1])[None, :, None])
        # 4) viscous
        nt = nu_t
        t2 = np.zeros((nxg + 1, nyg + 1, nzg + 1))
        t2[:, 1:nyg, 1:nz + 1] = (W[:, 2:nyg + 1, 1:nz + 1] - W[:, 1:nyg, 1:nz + 1]) / (yg[2:nyg + 1] - yg[1:nyg])[None, :, None]
        dz1 = (z[2:nz] - z[1:nz - 1])[None, None, :]
        dz2 = (z[3:nz + 1] - z[2:nz])[None, None, :]
        dz3 = (zg[3:nz + 1] - zg[2:nz])[None, None, :]
        dy3 = (y[2:nyg] - y[1:nyg - 1])[None, :, None]
        dx1 = (xg[2:nxg] - xg[1:nxg - 1])[:, None, None]
        dx2 = (xg[3:nxg + 1] - xg[2:nxg])[:, None, None]
        dx3 = (x[2:nxg] - x[1:nxg - 1])[:, None, None]
        Kn = slice(3, nz + 1)
        nu_x1 = nu + 0.25 * (nt[I, J, K] + nt[I, J, Kn] + nt[Im, J, K] + nt[Im, J, Kn])
        nu_x2 = nu + 0.25 * (nt[I, J, K] + nt[I, J, Kn] + nt[Ip, J, K] + nt[Ip, J, Kn])
        w0m, w1m = w0[None, 1:nyg - 1, None], w1[None, 1:nyg - 1, None]
        w0j, w1j = w0[None, 2:nyg, None], w1[None, 2:nyg, None]
        nu_y1 = nu + 0.5 * (w0m * nt[I, Jm, K] + w1m * nt[I, J, K] + w0m * nt[I, Jm, Kn] + w1m * nt[I, J, Kn])
        nu_y2 = nu + 0.5 * (w0j * nt[I, J, K] + w1j * nt[I, Jp, K] + w0j * nt[I, J, Kn] + w1j * nt[I, Jp, Kn])
        nu_z1 = nu + nt[I, J, K]
        nu_z2 = nu + nt[I, J, Kn]
        visc = (1.0 / dx3 * (nu_x2 * 1.0 / dx2 * (W[Ip, J, K] - W[I, J, K]) - nu_x1 * 1.0 / dx1 * (W[I, J, K] - W[Im, J, K]))
                + 1.0 / dy3 * (nu_y2 * t2[I, J, K] - nu_y1 * t2[I, Jm, K])
                + 1.0 / dz3 * (nu_z2 * 1.0 / dz2 * (W[I, J, Kp] - W[I, J, K]) - nu_z1 * 1.0 / dz1 * (W[I, J, K] - W[I, J, Km])))
        return rhs + visc

    # -- projection (projection.f90:20-214) ----------------------------------
    def divergence(self, U, V, W):
        """compute_pseudo_pressure_rhs body: div at centres (2:nxg-1,2:nyg-1,2:nzg-1)."""
        g = self.g
        nxg, nyg, nzg = g.nxg, g.nyg, g.nzg
        I, J, K = slice(2, nxg), slice(2, nyg), slice(2, nzg)
        return ((U[I, J, K] - U[1:nxg - 1, J, K]) / (g.x[2:nxg] - g.x[1:nxg - 1])[:, None, None]
                + (V[I, J, K] - V[I, 1:nyg - 1, K]) / (g.y[2:nyg] - g.y[1:nyg - 1])[None, :, None]
                + (W[I, J, K] - W[I, J, 1:nzg - 1]) / (g.z[2:nzg] - g.z[1:nzg - 1])[None, None, :])

    def solve_modes(self, rhs_hat, bc_lo=None, bc_hi=None):
        """Per-mode tridiagonal solve (projection.f90:90-113, pressure.f90:118-144).
        rhs_hat: complex (Nx, Ny, Nz) spectrum in rows j=2..nyg-1.  The
        elimination is zgtsv's, which never pivots here (the bands are
        diagonally dominant); tests/test_oracle_kat.py checks it against
        LAPACK zgtsv."""
        g = self.g
        Ny = g.nyg - 2
        lam = g.kxx[:, None] + g.kzz[None, :]                  # (Nx, Nz)
        D = g.Dd[2:g.nyg][None, :, None] + lam[:, None, :]      # (Nx, Ny, Nz)
        D = D.astype(np.complex128)
        D[0, 0, 0] = 3.0 / 2.0 * D[0, 0, 0]
        DL = g.Dl[3:g.nyg]           # Dyy(j+1, j), j = 2..nyg-2
        DU = g.Du[2:g.nyg - 1]       # Dyy(j, j+1)
        b = rhs_hat.astype(np.complex128).copy()
        if bc_lo is not None:
            b[:, 0, :] += bc_lo
            b[:, Ny - 1, :] -= bc_hi
        d = D.copy()
        for j in range(1, Ny):
            mult = DL[j - 1] / d[:, j - 1, :]
            d[:, j, :] = d[:, j, :] - mult * DU[j - 1]
            b[:, j, :] = b[:, j, :] - mult * b[:, j - 1, :]
        xsol = np.empty_like(b)
        xsol[:, Ny - 1, :] = b[:, Ny - 1, :] / d[:, Ny - 1, :]
        for j in range(Ny - 2, -1, -1):
            xsol[:, j, :] = (b[:, j, :] - DU[j] * xsol[:, j + 1, :]) / d[:, j, :]
        return xsol

    def solve_poisson_equation(self, div):
        """projection.f90:74-128: FFT(x,z) of cells 2..Nx+1 x 2..Nz+1 per
        plane, per-mode tridiagonal, inverse FFT / (Nx*Nz), periodic copy."""
        g = self.g
        Nx, Nz = g.Nx, g.Nz
        plane = div[0:Nx, :, 0:Nz]
        hat = np.fft.fft2(plane, axes=(0, 2))
        sol = self.solve_modes(hat)
        # FFTW's unnormalised backward transform divided by Nx*Nz == ifft2
        rhs_p = alloc(g.nxg, g.nyg, g.nzg)
        rhs_p[2:Nx + 2, 2:g.nyg, 2:Nz + 2] = np.real(np.fft.ifft2(sol, axes=(0, 2)))
        # apply_periodic_xz_pressure (projection.f90:133-151)
        rhs_p[g.nxg - 1, :, :] = rhs_p[2, :, :]
        rhs_p[2:g.nxg, :, Nz + 2] = rhs_p[2:g.nxg, :, 2]
        return rhs_p

    def project_velocity(self, rhs_p):
        """projection.f90:192-214."""
        g = self.g
        nx, ny, nz, nxg, nyg, nzg = g.nx, g.ny, g.nz, g.nxg, g.nyg, g.nzg
        U, V, W = self.U, self.V, self.W
        U[2:nx, 2:nyg, 2:nzg] -= (rhs_p[3:nx + 1, 2:nyg, 2:nzg] - rhs_p[2:nx, 2:nyg, 2:nzg]) / (g.xg[3:nx + 1] - g.xg[2:nx])[:, None, None]
        V[2:nxg, 2:ny, 2:nzg] -= (rhs_p[2:nxg, 3:ny + 1, 2:nzg] - rhs_p[2:nxg, 2:ny, 2:nzg]) / (g.yg[3:ny + 1] - g.yg[2:ny])[None, :, None]
        W[2:nxg, 2:nyg, 2:nz] -= (rhs_p[2:nxg, 2:nyg, 3:nz + 1] - rhs_p[2:nxg, 2:nyg, 2:nz]) / (g.zg[3:nz + 1] - g.zg[2:nz])[None, None, :]

    def compute_projection_step(self):
        div = self.divergence(self.U, self.V, self.W)
        self.rhs_p = self.solve_poisson_equation(div)
        self.project_velocity(self.rhs_p)

    def check_divergence(self):
        """projection.f90:223-245 (signed maximum, as written) plus max|div|."""
        div = self.divergence(self.U, self.V, self.W)
        return max(0.0, float(div.max())), float(np.abs(div[0:self.g.Nx, :, 0:self.g.Nz]).max())

    # -- mass flow (mass_flow.f90) -------------------------------------------
    def compute_mean_mass_flow_U(self, U):
        """mass_flow.f90:24-61 (union of the per-rank k ranges: 2..nzg-2)."""
        g = self.g
        dyg = (g.yg[3:g.nyg] - g.yg[2:g.nyg - 1])
        Q = (U[2:g.nx, 3:g.nyg, 2:g.nzg - 1] + U[2:g.nx, 2:g.nyg - 1, 2:g.nzg - 1]) * 0.5 * dyg[None, :, None]
        nrm = np.broadcast_to((1.0 + 1.0) * 0.5 * dyg[None, :, None], Q.shape)
        return float(Q.sum()) / float(nrm.sum())

    def compute_mean_mass_flow_V(self, V):
        """mass_flow.f90:70-98."""
        g = self.g
        dy = (g.y[2:g.ny + 1] - g.y[1:g.ny])
        Q = (V[2:g.nxg, 2:g.ny + 1, 2:g.nzg] + V[2:g.nxg, 1:g.ny, 2:g.nzg]) * 0.5 * dy[None, :, None]
        nrm = np.broadcast_to((1.0 + 1.0) * 0.5 * dy[None, :, None], Q.shape)
        return float(Q.sum()) / float(nrm.sum())

    def compute_dPx_for_constant_mass_flow(self):
        """mass_flow.f90:113-166 (k = 2..nzg-2)."""
        g = self.g
        Ui = 0.5 * (self.U[2:g.nx, 3, 2:g.nzg - 1] + self.U[2:g.nx, g.nyg - 2, 2:g.nzg - 1])
        return self.Qflow_x_0 - float(Ui.sum()) / float(Ui.size)

    # -- RK3 step (time_integration.f90:24-96) -------------------------------
    def _stage_sgs_wm(self, stage=0):
        self.compute_eddy_viscosity()
        if self.p.wall_model in (WM_EQLOG, WM_MLP):
            alpha = self.compute_wall_stress_eqlog()
            if self.p.wall_model == WM_MLP:
                from . import mlp_wm_ref
                act = self.mlp_actions(stage) if self.mlp_actions else None
                alpha, self.mlp_info[stage] = mlp_wm_ref.wall_stress(self, alpha, self.mlp_nutot,
                                                                     self.mlp_theta, act)
            self.set_wall_stress(alpha)
        if self.p.wall_model != WM_NONE:
            self.compute_wall_model()
        if self.p.wall_model == WM_MLP:
            self.mlp_nutot = self.p.nu + self.nu_t

    def compute_time_step_RK3(self):
        g, dt = self.g, self.dt
        nx, ny, nz, nxg, nyg, nzg = g.nx, g.ny, g.nz, g.nxg, g.nyg, g.nzg
        to = self.t
        Uo, Vo, Wo = self.U.copy(), self.V.copy(), self.W.copy()
        Fu, Fv, Fw = [None] * 3, [None] * 3, [None] * 3
        for s in range(3):
            self._stage_sgs_wm(s)
            Fu[s] = self.compute_rhs_u(self.U, self.V, self.W, self.nu_t, self.dPdx)
            Fv[s] = self.compute_rhs_v(self.U, self.V, self.W, self.nu_t)
            Fw[s] = self.compute_rhs_w(self.U, self.V, self.W, self.nu_t)
            if s == 0:
                self.U[2:nx, 2:nyg, 2:nzg] = Uo[2:nx, 2:nyg, 2:nzg] + dt * RK_COEF[0][0] * Fu[0]
                self.V[2:nxg, 2:ny, 2:nzg] = Vo[2:nxg, 2:ny, 2:nzg] + dt * RK_COEF[0][0] * Fv[0]
                self.W[2:nxg, 2:nyg, 2:nz] = Wo[2:nxg, 2:nyg, 2:nz] + dt * RK_COEF[0][0] * Fw[0]
            elif s == 1:
                self.U[2:nx, 2:nyg, 2:nzg] = Uo[2:nx, 2:nyg, 2:nzg] + dt * (RK_COEF[1][0] * Fu[0] + RK_COEF[1][1] * Fu[1])
                self.V[2:nxg, 2:ny, 2:nzg] = Vo[2:nxg, 2:ny, 2:nzg] + dt * (RK_COEF[1][0] * Fv[0] + RK_COEF[1][1] * Fv[1])
                self.W[2:nxg, 2:nyg, 2:nz] = Wo[2:nxg, 2:nyg, 2:nz] + dt * (RK_COEF[1][0] * Fw[0] + RK_COEF[1][1] * Fw[1])
            else:
                self.U[2:nx, 2:nyg, 2:nzg] = Uo[2:nx, 2:nyg, 2:nzg] + dt * (RK_COEF[2][0] * Fu[0] + RK_COEF[2][1] * Fu[1] + RK_COEF[2][2] * Fu[2])
                self.V[2:nxg, 2:ny, 2:nzg] = Vo[2:nxg, 2:ny, 2:nzg] + dt * (RK_COEF[2][0] * Fv[0] + RK_COEF[2][1] * Fv[1] + RK_COEF[2][2] * Fv[2])
                self.W[2:nxg, 2:nyg, 2:nz] = Wo[2:nxg, 2:nyg, 2:nz] + dt * (RK_COEF[2][0] * Fw[0] + RK_COEF[2][1] * Fw[1] + RK_COEF[2][2] * Fw[2])
            self.t = to + RK_T[s] * dt
            self.apply_boundary_conditions()
            self.compute_projection_step()
            self.apply_boundary_conditions()
        if self.p.x_mass_cte == 1:
            d = self.compute_dPx_for_constant_mass_flow()
            self.U[2:nx, 2:nyg, 2:nzg] = self.U[2:nx, 2:nyg, 2:nzg] + d
            self.last_mass_shift = d
            self.dPdx = 0.0
            self.apply_boundary_conditions()

    def step(self):
        """One iteration of the app_main loop's solver part (app_main.f90:114-117)."""
        self.compute_dt()
        self.compute_time_step_RK3()

    # -- actual pressure (pressure.f90:21-340) --------------------------------
    def compute_pressure_BC(self):
        g, p = self.g, self.p
        y, V, nt, yg = g.y, self.V, self.nu_t, g.yg
        ny, nyg = g.ny, g.nyg
        I, K = slice(2, g.nxg), slice(2, g.nzg)
        dzeta = 1.0
        gg = (-3.0 * y[1] + 4.0 * y[2] - y[3]) / (2.0 * dzeta)
        g2 = (2.0 * y[1] - 5.0 * y[2] + 4.0 * y[3] - 1.0 * y[4]) / dzeta ** 2.0
        nui = p.nu + 0.5 * (nt[I, 1, K] + nt[I, 2, K])
        dnu = (nt[I, 2, K] - nt[I, 1, K]) / (yg[2] - yg[1])
        dV = (-3.0 * V[I, 1, K] + 4.0 * V[I, 2, K] - V[I, 3, K]) / (2.0 * dzeta) * 1.0 / gg
        ddV = (2.0 * V[I, 1, K] - 5.0 * V[I, 2, K] + 4.0 * V[I, 3, K] - 1.0 * V[I, 4, K]) / dzeta ** 2.0
        ddV = (ddV - dV * g2) / gg ** 2.0
        bc_1 = dnu * dV + nui * ddV
        gg = (3.0 * y[ny] - 4.0 * y[ny - 1] + y[ny - 2]) / (2.0 * dzeta)
        g2 = (2.0 * y[ny] - 5.0 * y[ny - 1] + 4.0 * y[ny - 2] - 1.0 * y[ny - 3]) / dzeta ** 2.0
        nui = p.nu + 0.5 * (nt[I, nyg, K] + nt[I, nyg - 1, K])
        dnu = (nt[I, nyg, K] - nt[I, nyg - 1, K]) / (yg[nyg] - yg[nyg - 1])
        dV = (3.0 * V[I, ny, K] - 4.0 * V[I, ny - 1, K] + V[I, ny - 2, K]) / (2.0 * dzeta) * 1.0 / gg
        ddV = (2.0 * V[I, ny, K] - 5.0 * V[I, ny - 1, K] + 4.0 * V[I, ny - 2, K] - 1.0 * V[I, ny - 3, K]) / dzeta ** 2.0
        ddV = (ddV - dV * g2) / gg ** 2.0
        bc_2 = dnu * dV + nui * ddV
        return bc_1, bc_2       # indexed (i-2, k-2) for i = 2..nxg-1, k = 2..nzg-1

    def compute_pressure(self):
        """pressure.f90:21-29 -> self.P (intended full-extent rhs_uf/vf/wf)."""
        g = self.g
        nx, ny, nz, nxg, nyg, nzg = g.nx, g.ny, g.nz, g.nxg, g.nyg, g.nzg
        Nx, Nz = g.Nx, g.Nz
        bc_1, bc_2 = self.compute_pressure_BC()
        ruf = alloc(nx, nyg, nzg)
        rvf = alloc(nxg, ny, nzg)
        rwf = alloc(nxg, nyg, nz)
        ruf[2:nx, 2:nyg, 2:nzg] = self.compute_rhs_u(self.U, self.V, self.W, self.nu_t, self.dPdx)
        rvf[2:nxg, 2:ny, 2:nzg] = self.compute_rhs_v(self.U, self.V, self.W, self.nu_t)
        rwf[2:nxg, 2:nyg, 2:nz] = self.compute_rhs_w(self.U, self.V, self.W, self.nu_t)
        per_x(ruf, g, 1)
        rvf[2:nxg, 1, 2:nzg] = bc_1
        rvf[2:nxg, ny, 2:nzg] = bc_2
        per_z(rwf, g, 3)
        div = self.divergence(ruf, rvf, rwf)
        hat = np.fft.fft2(div[0:Nx, :, 0:Nz], axes=(0, 2))
        b1 = np.fft.fft2(bc_1[0:Nx, 0:Nz])
        b2 = np.fft.fft2(bc_2[0:Nx, 0:Nz])
        lo = g.coef_bc_1 * (g.yg[2] - g.yg[1]) * b1
        hi = g.coef_bc_2 * (g.yg[nyg] - g.yg[nyg - 1]) * b2
        sol = self.solve_modes(hat, lo, hi)
        P = self.P
        P[2:Nx + 2, 2:nyg, 2:Nz + 2] = np.real(np.fft.ifft2(sol, axes=(0, 2)))
        # ghost extension in y (pressure.f90:158-159) over i=2..nxg-1, k=2..nzg-1
        P[2:nxg, 1, 2:nzg] = P[2:nxg, 2, 2:nzg] - (g.yg[2] - g.yg[1]) * bc_1
        P[2:nxg, nyg, 2:nzg] = P[2:nxg, nyg - 1, 2:nzg] + (g.yg[nyg] - g.yg[nyg - 1]) * bc_2
        P[nxg - 1, :, :] = P[2, :, :]
        P[2:nxg, :, Nz + 2] = P[2:nxg, :, 2]
        return P

    # -- statistics (statistics.f90:22-145) -----------------------------------
    def compute_statistics(self):
        """Plane means over the union of the per-rank ranges; the wall shear
        uses the bottom wall for both walls as statistics.f90:108-116 does."""
        g, p = self.g, self.p
        nx, ny, nz, nxg, nyg, nzg = g.nx, g.ny, g.nz, g.nxg, g.nyg, g.nzg
        U, V, W = self.U, self.V, self.W
        st = {}
        Uy = g.w0[None, 1:ny + 1, None] * U[1:nx + 1, 1:ny + 1, :] + g.w1[None, 1:ny + 1, None] * U[1:nx + 1, 2:ny + 2, :]
        # term(i) = 0.5(Uy(i) + Uy(i+1)), i = 1..nx-1
        Uyx = 0.5 * (Uy[0:nx - 1] + Uy[1:nx])
        Umean = np.zeros(ny + 1); Vmean = np.zeros(ny + 1); Wmean = np.zeros(ny + 1)
        U2 = np.zeros(ny + 1); V2 = np.zeros(ny + 1); W2 = np.zeros(ny + 1); UV = np.zeros(ny + 1)
        for jj in range(1, ny + 1):
            Umean[jj] = U[1:nx - 1, jj, 1:nzg - 1].sum()
            Wmean[jj] = W[1:nxg - 1, jj, 1:nz - 1].sum()
            Vmean[jj] = V[2:nxg, jj, 2:nzg].sum()
            U2[jj] = (U[1:nx - 1, jj, 1:nzg - 1] ** 2.0).sum()
            W2[jj] = (W[1:nxg - 1, jj, 1:nz - 1] ** 2.0).sum()
            V2[jj] = (V[2:nxg, jj, 2:nzg] ** 2.0).sum()
            UV[jj] = (V[2:nxg, jj, 2:nzg] * Uyx[0:nxg - 2, jj - 1, 2:nzg]).sum()
        cu = float((nx - 2) * (nzg - 2)); cv = float((nxg - 2) * (nzg - 2)); cw = float((nxg - 2) * (nz - 2))
        st["Umean"] = Umean[1:] / cu; st["Vmean"] = Vmean[1:] / cv; st["Wmean"] = Wmean[1:] / cw
        st["U2mean"] = U2[1:] / cu; st["V2mean"] = V2[1:] / cv; st["W2mean"] = W2[1:] / cw
        st["UVmean"] = UV[1:] / cv
        # wall shear: interpolate_x(nu_t -> faces) then interpolate_y to y(1)
        nt = self.nu_t
        ntx = 0.5 * (nt[1:nx + 1, :, :] + nt[2:nx + 2, :, :])          # x face i (i=1..nx)
        nty1 = g.w0[1] * ntx[:, 1, :] + g.w1[1] * ntx[:, 2, :]          # at y(1)
        dUdy = (U[2:nx, 2, 2:nzg - 1] - U[2:nx, 1, 2:nzg - 1]) / (g.yg[2] - g.yg[1]) * (p.nu + nty1[1:nx - 1, 2:nzg - 1])
        tb = float(dUdy.sum()) / float((nx - 2) * (nzg - 3))
        st["tau_wall"] = tb
        st["utau"] = ((tb + tb) / g.Ly) ** 0.5
        st["Retau"] = st["utau"] * (g.y[ny] - g.y[1]) / 2.0 / p.nu
        st["Qflow_x"] = self.compute_mean_mass_flow_U(U)
        st["Qflow_y"] = self.compute_mean_mass_flow_V(V)
        return st


def eqlog_tau(u, h, nu):
    """Equilibrium log-law wall stress tau = sign(u) u_tau^2 with u_tau from
    |u|/u_tau = ln(h u_tau/nu)/kappa + B (Newton, EQWM_NEWTON_ITERS steps from
    the laminar u_tau), or the laminar value u_tau^2 = nu|u|/h where the log
    law is not above the linear law."""
    au = np.abs(u)
    ut_lam = np.sqrt(nu * au / h)
    ut = ut_lam.copy()
    lam = np.zeros(au.shape, dtype=bool)
    with np.errstate(divide="ignore", invalid="ignore"):
        yp_lam = h * ut_lam / nu
        f0 = ut_lam * (np.log(yp_lam) / KAPPA + B_LOG) - au
        # log law only above the upper crossing with u+ = y+ (y+ ~ 11);
        # below y+ = 1 the log law is meaningless (second crossing near 0.05)
        lam = ~((f0 < 0.0) & (yp_lam >= 1.0))
        for _ in range(EQWM_NEWTON_ITERS):
            lg = np.log(h * ut / nu)
            f = ut * (lg / KAPPA + B_LOG) - au
            fp = lg / KAPPA + B_LOG + 1.0 / KAPPA
            ut = ut - f / fp
    ut = np.where(lam, ut_lam, ut)
    return np.sign(u) * ut * ut
