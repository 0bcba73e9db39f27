"""Shared test helpers: oracle construction and error measures."""
import numpy as np

from channel_rl_gb300 import cases as C
from oracle.channel_ref import ChannelOracle, Grid, Params

# Parity tolerance of the velocity and pressure fields (relative max error).
FIELD_RTOL = 1e-12
# nu_t of the dynamic model is the plane-sum ratio <LM>/<MM>; the sums cancel
# (L:M takes both signs), so a last-bit difference in summation order shows
# up amplified in nu_t.  The velocity fields stay within FIELD_RTOL.
NUT_RTOL = 1e-10


def oracle_for(case):
    g = Grid(*C.faces(case))
    p = Params(nu=case.nu, CFL=case.CFL, dPdx=case.dPdx, x_mass_cte=case.x_mass_cte,
               LES_model=case.LES_model, Dirichlet_nu_t=case.Dirichlet_nu_t,
               wall_model=case.wall_model, Cs=case.Cs, Re_tau=case.Retau)
    return ChannelOracle(g, p)


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    m = np.max(np.abs(b))
    d = np.max(np.abs(a - b))
    return d / m if m > 0 else d


def regions(g):
    """Fortran-index regions (0-based into the unpadded arrays) that hold
    each field's unique points plus its y ghost/wall rows."""
    return {
        "U": (slice(1, g.nx - 1), slice(0, g.nyg), slice(1, g.nzg - 2)),
        "V": (slice(1, g.nxg - 2), slice(0, g.ny), slice(1, g.nzg - 2)),
        "W": (slice(1, g.nxg - 2), slice(0, g.nyg), slice(1, g.nz - 1)),
        "C": (slice(1, g.nxg - 2), slice(0, g.nyg), slice(1, g.nzg - 2)),
    }
