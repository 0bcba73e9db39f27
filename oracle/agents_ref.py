"""Wall agents of the reference's RL environment, restated on the oracle's
Fortran-indexed arrays — TEST INFRASTRUCTURE ONLY.

send_recv_state_action (smarties_stat.f90:24-260): observation of the 6-D
state and the reward per agent (:38-176) and the wall stress built from the
agents' actions (:193-256).  The reference's RANDOM_NUMBER draws (sampling
row y_ind in {3, 4} and weight y_rand) are inputs here.  Parity unpinned,
like the oracle it extends.
"""
from __future__ import annotations

import math

import numpy as np


def observe(o, nagents, y_ind, y_rand, dPdx_ref):
    """states[2][nagents][6], rewards[2][nagents] from oracle `o` (U and nu_t
    with ghosts filled, as after a step).  y_ind, y_rand: [2][nagents]."""
    g = o.g
    nx, nyg, nu = g.nx, g.nyg, o.p.nu
    nxa = (nx - 2) // nagents
    yg = g.yg
    U, nt = o.U, o.nu_t
    states = np.zeros((2, nagents, 6))
    rewards = np.zeros((2, nagents))
    for i in range(1, nagents + 1):
        b = (i - 1) * nxa                   # face (i-1)*nx_nagents+2 is b+2
        # bottom wall (smarties_stat.f90:62-106)
        yi, r = int(y_ind[0][i - 1]), float(y_rand[0][i - 1])
        utau = math.sqrt((nu + 0.25 * (nt[b + 3, 2, 2] + nt[b + 2, 2, 2] + nt[b + 3, 1, 2] + nt[b + 2, 1, 2]))
                         * (U[b + 2, 2, 2] - U[b + 2, 1, 2]) / (yg[2] - yg[1]))
        l_sca = r * yg[yi] + (1.0 - r) * yg[yi + 1]
        Uloc = (0.2 * (r * U[b + 2, yi, 2] + ((1.0 - r) * U[b + 2, yi + 1, 2]))
                + 0.2 * (r * U[b + 1, yi, 2] + ((1.0 - r) * U[b + 1, yi + 1, 2]))
                + 0.2 * (r * U[b + 3, yi, 2] + ((1.0 - r) * U[b + 3, yi + 1, 2]))
                + 0.2 * (r * U[b + 2, yi, 1] + ((1.0 - r) * U[b + 2, yi + 1, 1]))
                + 0.2 * (r * U[b + 2, yi, 3] + ((1.0 - r) * U[b + 2, yi + 1, 3])))
        dUloc = 0.2 * (U[b + 2, yi + 1, 2] - U[b + 2, yi, 2] + U[b + 1, yi + 1, 2] - U[b + 1, yi, 2]
                       + U[b + 3, yi + 1, 2] - U[b + 3, yi, 2] + U[b + 2, yi + 1, 1] - U[b + 2, yi, 1]
                       + U[b + 2, yi + 1, 3] - U[b + 2, yi, 3]) / (yg[yi + 1] - yg[yi])
        states[0, i - 1] = _state(dUloc, l_sca, utau, Uloc, nu, dPdx_ref)
        # top wall (smarties_stat.f90:117-156)
        yi, r = int(y_ind[1][i - 1]), float(y_rand[1][i - 1])
        utau = math.sqrt((nu + 0.25 * (nt[b + 3, nyg, 2] + nt[b + 2, nyg, 2] + nt[b + 3, nyg - 1, 2]
                                       + nt[b + 2, nyg - 1, 2]))
                         * (U[b + 2, nyg - 1, 2] - U[b + 2, nyg, 2]) / (yg[2] - yg[1]))
        l_sca = 2.0 - (r * yg[nyg - yi + 1] + (1.0 - r) * yg[nyg - yi])
        hi, lo = nyg - yi + 1, nyg - yi
        Uloc = (0.2 * (r * U[b + 2, hi, 2] + ((1.0 - r) * U[b + 2, lo, 2]))
                + 0.2 * (r * U[b + 1, hi, 2] + ((1.0 - r) * U[b + 1, lo, 2]))
                + 0.2 * (r * U[b + 3, hi, 2] + ((1.0 - r) * U[b + 3, lo, 2]))
                + 0.2 * (r * U[b + 2, hi, 1] + ((1.0 - r) * U[b + 2, lo, 1]))
                + 0.2 * (r * U[b + 2, hi, 3] + ((1.0 - r) * U[b + 2, lo, 3])))
        dUloc = 0.2 * (U[b + 2, lo, 2] - U[b + 2, hi, 2] + U[b + 1, lo, 2] - U[b + 1, hi, 2]
                       + U[b + 3, lo, 2] - U[b + 3, hi, 2] + U[b + 2, lo, 1] - U[b + 2, hi, 1]
                       + U[b + 2, lo, 3] - U[b + 2, hi, 3]) / (yg[hi] - yg[lo])
        states[1, i - 1] = _state(dUloc, l_sca, utau, Uloc, nu, dPdx_ref)
        # rewards (smarties_stat.f90:158-176)
        s = math.sqrt(dPdx_ref)
        tb = (nu + 0.25 * (nt[b + 2, 1, 2] + nt[b + 3, 1, 2] + nt[b + 2, 2, 2] + nt[b + 3, 2, 2])) \
            * (U[b + 2, 2, 2] - U[b + 2, 1, 2]) / (yg[2] - yg[1])
        tt = (nu + 0.25 * (nt[b + 2, nyg - 1, 2] + nt[b + 3, nyg - 1, 2] + nt[b + 2, nyg, 2] + nt[b + 3, nyg, 2])) \
            * (U[b + 2, nyg - 1, 2] - U[b + 2, nyg, 2]) / (yg[nyg] - yg[nyg - 1])
        rewards[0, i - 1] = 100.0 - 5000.0 * abs(tb ** 0.5 - s) / s
        rewards[1, i - 1] = 100.0 - 5000.0 * abs(tt ** 0.5 - s) / s
    return states, rewards


def _state(dUloc, l_sca, v2, Uloc, nu, dPdx_ref):
    # l_sca is a y coordinate: a wall distance only on the reference's meshes,
    # whose walls are at y = 0 and y = 2 (otherwise the log gives NaN, as in Fortran)
    with np.errstate(invalid="ignore"):
        lg = np.log(l_sca * v2 / nu)
    return np.array([(dUloc * l_sca) / v2,
                     Uloc / v2 - (dUloc * l_sca) / v2 * lg,
                     Uloc, l_sca, v2, dPdx_ref])


def alpha_from_actions(o, nagents, action):
    """The wall stress alpha_x(:, wall, :) after the agents act
    (smarties_stat.f90:193-256) on oracle `o`; returns the unique part
    [2][Nz][Nx] (faces 2..nx-1, planes 2..nzg-2), the device layout."""
    g = o.g
    Nx, Nz = g.Nx, g.Nz
    nxa = Nx // nagents
    a = o.alpha_x
    acts = np.zeros((2, nagents))
    for w in range(2):
        for na in range(1, nagents + 1):
            acts[w, na - 1] = a[(na - 1) * nxa + 2, w + 1, 2] * action[w][na - 1]
    new = np.zeros((2, Nz, Nx))
    for w in range(2):
        for j in range(1, nxa + 1):
            for i in range(1, nagents + 1):
                nxt = acts[w, i] if i < nagents else acts[w, 0]
                ax = (acts[w, i - 1] * float(nxa - j + 1)) / float(nxa) + (nxt * float(j - 1)) / float(nxa)
                face = (i - 1) * nxa + j + 1          # Fortran face; unique index face - 2
                for kk in range(1, Nz + 1):           # alpha_x(:,:,kk+1), nz_nagents = Nz
                    new[w, kk - 1, face - 2] = (ax * float(Nz - kk + 1)) / float(Nz) + (ax * float(kk - 1)) / float(Nz)
    return new
