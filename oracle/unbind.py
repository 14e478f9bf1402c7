"""ORACLE (test infrastructure only): iterative FP64 unbinding of one halo.

pyHALMA's stellar cut is a single pass (python_scripts/halo_properties.py:282-361,
``escape_velocity_unbinding_fortran``):

    phi_i = sum_j m_j / |x_j - x_i|                      (brute_force_binding_energy)
    E_i   = 1/2 |v_i - v_bulk|^2 - G * phi_i * factor_v^2 (halo_properties.py:342-357)
    bound = E_i <= 0                                      (halo_properties.py:359)

with G = 4.3e-9 (km/s)^2 Mpc / Msun (halo_properties.py:346-347).  The iterative unbinding
repeats that pass: recompute the FP64 mass-weighted bulk velocity (halo_properties.py:45-60)
over the particles still bound, recompute phi over the bound particles only (a removed
particle is neither a source nor a target again), drop every particle with E > 0, and stop
when a pass removes nothing or ``max_iter`` passes have run.  The potential here is softened
(phi_i = sum_{j != i} m_j / sqrt(r^2 + eps^2)), self pair excluded by index, all in FP64.
"""
from __future__ import annotations

import numpy as np

from . import MASK_SELF, potential_f64

G_MPC = 4.3e-9


def escape_pass(src_m, src_x, src_y, src_z, x, y, z, vx, vy, vz, v_bulk, eps=0.0, factor_v=1.0, G=G_MPC,
                mask=None, ncores=None):
    """The single-pass escape cut of halo_properties.py:320-361 in FP64: phi_i over the given
    sources (no softening and the coordinate-inequality mask of particle_subroutines.f90:499-501
    by default), E_i = 1/2 |v_i - v_bulk|^2 - G phi_i factor_v^2; returns (phi, E_kin, E)."""
    from . import MASK_COORD
    phi = potential_f64(src_m, src_x, src_y, src_z, x, y, z, eps2=float(eps) ** 2,
                        mask=MASK_COORD if mask is None else mask, ncores=ncores)
    ek = 0.5 * ((vx - v_bulk[0]) ** 2 + (vy - v_bulk[1]) ** 2 + (vz - v_bulk[2]) ** 2)
    return phi, ek, ek - G * phi * factor_v * factor_v


def unbind_pass(x, y, z, vx, vy, vz, m, eps=1e-4, factor_v=1.0, G=G_MPC, ncores=None):
    """One pass of the cut over the particles given (all treated as bound): returns
    (phi, kinetic energy, total energy) per particle in FP64; the particle stays iff
    energy <= 0 (halo_properties.py:359)."""
    # the escape pass with the set as both sources and targets, the set's own bulk velocity
    # and centre, softening and the self pair skipped
    M = m.sum()
    vb = [(m * v).sum() / M for v in (vx, vy, vz)]
    cx, cy, cz = ((m * a).sum() / M for a in (x, y, z))
    px, py, pz = x - cx, y - cy, z - cz
    return escape_pass(m, px, py, pz, px, py, pz, vx, vy, vz, vb, eps=eps, factor_v=factor_v, G=G,
                       mask=MASK_SELF, ncores=ncores)


def unbind_halo(x, y, z, vx, vy, vz, m, eps=1e-4, factor_v=1.0, max_iter=20, G=G_MPC,
                ncores=None, return_energy=False):
    """Returns (bound mask, passes run[, energies, potentials]).

    energy[i] / phi[i] are the values of particle i's last evaluation (the pass that removed
    it, or the final pass for particles still bound)."""
    n = len(x)
    bound = np.ones(n, dtype=bool)
    it = 0
    energy = np.full(n, np.nan)
    phi_last = np.full(n, np.nan)
    eps2 = float(eps) ** 2
    while it < max_iter:
        it += 1
        idx = np.nonzero(bound)[0]
        if idx.size == 0:
            break
        mb = m[idx]
        M = mb.sum()
        vbx = (mb * vx[idx]).sum() / M
        vby = (mb * vy[idx]).sum() / M
        vbz = (mb * vz[idx]).sum() / M
        # recentring does not change r_ij in exact arithmetic; it mirrors the GPU layout
        cx = (mb * x[idx]).sum() / M
        cy = (mb * y[idx]).sum() / M
        cz = (mb * z[idx]).sum() / M
        px, py, pz = x[idx] - cx, y[idx] - cy, z[idx] - cz
        phi = potential_f64(mb, px, py, pz, px, py, pz, eps2=eps2, mask=MASK_SELF, ncores=ncores)
        ek = 0.5 * ((vx[idx] - vbx) ** 2 + (vy[idx] - vby) ** 2 + (vz[idx] - vbz) ** 2)
        e = ek - G * phi * factor_v * factor_v
        energy[idx] = e
        phi_last[idx] = phi
        drop = e > 0.0
        if not drop.any():
            break
        bound[idx[drop]] = False
    if return_energy:
        return bound, it, energy, phi_last
    return bound, it
