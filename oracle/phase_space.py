"""ORACLE (test infrastructure only): pyHALMA's phase-space cleaning restated on the CPU.

Restates, group by group:

* ``calc_cell`` (halo_properties.py:113-158): each particle of the list goes to the grid
  point nearest to its position relative to the centre (``np.argmin(np.abs(grid - x))`` per
  axis, first index on ties); per cell, in list order: particle count, mass, mass-weighted
  velocity (then divided by the mass), and the velocity dispersion
  sqrt(sum |v_cell - v|^2 / 3 / count);
* ``clean_cell`` (halo_properties.py:160-278): a particle is dropped when its cell holds no
  more than q_fil particles, or when |v_cell - v| / sigma_cell >= fac_sig * sig_fil (the
  first pass divides by sigma only when the cell holds more than 2 particles and uses 0
  otherwise, later passes divide when it holds 2 or more); fac_sig starts at 2, is multiplied
  by 0.75 after every pass and is at least 1 from the second pass on; passes repeat on a new
  grid around the remaining particles while dropped / remaining > 0.1.  Later passes write
  ``control[ip]`` with ``ip`` the position in the *current* list, so (as in the reference)
  they mark entries of the original list by that position;
* the main script's loop over groups (pyHALMA.py:774-877): initial centre, furthest particle and
  grid (np.arange(-(r+LL), r+LL, 2LL)), cleaning, ``control`` reset to all ones when
  cleaning is off or the group has fewer than 50 particles, centre / mass / furthest particle
  of the kept particles, groups with at least MINP particles kept, then every array sorted by
  decreasing particle count (np.flip(np.argsort(num_particles))).
"""
from __future__ import annotations

import numpy as np


def center_of_mass(pl, x, y, z, m):
    mm = m[pl]
    M = mm.sum()
    if M > 0:
        return (mm * x[pl]).sum() / M, (mm * y[pl]).sum() / M, (mm * z[pl]).sum() / M, M
    return 0.0, 0.0, 0.0, 0.0


def furthest_particle(cx, cy, cz, pl, x, y, z):
    if len(pl) == 0:
        return 0.0
    dx, dy, dz = cx - x[pl], cy - y[pl], cz - z[pl]
    return float(max(0.0, np.sqrt((dx * dx + dy * dy) + dz * dz).max()))


def grid_for(rrhh, ll):
    return np.arange(-(rrhh + ll), rrhh + ll, 2 * ll)


def _nearest(grid, v):
    out = np.empty(len(v), dtype=np.int64)
    for s in range(0, len(v), 4096):
        out[s:s + 4096] = np.argmin(np.abs(grid[None, :] - v[s:s + 4096, None]), axis=1)
    return out


def calc_cell(cx, cy, cz, grid, pl, x, y, z, vx, vy, vz, m):
    """Returns (cell id per particle, count, mass, v_cell [.,3], sigma) with cells numbered
    (ix * n + iy) * n + iz and the per-cell arrays indexed by position in np.unique's order."""
    n = len(grid)
    ix, iy, iz = _nearest(grid, x[pl] - cx), _nearest(grid, y[pl] - cy), _nearest(grid, z[pl] - cz)
    key = (ix * n + iy) * n + iz
    cells, inv = np.unique(key, return_inverse=True)
    k = len(cells)
    q = np.zeros(k)
    mass = np.zeros(k)
    vm = np.zeros((k, 3))
    mp = m[pl]
    np.add.at(q, inv, 1.0)
    np.add.at(mass, inv, mp)
    for a, v in enumerate((vx, vy, vz)):
        np.add.at(vm[:, a], inv, v[pl] * mp)     # in list order, one cell at a time
    vc = vm / mass[:, None]
    d = vc[inv] - np.stack([vx[pl], vy[pl], vz[pl]], 1)
    s = np.zeros(k)
    np.add.at(s, inv, (d[:, 0] ** 2 + d[:, 1] ** 2) + d[:, 2] ** 2)
    sig = np.sqrt(s / 3.0 / q)
    return (ix, iy, iz), inv, q, vc, sig


def clean_cell(cx, cy, cz, pl, x, y, z, vx, vy, vz, m, ll, q_fil, sig_fil):
    """Returns (cx, cy, cz, M, RRHH, control, (which_x, which_y, which_z))."""
    npart = len(pl)
    control = np.ones(npart, dtype=np.int32)
    cleaned, remaining = 0, npart
    fac_sig = 2.0
    rr = furthest_particle(cx, cy, cz, pl, x, y, z)
    which, inv, q, vc, sig = calc_cell(cx, cy, cz, grid_for(rr, ll), pl, x, y, z, vx, vy, vz, m)

    def sweep(lst, inv, q, vc, sig, first):
        nonlocal cleaned, remaining
        d = vc[inv] - np.stack([vx[lst], vy[lst], vz[lst]], 1)
        bas = np.sqrt((d[:, 0] ** 2 + d[:, 1] ** 2) + d[:, 2] ** 2)
        qq = q[inv]
        norm = qq > 2 if first else qq >= 2
        with np.errstate(divide="ignore", invalid="ignore"):
            bas = np.where(norm, bas / sig[inv], 0.0)
        drop = np.where(qq > q_fil, bas >= fac_sig * sig_fil, True)
        idx = np.nonzero(drop)[0]
        control[idx] = 0            # position in the current list (see the module docstring)
        cleaned += len(idx)
        remaining -= len(idx)

    cleaned = 0
    sweep(pl, inv, q, vc, sig, True)
    clean = pl[np.nonzero(control)[0]]
    fac_sig *= 0.75
    if remaining > 0:
        frac = cleaned / remaining
        while frac > 0.1:
            cx, cy, cz, M = center_of_mass(clean, x, y, z, m)
            rr = furthest_particle(cx, cy, cz, clean, x, y, z)
            which, inv, q, vc, sig = calc_cell(cx, cy, cz, grid_for(rr, ll), clean, x, y, z, vx, vy, vz, m)
            cleaned = 0
            sweep(clean, inv, q, vc, sig, False)
            clean = pl[np.nonzero(control)[0]]
            if remaining == 0:
                return 0.0, 0.0, 0.0, 0.0, 0, control, which
            frac = cleaned / remaining
            fac_sig *= 0.75
            fac_sig = max(1.0, fac_sig)
    cx, cy, cz, M = center_of_mass(clean, x, y, z, m)
    rr = furthest_particle(cx, cy, cz, clean, x, y, z)
    which, _, _, _, _ = calc_cell(cx, cy, cz, grid_for(rr, ll), clean, x, y, z, vx, vy, vz, m)
    return cx, cy, cz, M, rr, control, which


def phase_space_cleaning(groups, st_x, st_y, st_z, st_vx, st_vy, st_vz, st_mass, LL, Q_FIL, SIG_FIL, PSC_FLAG,
                         MINP, min_part_PSC=50):
    """The main script's block: returns dict of the arrays it leaves (sorted by decreasing size)."""
    x, y, z, vx, vy, vz, m = (np.asarray(a, dtype=np.float64) for a in (st_x, st_y, st_z, st_vx, st_vy, st_vz,
                                                                         st_mass))
    keep = {k: [] for k in ("center_x", "center_y", "center_z", "masses", "rmax", "num_particles", "num_cells",
                            "new_groups", "which_x", "which_y", "which_z")}
    for g in groups:
        pl = np.array(g, dtype=np.int64)
        cx, cy, cz, mass = center_of_mass(pl, x, y, z, m)
        r = furthest_particle(cx, cy, cz, pl, x, y, z)
        n_cell = len(grid_for(r, LL))
        _, _, _, _, _, control, which = clean_cell(cx, cy, cz, pl, x, y, z, vx, vy, vz, m, LL, Q_FIL, SIG_FIL)
        if not PSC_FLAG or len(pl) < min_part_PSC:
            control = np.ones(len(pl), dtype=np.int32)
        control = control.astype(bool)
        sel = pl[control]
        cx, cy, cz, mass = center_of_mass(sel, x, y, z, m)
        r = furthest_particle(cx, cy, cz, sel, x, y, z)
        if len(sel) >= MINP:
            for k, v in (("center_x", cx), ("center_y", cy), ("center_z", cz), ("masses", mass), ("rmax", r),
                         ("num_particles", len(sel)), ("num_cells", n_cell), ("new_groups", sel),
                         ("which_x", which[0]), ("which_y", which[1]), ("which_z", which[2])):
                keep[k].append(v)
    order = np.flip(np.argsort(np.array(keep["num_particles"], dtype=np.int32)))
    return {k: [v[i] for i in order] for k, v in keep.items()}
