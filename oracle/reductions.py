"""ORACLE (test infrastructure only): FP64 per-halo reductions of the reference.

Each function restates one numba kernel of python_scripts/halo_properties.py with NumPy in
float64 (the reference runs them with ``fastmath=True``, so its summation order is
unspecified and comparisons use a relative tolerance of ~1e-12):

* ``total_mass``         halo_properties.py:16-24      M = sum m
* ``center_of_mass``     halo_properties.py:26-43      (sum m x / M, ..., M), zeros if M <= 0
* ``CM_velocity``        halo_properties.py:45-60      sum m v / M, zeros if M <= 0
* ``furthest_particle``  halo_properties.py:98-111     max |x - c| (starts at 0)
* ``half_mass_radius``   halo_properties.py:365-392    radius of the last particle, in
  increasing distance order, before the running mass exceeds M/2 (the smallest radius if
  the first particle already exceeds it)
* ``sigma_effective``    halo_properties.py:607-625    sqrt(sum |v - v_bulk|^2 / 3 / n) over
  particles strictly inside R05, 0 if none
"""
from __future__ import annotations

import numpy as np


def total_mass(part_list, st_mass):
    return float(np.sum(np.asarray(st_mass, dtype=np.float64)[part_list]))


def center_of_mass(part_list, st_x, st_y, st_z, st_mass):
    m = np.asarray(st_mass, dtype=np.float64)[part_list]
    M = m.sum()
    if M > 0:
        return (float((m * np.asarray(st_x, np.float64)[part_list]).sum() / M),
                float((m * np.asarray(st_y, np.float64)[part_list]).sum() / M),
                float((m * np.asarray(st_z, np.float64)[part_list]).sum() / M), float(M))
    return 0.0, 0.0, 0.0, 0.0


def CM_velocity(M, part_list, st_vx, st_vy, st_vz, st_mass):
    m = np.asarray(st_mass, dtype=np.float64)[part_list]
    if M > 0.0:
        return (float((m * np.asarray(st_vx, np.float64)[part_list]).sum() / M),
                float((m * np.asarray(st_vy, np.float64)[part_list]).sum() / M),
                float((m * np.asarray(st_vz, np.float64)[part_list]).sum() / M))
    return 0.0, 0.0, 0.0


def _dist(cx, cy, cz, part_list, st_x, st_y, st_z):
    dx = cx - np.asarray(st_x, np.float64)[part_list]
    dy = cy - np.asarray(st_y, np.float64)[part_list]
    dz = cz - np.asarray(st_z, np.float64)[part_list]
    return np.sqrt(dx * dx + dy * dy + dz * dz)


def furthest_particle(cx, cy, cz, part_list, st_x, st_y, st_z):
    d = _dist(cx, cy, cz, part_list, st_x, st_y, st_z)
    return float(max(0.0, d.max())) if d.size else 0.0


def half_mass_radius(cx, cy, cz, M, part_list, st_x, st_y, st_z, st_mass):
    part_list = np.asarray(part_list)
    d = _dist(cx, cy, cz, part_list, st_x, st_y, st_z)
    order = np.argsort(d, kind="stable")
    ds = d[order]
    cm = np.cumsum(np.asarray(st_mass, np.float64)[part_list][order])
    k = int(np.argmax(cm > 0.5 * M)) if np.any(cm > 0.5 * M) else len(ds)
    return float(ds[k - 1]) if k > 0 else float(ds[0])


def sigma_effective(part_list, R05, st_x, st_y, st_z, st_vx, st_vy, st_vz, cx, cy, cz, vx, vy, vz):
    d = _dist(cx, cy, cz, part_list, st_x, st_y, st_z)
    inside = d < R05
    n = int(inside.sum())
    if n == 0:
        return 0.0
    pl = np.asarray(part_list)[inside]
    s = ((np.asarray(st_vx, np.float64)[pl] - vx) ** 2 + (np.asarray(st_vy, np.float64)[pl] - vy) ** 2
         + (np.asarray(st_vz, np.float64)[pl] - vz) ** 2).sum()
    return float(np.sqrt(s / 3.0 / n))
