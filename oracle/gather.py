"""ORACLE (test infrastructure only): the range queries of halo_gas.py:218-277 restated.

* ``query_ball_point(x, y, z, c, R)`` — the set that ``KDTree.query_ball_point(c, R)``
  returns (halo_gas.py:254, 268): indices with ((dx*dx + dy*dy) + dz*dz) <= R*R in IEEE
  double (scipy's pair rule, pinned for its FoF by tests/golden/predicate.npz), ascending.
* ``parallel_inside(x, y, z, R, cx, cy, cz)`` — halo_gas.py:218-220,
  sqrt((x-cx)**2 + (y-cy)**2 + (z-cz)**2) < R, evaluated left to right.
"""
from __future__ import annotations

import numpy as np


def query_ball_point(x, y, z, c, R):
    dx = np.asarray(x, np.float64) - c[0]
    dy = np.asarray(y, np.float64) - c[1]
    dz = np.asarray(z, np.float64) - c[2]
    d2 = (dx * dx + dy * dy) + dz * dz
    return np.nonzero(d2 <= R * R)[0]


def parallel_inside(array_x, array_y, array_z, R, cx, cy, cz):
    dx = np.asarray(array_x, np.float64) - cx
    dy = np.asarray(array_y, np.float64) - cy
    dz = np.asarray(array_z, np.float64) - cz
    return np.sqrt((dx * dx + dy * dy) + dz * dz) < R
