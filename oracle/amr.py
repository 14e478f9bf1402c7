"""ORACLE (test infrastructure only): AMR gas cells to gas particles.

Restates python_scripts/halo_gas.py:9-52 (``patch_to_particles``) and the patch loop of
:56-141 (``AMRgrid_to_particles``) with NumPy: for each refined patch in order (level >= 1),
cell centres x0 + ix*res with x0 = rx - res/2 and res = (L/ncoarse)/2**level, the cells whose
centre is strictly inside the box and whose cr0amr and solapst flags are set, x-major
(ix outer, iz inner); mass = ((1 + delta) * rho_B) * res**3; velocities times 3e5.  Every
patch of level >= 1 is visited (the cell test alone decides), which is what the reference's
preselection of patches overlapping the box amounts to.
"""
from __future__ import annotations

import numpy as np


def amr_to_particles(L, ncoarse, levels, patchn, patchr, fields, box, rho_B):
    """levels[p], patchn[p] = (nx, ny, nz), patchr[p] = (rx, ry, rz), fields[j][p] the
    per-patch arrays of delta, vx, vy, vz, temp, cr0amr, solapst.  Returns 8 float64 arrays."""
    out = [[] for _ in range(8)]
    for p in range(len(levels)):
        lev = int(levels[p])
        if lev < 1:
            continue
        res = (L / ncoarse) / 2 ** lev
        nx, ny, nz = (int(v) for v in patchn[p])
        x = (patchr[p][0] - res / 2) + np.arange(nx) * res
        y = (patchr[p][1] - res / 2) + np.arange(ny) * res
        z = (patchr[p][2] - res / 2) + np.arange(nz) * res
        X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
        inside = (X > box[0]) & (X < box[1]) & (Y > box[2]) & (Y < box[3]) & (Z > box[4]) & (Z < box[5])
        leaf = (np.asarray(fields[5][p]) != 0) & (np.asarray(fields[6][p]) != 0)
        sel = (inside & leaf).ravel()
        delta = np.asarray(fields[0][p], dtype=np.float64).ravel()[sel]
        out[0].append(X.ravel()[sel])
        out[1].append(Y.ravel()[sel])
        out[2].append(Z.ravel()[sel])
        for q, j in ((3, 1), (4, 2), (5, 3)):
            out[q].append(np.asarray(fields[j][p], dtype=np.float64).ravel()[sel] * 3e5)
        out[6].append((1 + delta) * rho_B * res ** 3)
        out[7].append(np.asarray(fields[4][p], dtype=np.float64).ravel()[sel])
    return tuple(np.concatenate(a) if a else np.zeros(0) for a in out)
