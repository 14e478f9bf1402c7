"""Phase-space cleaning of FoF groups, backed by the GB300 kernels.

pyHALMA cleans every FoF group in phase space before computing its properties: its main script
(pyHALMA.py:774-877) calls ``halo_properties.calc_cell`` and ``clean_cell``
(python_scripts/halo_properties.py:113-278) group by group.  Particles are binned on a grid of
2*LL cells around the group's centre of mass; a particle is dropped when its cell holds no
more than Q_FIL particles or when its velocity differs from the cell's mean by at least
fac_sig * SIG_FIL cell dispersions (fac_sig = 2, then 1.5, 1.125, then 1); sweeps repeat on a
new grid while they drop more than 10 % of the remaining particles.  Small groups
(< 50 particles) and runs with cleaning switched off keep every particle; groups left with
fewer than MINP particles are discarded; the survivors are sorted by decreasing size.

``phase_space_cleaning`` runs that whole block for all groups at once (C ABI
``halma_phase_space_clean``) and returns the arrays the main script builds, in its order.  Like the
reference, sweeps after the first mark particles by their position in the list being swept.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def sequential_sums(values, offsets):
    """Left-to-right FP64 sum of every segment values[offsets[s]:offsets[s+1]], rounded after
    each addition like the reference's numba loops (the building block of the per-cell sums);
    C ABI ``halma_sequential_sum_f64``.  Host or device arrays; returns float64 [segments]."""
    dev = _lib._is_torch(values)
    if dev:
        nseg = int(offsets.shape[0]) - 1
        n = int(values.shape[0])
        _lib.check_arrays(np.float64, n, values=values)
        _lib.check_arrays(np.int64, None, offsets=offsets)
        out = _lib.like(values, (max(nseg, 0),), np.float64)
        arrs = (values, offsets)
    else:
        values = _lib.as_host(values, np.float64)
        offsets = _lib.as_host(offsets, np.int64)
        nseg = offsets.shape[0] - 1
        n = values.shape[0]
        out = np.zeros(max(nseg, 0), dtype=np.float64)
        arrs = (values, offsets)
    if nseg <= 0:
        return out
    st = _lib.lib().halma_sequential_sum_f64(n, _lib.ptr(arrs[0]), nseg, _lib.ptr(arrs[1]), _lib.ptr(out),
                                             _lib.stream_of(*arrs))
    _lib.check(st, "halma_sequential_sum_f64")
    return out


def clean_groups(offsets, members, st_x, st_y, st_z, st_vx, st_vy, st_vz, st_mass, LL, Q_FIL, SIG_FIL,
                 PSC_FLAG=True, MINP=50, min_part_PSC=50, max_passes=100_000):
    """CSR form: returns (control uint8 [members], which_cell int32 [3, members] with group
    g's first n_which[g] entries from offsets[g] on, n_which int64 [groups], table float64
    [groups, len(PSC_FIELDS)])."""
    offsets = _lib.as_host(offsets, np.int64)
    members = _lib.as_host(members, np.int32)
    arrs = tuple(_lib.as_host(a, np.float64) for a in (st_x, st_y, st_z, st_vx, st_vy, st_vz, st_mass))
    n = arrs[0].shape[0]
    if any(a.shape[0] != n for a in arrs):
        raise ValueError("particle arrays must have the same length")
    G = offsets.shape[0] - 1
    nm = members.shape[0]
    if G > 0 and not 0 <= offsets[-1] <= nm:
        raise ValueError(f"the offsets cover {offsets[-1]} members, {nm} given")
    control = np.zeros(max(nm, 1), dtype=np.uint8)
    which = np.zeros((3, max(nm, 1)), dtype=np.int32)
    n_which = np.zeros(max(G, 1), dtype=np.int64)
    table = np.zeros((max(G, 1), len(_lib.PSC_FIELDS)), dtype=np.float64)
    p = _lib.PscParams(float(LL), float(Q_FIL), float(SIG_FIL), int(bool(PSC_FLAG)), int(min_part_PSC), int(MINP),
                       int(max_passes))
    if G > 0:
        st = _lib.lib().halma_phase_space_clean(n, *[_lib.ptr(a) for a in arrs], G, _lib.ptr(offsets),
                                                _lib.ptr(members), ctypes.byref(p), _lib.ptr(control),
                                                _lib.ptr(which), _lib.ptr(n_which), _lib.ptr(table), None)
        _lib.check(st, "halma_phase_space_clean")
    return control[:nm], which[:, :nm], n_which[:G], table[:G]


def phase_space_cleaning(groups, st_x, st_y, st_z, st_vx, st_vy, st_vz, st_mass, LL, Q_FIL, SIG_FIL, PSC_FLAG, MINP,
                         min_part_PSC=50):
    """pyHALMA.py:774-877 for all groups at once.  Returns a dict with the main script's arrays
    after its sort by decreasing size: center_x, center_y, center_z, masses, rmax,
    num_particles, num_cells, new_groups (index arrays), which_x / which_y / which_z (the
    cells of clean_cell's final grid, one int32 array per group)."""
    lens = np.fromiter((len(g) for g in groups), dtype=np.int64, count=len(groups))
    offsets = np.zeros(len(groups) + 1, dtype=np.int64)
    np.cumsum(lens, out=offsets[1:])
    members = np.concatenate([np.asarray(g, dtype=np.int64) for g in groups]) if offsets[-1] > 0 \
        else np.zeros(0, dtype=np.int64)
    if members.size and (members.min() < 0 or members.max() >= len(st_x)):
        raise ValueError("group members must be indices into the particle arrays")
    control, which, n_which, table = clean_groups(offsets, members, st_x, st_y, st_z, st_vx, st_vy, st_vz, st_mass,
                                                  LL, Q_FIL, SIG_FIL, PSC_FLAG, MINP, min_part_PSC)
    F = {k: i for i, k in enumerate(_lib.PSC_FIELDS)}
    out = {k: [] for k in ("center_x", "center_y", "center_z", "masses", "rmax", "num_particles", "num_cells",
                           "new_groups", "which_x", "which_y", "which_z")}
    for g in range(len(groups)):
        row = table[g]
        if not row[F["kept"]]:
            continue
        b, e = offsets[g], offsets[g + 1]
        out["center_x"].append(row[F["cx"]])
        out["center_y"].append(row[F["cy"]])
        out["center_z"].append(row[F["cz"]])
        out["masses"].append(row[F["mass"]])
        out["rmax"].append(row[F["rmax"]])
        out["num_particles"].append(int(row[F["npart"]]))
        out["num_cells"].append(int(row[F["n_cell"]]))
        out["new_groups"].append(members[b:e][control[b:e].astype(bool)])
        k = int(n_which[g])
        for a, name in enumerate(("which_x", "which_y", "which_z")):
            out[name].append(which[a, b:b + k].copy())
    # the main script's sort: np.flip(np.argsort(num_particles)) (pyHALMA.py:863)
    order = np.flip(np.argsort(np.array(out["num_particles"], dtype=np.int32)))
    return {k: [v[i] for i in order] for k, v in out.items()}
