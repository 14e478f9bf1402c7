"""Batched substructure identification (bridge splitting), backed by the GB300 kernels.

pyHALMA splits FoF groups joined by thin bridges in an inline block of its main script
(pyHALMA.py:703-766, parameters MINP_SUB, DEC_FACTOR, MIN_LL, DIST_FACTOR read at
pyHALMA.py:96-98).  For every group, at sub_LL = LL/DEC_FACTOR, LL/DEC_FACTOR^2, ... while
sub_LL > MIN_LL, it runs a FoF on the group's particles at sub_LL
(``fof.friends_of_friends_serial(st_x[part_list], ...)``), keeps the sub-groups with at least
MINP_SUB members, and cuts a sub-group off when it holds more than 1 % and less than 60 % of
the group's current particles and its centre of mass lies farther than DIST_FACTOR times the
group's half-mass radius from the group's centre of mass.  The cut-off sub-groups become
groups of their own, appended after all groups; a group left with less than 30 % of its
particles is emptied; groups with fewer than MINP members are dropped at the end.

* ``identify_substructure`` — the whole block, all groups per level in one C-ABI call
  (``halma_split_bridges``); returns the new ``groups`` and ``counter_sub`` as the block
  leaves them.
* ``sub_friends_of_friends`` — the batched form of the block's per-group FoF call:
  ``[fof.friends_of_friends_serial(st_x[pl], st_y[pl], st_z[pl], LL) for pl in part_lists]``
  in one launch sequence (``halma_fof_segmented``).
* ``fof_segmented_labels`` — the segmented FoF labels themselves.

Difference from the reference: when every sub-group that FoF returns for a group has the
same length, ``np.array(sub_groups, dtype=object)`` at pyHALMA.py:721/725 builds a 2-D
object array and ``part_list[group]`` at pyHALMA.py:735 raises ``IndexError`` (object
arrays are not valid indices); this module computes what the block computes in every other
case and returns that result there too.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def fof_segmented_labels(x, y, z, seg_offsets, linking_length):
    """FoF labels with links confined to segments (rows seg_offsets[s]..seg_offsets[s+1]).

    Labels are the smallest row index of each component, -1 for rows with no friend in their
    own segment.  Host NumPy arrays or CUDA torch tensors (labels returned on the same side).
    """
    if _lib._is_torch(x):
        n = int(x.shape[0])
        ns = int(seg_offsets.shape[0]) - 1
        _lib.check_arrays(np.float64, n, x=x, y=y, z=z)
        _lib.check_arrays(np.int64, None, seg_offsets=seg_offsets)
        px, py, pz, off = x, y, z, seg_offsets
        labels = _lib.like(x, (n,), np.int32)
    else:
        px, py, pz = (_lib.as_host(a, np.float64) for a in (x, y, z))
        off = _lib.as_host(seg_offsets, np.int64)
        n, ns = px.shape[0], off.shape[0] - 1
        if py.shape[0] != n or pz.shape[0] != n:
            raise ValueError("x, y and z must have the same length")
        labels = np.empty(n, dtype=np.int32)
    ng = ctypes.c_int64(0)
    st = _lib.lib().halma_fof_segmented(n, _lib.ptr(px), _lib.ptr(py), _lib.ptr(pz), ns, _lib.ptr(off),
                                        float(linking_length), _lib.ptr(labels), ctypes.byref(ng),
                                        _lib.stream_of(px, labels))
    _lib.check(st, "halma_fof_segmented")
    return labels


def _csr(groups):
    lens = np.fromiter((len(g) for g in groups), dtype=np.int64, count=len(groups))
    offsets = np.zeros(len(groups) + 1, dtype=np.int64)
    np.cumsum(lens, out=offsets[1:])
    if offsets[-1] > 0:
        members = np.concatenate([np.asarray(g, dtype=np.int64) for g in groups if len(g) > 0])
    else:
        members = np.zeros(0, dtype=np.int64)
    return offsets, members


def sub_friends_of_friends(st_x, st_y, st_z, part_lists, linking_length):
    """For every index list pl: fof.friends_of_friends_serial(st_x[pl], st_y[pl], st_z[pl], LL)
    (fof.py:87-89) — groups of local indices into pl, ascending, ordered by smallest member."""
    from . import fof
    offsets, members = _csr(part_lists)
    gx, gy, gz = (np.ascontiguousarray(np.asarray(a, dtype=np.float64)[members]) for a in (st_x, st_y, st_z))
    lab = fof_segmented_labels(gx, gy, gz, offsets, linking_length)
    goff, gmem = fof.fof_groups(lab, 2)
    out = [[] for _ in part_lists]
    seg = np.searchsorted(offsets, np.asarray(gmem)[np.asarray(goff[:-1])], side="right") - 1 if len(goff) > 1 \
        else np.zeros(0, dtype=np.int64)
    for g in range(len(goff) - 1):
        s = int(seg[g])
        out[s].append((np.asarray(gmem[goff[g]:goff[g + 1]]) - offsets[s]).tolist())
    return out


def identify_substructure(groups, st_x, st_y, st_z, st_mass, LL, MINP_SUB, DEC_FACTOR, MIN_LL, DIST_FACTOR, MINP):
    """pyHALMA.py:703-766 for all groups at once.

    groups: the FoF groups after ``good_groups(groups, MINP)`` (sequences of snapshot indices,
    ascending, as FoF returns them).  Lengths (LL, MIN_LL) in the unit of the positions.
    Returns (groups, counter_sub): ``groups`` as the block leaves it (a 1-D object array of
    index lists), ``counter_sub`` the number of sub-groups cut off.
    """
    offsets, members = _csr(groups)
    if members.size and (members.min() < 0 or members.max() >= len(st_x)):
        raise ValueError("group members must be indices into the particle arrays")
    start = np.zeros(members.size, dtype=bool)
    start[offsets[:-1][offsets[:-1] < offsets[1:]]] = True
    if members.size > 1 and np.any((np.diff(members) <= 0) & ~start[1:]):
        raise ValueError("group members must be strictly ascending within each group (as FoF returns them)")
    x, y, z, m = (_lib.as_host(a, np.float64) for a in (st_x, st_y, st_z, st_mass))
    mem32 = np.ascontiguousarray(members, dtype=np.int32)
    params = _lib.SubstructureParams(float(LL), float(DEC_FACTOR), float(MIN_LL), float(DIST_FACTOR),
                                     int(MINP_SUB), int(MINP))
    cap = len(groups) + members.size // max(2, int(MINP_SUB)) + 1
    out_off = np.zeros(cap + 1, dtype=np.int64)
    out_mem = np.empty(max(members.size, 1), dtype=np.int32)
    n_out = ctypes.c_int64(0)
    n_cut = ctypes.c_int64(0)
    st = _lib.lib().halma_split_bridges(x.shape[0], _lib.ptr(x), _lib.ptr(y), _lib.ptr(z), _lib.ptr(m), len(groups),
                                        _lib.ptr(offsets), _lib.ptr(mem32), ctypes.byref(params),
                                        ctypes.byref(n_out), cap, _lib.ptr(out_off), _lib.ptr(out_mem),
                                        ctypes.byref(n_cut), None)
    _lib.check(st, "halma_split_bridges")
    G = int(n_out.value)
    res = np.empty(G, dtype=object)
    for g in range(G):
        res[g] = out_mem[out_off[g]:out_off[g + 1]].tolist()
    return res, int(n_cut.value)
