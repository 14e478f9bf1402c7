"""Drop-in replacement of python_scripts/fof.py (pyHALMA) backed by the GB300 FoF kernels.

Same function names, arguments and return types as the reference module:

* ``friends_of_friends(data, linking_length)``                       fof.py:18-79
* ``friends_of_friends_serial(st_x, st_y, st_z, linking_length)``    fof.py:87-89
* ``friends_of_friends_parallel(st_x, st_y, st_z, linking_length, L, minp, st_mass)``
                                                                      fof.py:95-176
* ``pyfof_friends_of_friends_serial`` / ``pyfof_friends_of_friends_parallel``
                                                                      fof.py:184-187, 192-272
* ``good_groups(groups, minp)``                                       pyHALMA.py:148-149

The serial functions return exactly the reference's value: a list of groups (lists of
Python ints, ascending), ordered by smallest member, singletons dropped.  The "parallel"
variants of the reference cut the box into n^3 sub-cubes with a 0.1 Mpc buffer and keep
groups with more than ``minp`` members whose centre of mass lies in their cube, which can
split or lose groups longer than the buffer; here they return the exact global partition
filtered with the same strict ``len(group) > minp`` rule, as NumPy index arrays like the
reference.  The GPU computes the partition, the ordering and the size filter.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def fof_labels(x, y, z, linking_length, boxsize=None):
    """Canonical FoF labels: smallest member index of each particle's group, -1 if alone.

    x, y, z: float64 NumPy arrays (host) or CUDA torch tensors (device, used in place).
    boxsize: None (non-periodic, as fof.py) or the side of a periodic box [0, boxsize)^3 whose
    faces the groups may cross (nearest-image distances; boxsize >= 3 linking lengths).
    Returns int32 labels on the same side as the inputs.
    """
    if _lib._is_torch(x):
        n = int(x.shape[0])
        _lib.check_arrays(np.float64, n, x=x, y=y, z=z)
        labels = _lib.like(x, (n,), np.int32)
        px, py, pz = x, y, z
    else:
        px = _lib.as_host(x, np.float64)
        py = _lib.as_host(y, np.float64)
        pz = _lib.as_host(z, np.float64)
        n = px.shape[0]
        if py.shape[0] != n or pz.shape[0] != n:
            raise ValueError("x, y and z must have the same length")
        labels = np.empty(n, dtype=np.int32)
    ng = ctypes.c_int64(0)
    if boxsize is None:
        st = _lib.lib().halma_fof(n, _lib.ptr(px), _lib.ptr(py), _lib.ptr(pz), float(linking_length),
                                  _lib.ptr(labels), ctypes.byref(ng), _lib.stream_of(px, labels))
        _lib.check(st, "halma_fof")
    else:
        st = _lib.lib().halma_fof_periodic(n, _lib.ptr(px), _lib.ptr(py), _lib.ptr(pz), float(linking_length),
                                           float(boxsize), _lib.ptr(labels), ctypes.byref(ng),
                                           _lib.stream_of(px, labels))
        _lib.check(st, "halma_fof_periodic")
    return labels


def fof_groups(labels, min_members=2):
    """Groups as CSR (offsets int64 [G+1], members int32) in the reference order."""
    if _lib._is_torch(labels):
        n = int(labels.shape[0])
        _lib.check_arrays(np.int32, n, labels=labels)
        offsets = _lib.like(labels, (n + 1,), np.int64)
        members = _lib.like(labels, (max(n, 1),), np.int32)
    else:
        labels = _lib.as_host(labels, np.int32)
        n = labels.shape[0]
        offsets = np.zeros(n + 1, dtype=np.int64)
        members = np.empty(max(n, 1), dtype=np.int32)
    ng = ctypes.c_int64(0)
    st = _lib.lib().halma_fof_groups(n, _lib.ptr(labels), int(min_members), _lib.ptr(offsets),
                                     _lib.ptr(members), ctypes.byref(ng), _lib.stream_of(labels))
    _lib.check(st, "halma_fof_groups")
    g = int(ng.value)
    offsets = offsets[: g + 1]
    return offsets, members[: int(offsets[-1])] if g > 0 else members[:0]


def _split(offsets, members):
    offsets = np.asarray(offsets)
    members = np.asarray(members)
    return [members[offsets[g]:offsets[g + 1]] for g in range(len(offsets) - 1)]


def friends_of_friends(data, linking_length, boxsize=None):
    """fof.py:18-79; ``boxsize`` (an addition, None by default as in the reference) makes the
    box periodic, as ``KDTree(data, boxsize=...)`` would."""
    data = np.asarray(data, dtype=np.float64)
    if data.ndim != 2 or data.shape[1] != 3:
        raise ValueError("data must have shape (N, 3)")
    lab = fof_labels(np.ascontiguousarray(data[:, 0]), np.ascontiguousarray(data[:, 1]),
                     np.ascontiguousarray(data[:, 2]), linking_length, boxsize)
    off, mem = fof_groups(lab, 2)
    return [g.tolist() for g in _split(off, mem)]


def friends_of_friends_serial(st_x, st_y, st_z, linking_length, boxsize=None):
    lab = fof_labels(st_x, st_y, st_z, linking_length, boxsize)
    off, mem = fof_groups(lab, 2)
    return [g.tolist() for g in _split(off, mem)]


def friends_of_friends_parallel(st_x, st_y, st_z, linking_length, L, minp, st_mass):
    lab = fof_labels(st_x, st_y, st_z, linking_length)
    off, mem = fof_groups(lab, int(minp) + 1)          # reference keeps len > minp
    return [g.astype(np.int64) for g in _split(off, mem)]


def pyfof_friends_of_friends_serial(st_x, st_y, st_z, linking_length):
    return friends_of_friends_serial(st_x, st_y, st_z, linking_length)


def pyfof_friends_of_friends_parallel(st_x, st_y, st_z, linking_length, L, minp, st_mass):
    return friends_of_friends_parallel(st_x, st_y, st_z, linking_length, L, minp, st_mass)


def good_groups(groups, minp):
    return np.array([len(groups[ig]) >= minp for ig in range(len(groups))], dtype=bool)
