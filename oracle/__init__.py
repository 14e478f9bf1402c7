"""ORACLE — test infrastructure, not product code.

CPU restatements of pyHALMA's halo-finding hot path, used only by ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` to check (or time
beside) the CUDA path.  The product package ``pyhalma_gb300`` never imports this package.

* ``potential_oracle.c``  — float32 restatement of particle_subroutines.f90:466-514 and an
  FP64 twin (softening, self mask) plus its FP64 gradient.
* ``fof_oracle.c``        — exact FoF partition with scipy's pinned pair predicate.
* ``fof_kdtree.py``       — the reference's KDTree flood fill (fof.py:18-79) restated.
* ``reductions.py``       — FP64 per-halo reductions (halo_properties.py).
* ``unbind.py``           — iterative FP64 unbinding composed from the single-pass cut.

``build()`` compiles the C files with gcc into ``oracle/_build/liboracle.so``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "liboracle.so")
_SOURCES = ["potential_oracle.c", "fof_oracle.c"]
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the C oracle (gcc, OpenMP, no FMA contraction, no fast-math)."""
    srcs = [os.path.join(_HERE, s) for s in _SOURCES]
    if not force and os.path.exists(_LIB_PATH):
        newest = max(os.path.getmtime(s) for s in srcs)
        if os.path.getmtime(_LIB_PATH) >= newest:
            return _LIB_PATH
    os.makedirs(_BUILD, exist_ok=True)
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
           "-shared", "-o", tmp, *srcs, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            path = build()
            L = ctypes.CDLL(path)
            P = ctypes.c_void_p
            i32, i64, f64 = ctypes.c_int32, ctypes.c_int64, ctypes.c_double
            L.oracle_bf_potential_f32.argtypes = [i32, i32, P, P, P, P, i32, P, P, P, P]
            L.oracle_bf_potential_f32.restype = None
            L.oracle_potential_f64.argtypes = [i32, i64, P, P, P, P, i64, P, P, P, f64, i32, i64, P]
            L.oracle_potential_f64.restype = None
            L.oracle_potential_grad_f64.argtypes = [i32, i64, P, P, P, P, i64, P, P, P, P, f64,
                                                   i32, i64, P, P, P]
            L.oracle_potential_grad_f64.restype = None
            L.oracle_fof_labels.argtypes = [i64, P, P, P, f64, P]
            L.oracle_fof_labels.restype = ctypes.c_int
            _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def ncores_default() -> int:
    return max(1, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count())


def bf_potential_f32(total_mass, total_x, total_y, total_z, test_x, test_y, test_z, ncores=None):
    """float32 sequential potential exactly as particle_subroutines.f90:466-514."""
    c = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    m, x, y, z = c(total_mass), c(total_x), c(total_y), c(total_z)
    tx, ty, tz = c(test_x), c(test_y), c(test_z)
    out = np.zeros(tx.shape[0], dtype=np.float32)
    lib().oracle_bf_potential_f32(int(ncores or ncores_default()), m.shape[0], _ptr(m), _ptr(x),
                                  _ptr(y), _ptr(z), tx.shape[0], _ptr(tx), _ptr(ty), _ptr(tz),
                                  _ptr(out))
    return out


MASK_COORD, MASK_SELF, MASK_NONE = 0, 1, 2


def potential_f64(m, x, y, z, tx, ty, tz, eps2=0.0, mask=MASK_COORD, self_offset=0, ncores=None):
    c = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    m, x, y, z, tx, ty, tz = map(c, (m, x, y, z, tx, ty, tz))
    out = np.zeros(tx.shape[0], dtype=np.float64)
    lib().oracle_potential_f64(int(ncores or ncores_default()), m.shape[0], _ptr(m), _ptr(x),
                               _ptr(y), _ptr(z), tx.shape[0], _ptr(tx), _ptr(ty), _ptr(tz),
                               float(eps2), int(mask), int(self_offset), _ptr(out))
    return out


def potential_grad_f64(m, x, y, z, tx, ty, tz, g, eps2=0.0, mask=MASK_NONE, self_offset=0,
                       ncores=None):
    """Returns (dL/dm [ns], dL/dsource_pos [ns,3], dL/dtarget_pos [nt,3])."""
    c = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    m, x, y, z, tx, ty, tz, g = map(c, (m, x, y, z, tx, ty, tz, g))
    gm = np.zeros(m.shape[0])
    gs = np.zeros((m.shape[0], 3))
    gt = np.zeros((tx.shape[0], 3))
    lib().oracle_potential_grad_f64(int(ncores or ncores_default()), m.shape[0], _ptr(m),
                                    _ptr(x), _ptr(y), _ptr(z), tx.shape[0], _ptr(tx), _ptr(ty),
                                    _ptr(tz), _ptr(g), float(eps2), int(mask), int(self_offset),
                                    _ptr(gm), _ptr(gs), _ptr(gt))
    return gm, gs, gt


def fof_labels(x, y, z, linking_length):
    """Exact FoF labels (min index of the component, -1 for particles without friends)."""
    c = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    x, y, z = c(x), c(y), c(z)
    out = np.empty(x.shape[0], dtype=np.int32)
    rc = lib().oracle_fof_labels(x.shape[0], _ptr(x), _ptr(y), _ptr(z), float(linking_length),
                                 _ptr(out))
    if rc != 0:
        raise RuntimeError(f"oracle_fof_labels failed ({rc})")
    return out


def groups_to_labels(groups, n):
    """Reference output (list of index lists) -> canonical labels."""
    lab = np.full(n, -1, dtype=np.int32)
    for g in groups:
        g = np.asarray(g, dtype=np.int64)
        if g.size:
            lab[g] = g.min()
    return lab


def labels_to_groups(labels):
    """Canonical labels -> list of sorted index lists ordered by smallest member."""
    labels = np.asarray(labels)
    idx = np.nonzero(labels >= 0)[0]
    if idx.size == 0:
        return []
    order = np.argsort(labels[idx], kind="stable")
    srt = idx[order]
    lab = labels[srt]
    cut = np.nonzero(np.diff(lab))[0] + 1
    return [g.tolist() for g in np.split(srt, cut)]
