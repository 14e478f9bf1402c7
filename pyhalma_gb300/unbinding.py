"""Batched iterative unbinding and the one-call snapshot pipeline.

``unbind_batched`` runs pyHALMA's single-pass escape cut (python_scripts/halo_properties.py:
282-361) repeatedly on thousands of haloes at once (C ABI ``halma_unbind_batched``):

    phi_i = sum_{j != i} m_j / sqrt(r_ij^2 + eps^2)          (bound particles only)
    E_i   = 1/2 |v_i - v_bulk|^2 - G * factor_v^2 * phi_i      (FP64)
    remove every particle with E_i > 0, recompute the FP64 bound mass, centre of mass and
    bulk velocity, repeat until a pass removes nothing (or max_iter passes).

precision="fp32c" — float32 pair terms with compensated summation in one persistent
                    work-queue kernel per pass, all passes replayed from one CUDA graph;
precision="fp64"  — the plain per-halo path: FP64 pair sums, one launch per halo per pass.

``find_haloes`` is the whole star-particle path of the main script pyHALMA.py (FoF, good_groups, unbinding)
in one C-ABI call (``halma_find_haloes``).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib

G_MPC = 4.3e-9   # (km/s)^2 Mpc / Msun, halo_gas.py:459-460
_PREC = {"fp32c": _lib.UNBIND_FP32C, "fp64": _lib.UNBIND_FP64}
_table_loaded = False


def _ensure_tile_table():
    """Loads the autotuner's saved tile table once per process (if one was saved)."""
    global _table_loaded
    if not _table_loaded:
        from . import autotune
        autotune.apply()
        _table_loaded = True


@dataclass
class UnbindOptions:
    eps: float = 1e-4          # softening, Mpc (0.1 kpc)
    G: float = G_MPC
    factor_v: float = 1.0
    max_iter: int = 20
    precision: str = "fp32c"
    use_graph: bool = True
    incremental: bool = True   # later passes subtract the removed particles' potential

    def params(self):
        flags = 0 if self.incremental else _lib.UNBIND_FULL_RECOMPUTE
        return _lib.UnbindParams(float(self.eps), float(self.G), float(self.factor_v), int(self.max_iter),
                                 _PREC[self.precision], int(bool(self.use_graph)), flags)


def unbind_batched(offsets, x, y, z, vx, vy, vz, m, options: UnbindOptions | None = None, want_phi=False, **kw):
    """Returns (bound uint8 [n], halo table [n_haloes, 11], phi [n] or None).

    Arrays are host NumPy (copied in and out) or CUDA torch tensors (used in place).
    """
    opt = options or UnbindOptions(**kw)
    _ensure_tile_table()
    dev = _lib._is_torch(x)
    if dev:
        n = int(x.shape[0])
        nh = int(offsets.shape[0]) - 1
        arrs = (offsets, x, y, z, vx, vy, vz, m)
    else:
        offsets = _lib.as_host(offsets, np.int64)
        arrs = (offsets,) + tuple(_lib.as_host(a, np.float64) for a in (x, y, z, vx, vy, vz, m))
        n = arrs[1].shape[0]
        nh = offsets.shape[0] - 1
    _lib.check_arrays(np.int64, None, offsets=arrs[0])
    _lib.check_arrays(np.float64, n, **dict(zip(("x", "y", "z", "vx", "vy", "vz", "m"), arrs[1:])))
    bound = _lib.like(arrs[1], (n,), np.uint8)
    halo = _lib.like(arrs[1], (max(nh, 0), len(_lib.UB_FIELDS)), np.float64)
    phi = _lib.like(arrs[1], (n,), np.float64) if want_phi else None
    if nh <= 0:
        return bound, halo, phi
    p = opt.params()
    st = _lib.lib().halma_unbind_batched(n, nh, *[_lib.ptr(a) for a in arrs], ctypes.byref(p), _lib.ptr(bound),
                                         _lib.ptr(phi), _lib.ptr(halo), _lib.stream_of(*arrs))
    _lib.check(st, "halma_unbind_batched")
    return bound, halo, phi


@dataclass
class HaloCatalogue:
    labels: object          # FoF labels (min index, -1 alone)
    bound: object           # 1 = member of a kept group that survived unbinding
    offsets: object         # groups as CSR over particle indices (reference order)
    members: object
    haloes: object          # [n_haloes, 11] unbinding table (UB_FIELDS)

    @property
    def n_haloes(self):
        return int(self.offsets.shape[0]) - 1


def find_haloes(st_x, st_y, st_z, st_vx, st_vy, st_vz, st_mass, linking_length, minp=50,
                options: UnbindOptions | None = None, **kw):
    """FoF (fof.py:18-79) + good_groups (pyHALMA.py:148-149) + batched unbinding, one call."""
    opt = options or UnbindOptions(**kw)
    _ensure_tile_table()
    dev = _lib._is_torch(st_x)
    if dev:
        arrs = (st_x, st_y, st_z, st_vx, st_vy, st_vz, st_mass)
        n = int(st_x.shape[0])
    else:
        arrs = tuple(_lib.as_host(a, np.float64) for a in (st_x, st_y, st_z, st_vx, st_vy, st_vz, st_mass))
        n = arrs[0].shape[0]
    _lib.check_arrays(np.float64, n, **dict(zip(("st_x", "st_y", "st_z", "st_vx", "st_vy", "st_vz", "st_mass"), arrs)))
    cap = max(n // max(int(minp), 2) + 1, 1)
    # host outputs in pinned memory: their copies are DMA transfers that overlap the unbinding
    out = _lib.like if dev else (lambda a, shape, dtype: _lib.pinned_empty(shape, dtype))
    labels = out(arrs[0], (n,), np.int32)
    bound = out(arrs[0], (n,), np.uint8)
    offsets = out(arrs[0], (cap + 1,), np.int64)
    members = out(arrs[0], (max(n, 1),), np.int32)
    haloes = out(arrs[0], (cap, len(_lib.UB_FIELDS)), np.float64)
    nh = ctypes.c_int64(0)
    p = opt.params()
    st = _lib.lib().halma_find_haloes(n, *[_lib.ptr(a) for a in arrs], float(linking_length), int(minp),
                                      ctypes.byref(p), _lib.ptr(labels), _lib.ptr(bound), ctypes.byref(nh), cap,
                                      _lib.ptr(offsets), _lib.ptr(members), _lib.ptr(haloes),
                                      _lib.stream_of(*arrs))
    _lib.check(st, "halma_find_haloes")
    g = int(nh.value)
    offsets = offsets[: g + 1]
    nm = int(offsets[-1]) if g > 0 else 0
    return HaloCatalogue(labels, bound, offsets, members[:nm], haloes[:g])
