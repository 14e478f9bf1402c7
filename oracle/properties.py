"""ORACLE (test infrastructure only): the O(N) per-halo properties of pyHALMA's main-script loop
(pyHALMA.py:930-1016) restated on the CPU.

NumPy FP64 restatements of the numba functions of python_scripts/halo_properties.py (fastmath,
so their summation order is unspecified; compared at 1e-10 relative):

* ``half_mass_radius_proj``  :397-458  projected half-mass radii along x, y, z;
* ``angular_momentum``       :461-481  specific angular momentum, including the reference's
  z component sum m (rx*vvy - ry*vvz) (vvz where the cross product has vvx);
* ``kinematic_morphology``   :483-515  kappa_co (Correa et al. 2017);
* ``tully_fisher_velocity``  :62-96    mass-weighted rotation speed in 0.9..1.1 R05.

The two Fortran routines go through the C restatement in properties_oracle.c (FP32, one
thread, particle order), with the Python wrappers' casts:

* ``halo_shape_fortran``        halo_properties.py:852-866 -> f90:160-214;
* ``sigma_projections_fortran`` halo_properties.py:781-814 -> f90:217-461.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libproperties_oracle.so")
_lock = threading.Lock()
_lib = None


def build(force=False):
    src = os.path.join(_HERE, "properties_oracle.c")
    if not force and os.path.exists(_LIB_PATH) and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(src):
        return _LIB_PATH
    os.makedirs(os.path.dirname(_LIB_PATH), exist_ok=True)
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-o", tmp, src, "-lm"],
                   check=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            L = ctypes.CDLL(build())
            P, i32, f32 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_float
            L.oracle_halo_shape.argtypes = [i32, P, P, P, P, P]
            L.oracle_halo_shape.restype = None
            L.oracle_sigma_projections.argtypes = [i32, P, i32, P, P, P, P, P, P, P, P, f32, f32, f32, f32, f32, f32,
                                                   f32, P]
            L.oracle_sigma_projections.restype = ctypes.c_int
            _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def half_mass_radius_proj(cx, cy, cz, M, part_list, st_x, st_y, st_z, st_mass):
    pl = np.asarray(part_list)
    dx, dy, dz = cx - st_x[pl], cy - st_y[pl], cz - st_z[pl]
    out = []
    for d in (np.sqrt(dy ** 2 + dz ** 2), np.sqrt(dx ** 2 + dz ** 2), np.sqrt(dx ** 2 + dy ** 2)):
        order = np.argsort(d)
        ds = d[order]
        cm = np.cumsum(st_mass[pl][order])
        k = int(np.argmax(cm > 0.5 * M)) if np.any(cm > 0.5 * M) else len(ds)
        out.append(float(ds[k - 1]) if k > 0 else float(ds[0]))
    return tuple(out)


def _rel(part_list, st_x, st_y, st_z, st_vx, st_vy, st_vz, cx, cy, cz, vx, vy, vz):
    pl = np.asarray(part_list)
    return (st_x[pl] - cx, st_y[pl] - cy, st_z[pl] - cz, st_vx[pl] - vx, st_vy[pl] - vy, st_vz[pl] - vz)


def angular_momentum(M, part_list, st_x, st_y, st_z, st_vx, st_vy, st_vz, st_mass, cx, cy, cz, vx, vy, vz):
    rx, ry, rz, ux, uy, uz = _rel(part_list, st_x, st_y, st_z, st_vx, st_vy, st_vz, cx, cy, cz, vx, vy, vz)
    m = st_mass[np.asarray(part_list)]
    lx = (m * (ry * uz - rz * uy)).sum()
    ly = (m * (rz * ux - rx * uz)).sum()
    lz = (m * (rx * uy - ry * uz)).sum()
    return lx / M, ly / M, lz / M


def kinematic_morphology(part_list, st_x, st_y, st_z, st_vx, st_vy, st_vz, st_mass, cx, cy, cz, vx, vy, vz,
                         lx, ly, lz):
    rx, ry, rz, ux, uy, uz = _rel(part_list, st_x, st_y, st_z, st_vx, st_vy, st_vz, cx, cy, cz, vx, vy, vz)
    m = st_mass[np.asarray(part_list)]
    L = np.array([lx, ly, lz])
    L = L / np.linalg.norm(L)
    llx, lly, llz = m * (ry * uz - rz * uy), m * (rz * ux - rx * uz), m * (rx * uy - ry * ux)
    Lz = (llx * L[0] + lly * L[1]) + llz * L[2]
    z = (rx * L[0] + ry * L[1]) + rz * L[2]
    with np.errstate(invalid="ignore", divide="ignore"):
        R = np.sqrt(rx ** 2 + ry ** 2 + rz ** 2 - z ** 2)
        tot = (0.5 * m * (ux ** 2 + uy ** 2 + uz ** 2)).sum()
        co = np.where(Lz > 0.0, 0.5 * m * (Lz / (m * R)) ** 2, 0.0).sum()
    return co / tot


def tully_fisher_velocity(part_list, cx, cy, cz, st_x, st_y, st_z, vx, vy, vz, lx, ly, lz, st_vx, st_vy, st_vz,
                          st_mass, RAD05):
    rx, ry, rz, ux, uy, uz = _rel(part_list, st_x, st_y, st_z, st_vx, st_vy, st_vz, cx, cy, cz, vx, vy, vz)
    m = st_mass[np.asarray(part_list)]
    L = np.array([lx, ly, lz])
    u = L / np.linalg.norm(L)
    dist = np.sqrt(rx ** 2 + ry ** 2 + rz ** 2)
    sel = (0.9 * RAD05 < dist) & (dist < 1.1 * RAD05)
    r = np.stack([rx, ry, rz], 1)[sel]
    v = np.stack([ux, uy, uz], 1)[sel]
    R = r - (r @ u)[:, None] * u[None, :]
    uR = R / np.linalg.norm(R, axis=1)[:, None]
    vrot = v - (v @ u)[:, None] * u[None, :] - np.sum(v * uR, axis=1)[:, None] * uR
    with np.errstate(invalid="ignore", divide="ignore"):
        return (np.linalg.norm(vrot, axis=1) * m[sel]).sum() / m[sel].sum()


def halo_shape_fortran(part_list, st_x, st_y, st_z, st_mass, cx, cy, cz, RAD05):
    pl = np.asarray(part_list)
    x = np.ascontiguousarray(np.float32(st_x[pl] - cx))
    y = np.ascontiguousarray(np.float32(st_y[pl] - cy))
    z = np.ascontiguousarray(np.float32(st_z[pl] - cz))
    m = np.ascontiguousarray(np.float32(st_mass[pl]))
    out = np.zeros(3, dtype=np.float32)
    lib().oracle_halo_shape(len(pl), _p(x), _p(y), _p(z), _p(m), _p(out))
    return out[0], out[1], out[2]


def sigma_projections_fortran(grid, n_cell, part_list, st_x, st_y, st_z, st_vx, st_vy, st_vz, vx, vy, vz, st_mass,
                              cx, cy, cz, R05x, R05y, R05z, ll):
    f = lambda a: np.ascontiguousarray(np.float32(a))
    g = f(grid)
    pl = np.ascontiguousarray(np.asarray(part_list, dtype=np.int64))
    arrs = [f(st_x), f(st_y), f(st_z), f(st_vx - vx), f(st_vy - vy), f(st_vz - vz), f(st_mass)]
    out = np.zeros(5, dtype=np.float32)
    rc = lib().oracle_sigma_projections(len(pl), _p(g), int(n_cell), _p(pl), *[_p(a) for a in arrs],
                                        *[float(np.float32(v)) for v in (cx, cy, cz, R05x, R05y, R05z, ll)], _p(out))
    if rc != 0:
        raise MemoryError("sigma_projections grid")
    return tuple(out)
