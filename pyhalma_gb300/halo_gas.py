"""Drop-in replacement of the potential paths of python_scripts/halo_gas.py (pyHALMA).

* ``brute_force_binding_energy_fortran(total_mass, total_x, total_y, total_z,
  test_x, test_y, test_z)``                                   halo_gas.py:164-187
* ``serial_brute_force_binding_energy_fortran(...)``          halo_gas.py:191-215
* ``RPS(...)``                                                halo_gas.py:285-492
* ``most_bound_particle(...)``                                halo_gas.py:498-634
* ``parallel_inside(...)``, ``st_gas_dm_particles_inside(...)`` halo_gas.py:218-277 (ball
  gather on the GPU; ``balls_inside`` does many haloes' spheres in one call)

The f2py kernel particle.particle.brute_force_binding_energy (particle_subroutines.f90:466-514)
is replaced by ``halma_bf_potential_f32``.  Like the wrapper it casts every input to float32
and returns a float32 array, or ``np.array([])`` when there are no test points.

``POTENTIAL_MODE`` chooses the kernel:
  "reference" (default) — float32 sequential sum per target in source order, each operation
                          rounded on its own: bit-identical to the Fortran loop;
  "fast"                — float32 rsqrt pair terms with compensated summation (closer to the
                          FP64 value, several times faster).
RPS and most_bound_particle reproduce the reference's host logic operation by operation —
source sub-sampling with ``np.random.choice`` (same calls in the same order, so a seeded
``np.random`` gives the same sample), the N/n_sample rescaling, the DM species split, the
energy formula E = 1/2 |v - v_bulk|^2 - 2 G phi with G = 4.3e-9 (km/s)^2 Mpc / Msun and the
mass tallies — with every potential evaluated on the GPU.
"""
from __future__ import annotations

import numpy as np

from . import _lib

POTENTIAL_MODE = "reference"
_MODES = {"reference": _lib.POT_REFERENCE, "fast": _lib.POT_FAST}


def bf_potential(total_mass, total_x, total_y, total_z, test_x, test_y, test_z, mode=None, eps2=0.0):
    """phi_i = sum_j m_j / sqrt(r_ij^2 + eps2) over sources whose x, y, z all differ from i's.

    Host inputs are cast to float32 NumPy arrays (as the f2py wrapper does); CUDA torch
    float32 tensors are used in place and the result stays on the device.
    """
    mode = _MODES[mode or POTENTIAL_MODE]
    if _lib._is_torch(test_x):
        nt = int(test_x.shape[0])
        ns = int(total_mass.shape[0])
        out = _lib.like(test_x, (nt,), np.float32)
        args = (total_mass, total_x, total_y, total_z, test_x, test_y, test_z)
    else:
        args = tuple(_lib.as_host(a, np.float32) for a in
                     (total_mass, total_x, total_y, total_z, test_x, test_y, test_z))
        ns = args[0].shape[0]
        nt = args[4].shape[0]
        if any(a.shape[0] != ns for a in args[1:4]) or any(a.shape[0] != nt for a in args[5:]):
            raise ValueError("source (or target) arrays must have equal lengths")
        out = np.empty(nt, dtype=np.float32)
    if nt == 0:
        return out
    m, x, y, z, tx, ty, tz = args
    st = _lib.lib().halma_bf_potential_f32(ns, _lib.ptr(m), _lib.ptr(x), _lib.ptr(y), _lib.ptr(z), nt,
                                           _lib.ptr(tx), _lib.ptr(ty), _lib.ptr(tz), _lib.ptr(out),
                                           mode, float(eps2), _lib.stream_of(tx, out))
    _lib.check(st, "halma_bf_potential_f32")
    return out


def brute_force_binding_energy_fortran(total_mass, total_x, total_y, total_z, test_x, test_y, test_z):
    if len(test_x) == 0:
        return np.array([])
    return bf_potential(total_mass, total_x, total_y, total_z, test_x, test_y, test_z)


def serial_brute_force_binding_energy_fortran(total_mass, total_x, total_y, total_z, test_x, test_y, test_z):
    # the reference's serial twin (f90:517-556) computes the same sums as the OpenMP one
    return brute_force_binding_energy_fortran(total_mass, total_x, total_y, total_z, test_x, test_y, test_z)


def _sampled_potential(src_m, src_x, src_y, src_z, tx, ty, tz, lim):
    """Potential of one source family, sub-sampled with replacement above ``lim`` sources
    (halo_gas.py:306-321): n_sample = max(lim, int(0.01 N)), result scaled by N / n_sample."""
    n = len(src_x)
    if n > lim:
        nsample = np.max([lim, int(0.01 * n)])
        pick = np.random.choice(np.arange(n), nsample, replace=True)
        phi = brute_force_binding_energy_fortran(src_m[pick], src_x[pick], src_y[pick], src_z[pick], tx, ty, tz)
        return phi * n / nsample
    if n > 0:
        return brute_force_binding_energy_fortran(src_m, src_x, src_y, src_z, tx, ty, tz)
    return None


def _dm_potential(dm_x, dm_y, dm_z, dm_mass, tx, ty, tz, lim, mass_dm_part, split_species):
    """Dark-matter term (halo_gas.py:331-410): with several species the two heaviest levels
    (m >= 0.9 * mass_dm_part / 8) are always summed in full and the rest is sub-sampled."""
    terms = []
    if split_species:
        heavy = dm_mass >= 0.9 * (mass_dm_part / 8)
        if np.count_nonzero(heavy) > 0:
            terms.append(brute_force_binding_energy_fortran(dm_mass[heavy], dm_x[heavy], dm_y[heavy],
                                                            dm_z[heavy], tx, ty, tz))
        light = np.logical_not(heavy)
        t = _sampled_potential(dm_mass[light], dm_x[light], dm_y[light], dm_z[light], tx, ty, tz, lim)
    else:
        t = _sampled_potential(dm_mass, dm_x, dm_y, dm_z, tx, ty, tz, lim)
    if t is not None:
        terms.append(t)
    return terms


G_MPC = 4.3 * 1e-3 * 1e-6   # (km/s)^2 Mpc / Msun, halo_gas.py:459-460


def RPS(gas_x, gas_y, gas_z, gas_vx, gas_vy, gas_vz, gas_mass, gas_temp,
        dm_x, dm_y, dm_z, dm_mass, st_x, st_y, st_z, st_mass, vx, vy, vz, BRUTE_FORCE_LIM,
        mass_dm_part, num_dm_species):
    """Bound/unbound gas masses of one halo (ram-pressure stripping), halo_gas.py:285-492.

    Returns (total gas mass, cold bound fraction, unbound cold mass, unbound hot mass)."""
    ngas = len(gas_x)
    phi = np.zeros((ngas,), dtype=np.float32)
    t = _sampled_potential(gas_mass, gas_x, gas_y, gas_z, gas_x, gas_y, gas_z, BRUTE_FORCE_LIM)
    if t is not None:
        phi += t
    for t in _dm_potential(dm_x, dm_y, dm_z, dm_mass, gas_x, gas_y, gas_z, BRUTE_FORCE_LIM, mass_dm_part,
                           num_dm_species > 1):
        phi += t
    t = _sampled_potential(st_mass, st_x, st_y, st_z, gas_x, gas_y, gas_z, BRUTE_FORCE_LIM)
    if t is not None:
        phi += t
    # potential energy per unit mass, km^2 s^-2, with the reference's factor 2 (halo_gas.py:465)
    epot = -phi
    epot *= G_MPC
    epot *= 2.
    ekin = 0.5 * ((gas_vx - vx) ** 2 + (gas_vy - vy) ** 2 + (gas_vz - vz) ** 2)
    energy = ekin + epot
    unbound = energy > 0.
    bound = energy <= 0.
    cold = gas_temp < 5 * 1e4
    hot = gas_temp >= 5 * 1e4
    total_gas_mass = np.sum(gas_mass)
    cold_bound = np.sum(gas_mass[cold * bound])
    frac_cold = cold_bound / total_gas_mass if total_gas_mass != 0. else 0.
    return total_gas_mass, frac_cold, np.sum(gas_mass[unbound * cold]), np.sum(gas_mass[unbound * hot])


def most_bound_particle(gas_x, gas_y, gas_z, gas_mass, dm_x, dm_y, dm_z, dm_mass,
                        st_x, st_y, st_z, st_mass, st_oripa, BRUTE_FORCE_LIM, mass_dm_part):
    """Position and id of the star with the deepest potential, halo_gas.py:498-634."""
    nst = len(st_x)
    phi = np.zeros((nst,), dtype=np.float32)
    t = _sampled_potential(gas_mass, gas_x, gas_y, gas_z, st_x, st_y, st_z, BRUTE_FORCE_LIM)
    if t is not None:
        phi += t
    for t in _dm_potential(dm_x, dm_y, dm_z, dm_mass, st_x, st_y, st_z, BRUTE_FORCE_LIM, mass_dm_part, True):
        phi += t
    t = _sampled_potential(st_mass, st_x, st_y, st_z, st_x, st_y, st_z, BRUTE_FORCE_LIM)
    if t is not None:
        phi += t
    k = np.argmin(-phi)
    return st_x[k], st_y[k], st_z[k], st_oripa[k]


# ---------------------------------------------------------------------------------------
# ball gather (halo_gas.py:218-277)
# ---------------------------------------------------------------------------------------
def balls_inside(x, y, z, cx, cy, cz, R, strict=False):
    """Particles inside many spheres at once (C ABI ``halma_ball_gather``).

    cx, cy, cz, R: one entry per sphere.  Returns CSR (offsets int64 [K+1], indices int32),
    each sphere's indices ascending.  strict=False: ((dx*dx + dy*dy) + dz*dz) <= R*R, the
    pair rule of ``KDTree.query_ball_point``; strict=True: sqrt(...) < R, ``parallel_inside``.
    Host NumPy arrays or CUDA torch tensors (outputs on the same side).
    """
    import ctypes
    if _lib._is_torch(x):
        n = int(x.shape[0])
        px, py, pz = x, y, z
        b = tuple(a.to(dtype=x.dtype).reshape(-1).contiguous() for a in (cx, cy, cz, R))
    else:
        px, py, pz = (_lib.as_host(a, np.float64) for a in (x, y, z))
        n = px.shape[0]
        b = tuple(np.atleast_1d(_lib.as_host(a, np.float64)) for a in (cx, cy, cz, R))
    k = int(b[0].shape[0])
    if any(int(a.shape[0]) != k for a in b):
        raise ValueError("cx, cy, cz and R must have the same length")
    offsets = _lib.like(px, (k + 1,), np.int64)
    found = ctypes.c_int64(0)
    L = _lib.lib()
    st = L.halma_ball_gather(n, _lib.ptr(px), _lib.ptr(py), _lib.ptr(pz), k, *[_lib.ptr(a) for a in b],
                             1 if strict else 0, _lib.ptr(offsets), None, 0, ctypes.byref(found),
                             _lib.stream_of(px))
    _lib.check(st, "halma_ball_gather")
    total = int(found.value)
    indices = _lib.like(px, (max(total, 1),), np.int32)
    if total > 0:
        st = L.halma_ball_gather(n, _lib.ptr(px), _lib.ptr(py), _lib.ptr(pz), k, *[_lib.ptr(a) for a in b],
                                 1 if strict else 0, _lib.ptr(offsets), _lib.ptr(indices), total,
                                 ctypes.byref(found), _lib.stream_of(px))
        _lib.check(st, "halma_ball_gather")
    return offsets, indices[:total]


def query_ball_point(x, y, z, centre, R):
    """``KDTree(np.array((x, y, z)).T).query_ball_point(centre, R)`` for one centre: the
    indices within R (inclusive), ascending (the KDTree returns the same set in tree order)."""
    _, idx = balls_inside(x, y, z, [centre[0]], [centre[1]], [centre[2]], [R])
    return idx


def parallel_inside(array_x, array_y, array_z, R, cx, cy, cz):
    """halo_gas.py:218-220: boolean mask sqrt((x-cx)**2 + (y-cy)**2 + (z-cz)**2) < R."""
    n = len(array_x)
    _, idx = balls_inside(array_x, array_y, array_z, [cx], [cy], [cz], [R], strict=True)
    mask = np.zeros(n, dtype=bool)
    mask[np.asarray(idx)] = True
    return mask


MASS_TO_SUN = 1.0   # masclet_framework units.mass_to_sun: set it when masses come in MASCLET units


def st_gas_dm_particles_inside(rete, L, ncoarse, grid_data, gas_data, masclet_dm_data, masclet_st_data,
                               st_kdtree, dm_kdtree, cx, cy, cz, R, rho_B):
    """halo_gas.py:223-277 with the particle side on the GPU.

    ``gas_data`` is the gas already turned into particles — the tuple (gas_x, gas_y, gas_z,
    gas_vx, gas_vy, gas_vz, gas_mass, gas_temp) that ``AMRgrid_to_particles`` (halo_gas.py:
    56-141) returns; that conversion reads MASCLET AMR grids and is not part of this package,
    so ``L``, ``ncoarse``, ``grid_data`` and ``rho_B`` are accepted and unused.  The KD-trees
    are replaced by the GPU ball gather (``st_kdtree`` / ``dm_kdtree`` are unused), so the DM
    and star selections come back in ascending index order instead of tree order.  Returns the
    reference's 17-tuple.
    """
    if grid_data is not None:
        raise NotImplementedError("AMR grid to particle conversion needs MASCLET grids; pass the gas as "
                                  "particles in gas_data and grid_data=None")
    gas_x, gas_y, gas_z, gas_vx, gas_vy, gas_vz, gas_mass, gas_temp = (np.asarray(a) for a in gas_data)
    inside = parallel_inside(gas_x, gas_y, gas_z, R, cx, cy, cz)
    gas_x, gas_y, gas_z = gas_x[inside], gas_y[inside], gas_z[inside]
    gas_vx, gas_vy, gas_vz = gas_vx[inside], gas_vy[inside], gas_vz[inside]
    gas_mass, gas_temp = gas_mass[inside], gas_temp[inside]
    gas_mass = gas_mass * rete ** 3      # comoving to physical volume (halo_gas.py:247)
    dm_x, dm_y, dm_z = (np.asarray(masclet_dm_data[k]) for k in range(3))
    dm_mass = np.asarray(masclet_dm_data[3]) * MASS_TO_SUN   # halo_gas.py:253
    sel = np.asarray(query_ball_point(dm_x, dm_y, dm_z, (cx, cy, cz), R))
    dm_x, dm_y, dm_z, dm_mass = dm_x[sel], dm_y[sel], dm_z[sel], dm_mass[sel]
    st_x, st_y, st_z = (np.asarray(masclet_st_data[k]) for k in range(3))
    st_mass, st_oripa = np.asarray(masclet_st_data[6]) * MASS_TO_SUN, np.asarray(masclet_st_data[9])
    sel = np.asarray(query_ball_point(st_x, st_y, st_z, (cx, cy, cz), R))
    st_x, st_y, st_z, st_mass, st_oripa = st_x[sel], st_y[sel], st_z[sel], st_mass[sel], st_oripa[sel]
    return (gas_x, gas_y, gas_z, gas_vx, gas_vy, gas_vz, gas_mass, gas_temp,
            dm_x, dm_y, dm_z, dm_mass, st_x, st_y, st_z, st_mass, st_oripa)
