"""Drop-in replacement of the potential paths of python_scripts/halo_gas.py (pyHALMA).

* ``brute_force_binding_energy_fortran(total_mass, total_x, total_y, total_z,
  test_x, test_y, test_z)``                                   halo_gas.py:164-187
* ``serial_brute_force_binding_energy_fortran(...)``          halo_gas.py:191-215
* ``RPS(...)``                                                halo_gas.py:285-492
* ``most_bound_particle(...)``                                halo_gas.py:498-634
* ``parallel_inside(...)``, ``st_gas_dm_particles_inside(...)`` halo_gas.py:218-277 (ball
  gather on the GPU; ``balls_inside`` does many haloes' spheres in one call)
* ``AMRgrid_to_particles(...)``                               halo_gas.py:56-141 (with the
  numba kernel patch_to_particles, :9-52): the box's AMR cells to gas particles on the GPU

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

import ctypes

import numpy as np

from . import _lib

POTENTIAL_MODE = "reference"
_MODES = {"reference": _lib.POT_REFERENCE, "fast": _lib.POT_FAST}

try:   # MASCLET's code mass unit in Msun, when masclet_framework is installed
    from masclet_framework import units as _units
    MASS_TO_SUN = float(_units.mass_to_sun)
except Exception:   # masses are taken as already in Msun
    MASS_TO_SUN = 1.0


def bf_potential(total_mass, total_x, total_y, total_z, test_x, test_y, test_z, mode=None, eps2=0.0):
    """phi_i = sum_j m_j / sqrt(r_ij^2 + eps2) over sources whose x, y, z all differ from i's.

    Host inputs are cast to float32 NumPy arrays (as the f2py wrapper does); CUDA torch
    float32 tensors are used in place and the result stays on the device.
    """
    mode = _MODES[mode or POTENTIAL_MODE]
    if _lib._is_torch(test_x):
        nt = int(test_x.shape[0])
        ns = int(total_mass.shape[0])
        _lib.check_arrays(np.float32, ns, total_mass=total_mass, total_x=total_x, total_y=total_y, total_z=total_z)
        _lib.check_arrays(np.float32, nt, test_x=test_x, test_y=test_y, test_z=test_z)
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
    if _lib._is_torch(x):
        n = int(x.shape[0])
        px, py, pz = x, y, z
        _lib.check_arrays(np.float64, n, x=x, y=y, z=z)
        b = tuple(a.to(dtype=x.dtype).reshape(-1).contiguous() for a in (cx, cy, cz, R))
    else:
        px, py, pz = (_lib.as_host(a, np.float64) for a in (x, y, z))
        n = px.shape[0]
        _lib.check_arrays(np.float64, n, x=px, y=py, z=pz)
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


def create_vector_levels(npatch):
    """Refinement level of every patch: patch 0 is the base grid (level 0), followed by
    npatch[1] patches of level 1, npatch[2] of level 2, ... (the patch numbering of MASCLET
    grids; masclet_framework.tools.create_vector_levels, a third-party helper the reference
    calls at halo_gas.py:91, restated)."""
    npatch = np.asarray(npatch, dtype=np.int64)
    return np.concatenate([np.zeros(1, dtype=np.int64)] +
                          [np.full(int(c), lev, dtype=np.int64) for lev, c in enumerate(npatch[1:], start=1)])


def _patches_in_box(box, levels, patchnx, patchny, patchnz, patchrx, patchry, patchrz, L, ncoarse):
    """Refined patches (level >= 1) whose extent, widened by one cell on each side, meets the
    box, in patch order.  A superset of the patches holding a cell centre strictly inside the
    box; the cell test itself runs in the kernel, so the particles do not depend on how tight
    this preselection is (the reference preselects with masclet_framework.tools.
    which_patches_inside_box, halo_gas.py:90)."""
    lev = np.asarray(levels, dtype=np.int64)
    res = (L / ncoarse) / 2.0 ** lev
    keep = lev >= 1
    for n, r, lo, hi in ((patchnx, patchrx, box[0], box[1]), (patchny, patchry, box[2], box[3]),
                         (patchnz, patchrz, box[4], box[5])):
        n = np.asarray(n, dtype=np.float64)
        r = np.asarray(r, dtype=np.float64)
        keep &= (r - 2.0 * res <= hi) & (r + (n + 1.0) * res >= lo)
    return np.nonzero(keep)[0]


def AMRgrid_to_particles(L, ncoarse, grid_data, gas_data, Rrps, cx, cy, cz, rho_B):
    """halo_gas.py:56-141: one gas particle per leaf cell (cr0amr and solapst true) of the
    refined patches whose centre lies strictly inside the cube of half-side Rrps about
    (cx, cy, cz); returns (x, y, z, vx, vy, vz, mass, temp) float64 arrays in the reference's
    order (patches in order, cells x-major), velocities in km/s (cell values times 3e5) and
    comoving masses (1 + delta) * rho_B * res^3.  ``grid_data`` / ``gas_data`` are the
    reference's MASCLET tuples (grid_data[5] npatch, [6:9] patchnx/ny/nz, [12:15]
    patchrx/ry/rz; gas_data[:7] delta, vx, vy, vz, temp, cr0amr, solapst as per-patch 3-D
    arrays indexed [ix, iy, iz]).  The cell loop runs on the GPU (halma_amr_to_particles);
    cell values are taken in float64 (numba's arithmetic on float32 fields)."""
    npatch = grid_data[5]
    patchnx, patchny, patchnz = grid_data[6], grid_data[7], grid_data[8]
    patchrx, patchry, patchrz = grid_data[12], grid_data[13], grid_data[14]
    gas_delta, gas_vx, gas_vy, gas_vz, gas_temp, gas_cr0amr, gas_solapst = gas_data[:7]
    box = np.array([cx - Rrps, cx + Rrps, cy - Rrps, cy + Rrps, cz - Rrps, cz + Rrps], dtype=np.float64)
    levels = create_vector_levels(npatch)
    sel = _patches_in_box(box, levels, patchnx, patchny, patchnz, patchrx, patchry, patchrz, float(L), int(ncoarse))
    k = len(sel)
    plev = np.ascontiguousarray(levels[sel], dtype=np.int32)
    pn = np.ascontiguousarray(np.stack([np.asarray(patchnx)[sel], np.asarray(patchny)[sel],
                                        np.asarray(patchnz)[sel]], 1), dtype=np.int32).reshape(-1)
    pr = np.ascontiguousarray(np.stack([np.asarray(patchrx)[sel], np.asarray(patchry)[sel],
                                        np.asarray(patchrz)[sel]], 1), dtype=np.float64).reshape(-1)
    cells = pn.reshape(-1, 3).astype(np.int64).prod(axis=1) if k else np.zeros(0, dtype=np.int64)
    coff = np.zeros(k + 1, dtype=np.int64)
    np.cumsum(cells, out=coff[1:])
    flat = lambda fields, dt: (np.ascontiguousarray(np.concatenate([np.ravel(np.asarray(fields[p], dtype=dt))
                                                                    for p in sel]), dtype=dt)
                               if k else np.zeros(0, dtype=dt))
    delta, vx, vy, vz, temp = (flat(f, np.float64) for f in (gas_delta, gas_vx, gas_vy, gas_vz, gas_temp))
    leaf = lambda fields: np.ascontiguousarray(np.concatenate([np.ravel(np.asarray(fields[p]) != 0) for p in sel])
                                               .astype(np.uint8) if k else np.zeros(0, dtype=np.uint8))
    cr0, sol = leaf(gas_cr0amr), leaf(gas_solapst)
    cap = int(coff[-1])
    out = [np.empty(max(cap, 1), dtype=np.float64) for _ in range(8)]
    n_out = ctypes.c_int64(0)
    st = _lib.lib().halma_amr_to_particles(k, _lib.ptr(plev), _lib.ptr(pn), _lib.ptr(pr), _lib.ptr(coff),
                                           *[_lib.ptr(a) for a in (delta, vx, vy, vz, temp, cr0, sol)], float(L),
                                           int(ncoarse), _lib.ptr(box), float(rho_B), cap,
                                           *[_lib.ptr(a) for a in out], ctypes.byref(n_out), None)
    _lib.check(st, "halma_amr_to_particles")
    m = int(n_out.value)
    return tuple(a[:m].copy() for a in out)


def st_gas_dm_particles_inside(rete, L, ncoarse, grid_data, gas_data, masclet_dm_data, masclet_st_data,
                               st_kdtree, dm_kdtree, cx, cy, cz, R, rho_B):
    """halo_gas.py:223-277 with the particle side on the GPU.

    With ``grid_data`` given, the gas comes from ``AMRgrid_to_particles(L, ncoarse,
    grid_data, gas_data, R, cx, cy, cz, rho_B)`` as in the reference (halo_gas.py:231-233).
    With ``grid_data=None``, ``gas_data`` is taken as gas already turned into particles — the
    tuple (gas_x, gas_y, gas_z, gas_vx, gas_vy, gas_vz, gas_mass, gas_temp) that conversion
    returns.  The KD-trees are replaced by the GPU ball gather (``st_kdtree`` / ``dm_kdtree``
    are unused), so the DM and star selections come back in ascending index order instead of
    tree order.  Returns the reference's 17-tuple.
    """
    if grid_data is not None:
        gas_data = AMRgrid_to_particles(L, ncoarse, grid_data, gas_data, R, cx, cy, cz, rho_B)
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
