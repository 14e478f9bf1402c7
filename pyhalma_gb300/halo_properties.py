"""Per-halo FP64 reductions of python_scripts/halo_properties.py on the GPU.

Batched form (the one the pipeline uses): ``halo_reductions(offsets, x, y, z, vx, vy, vz, m,
mask=None, about=None)`` returns one row per CSR halo segment with the fields of
``halma_halo_reductions``: mass, centre of mass, bulk velocity, R_max, R_1/2, sigma_eff, n.
``about`` (n_haloes x 8: cx, cy, cz, vx, vy, vz, M, R05; NaN = computed) supplies the values
the reference functions take as arguments instead of computing them.

Drop-in single-halo functions with the reference signatures, each one launch of the same
kernel over the halo's members:

* ``total_mass(part_list, st_mass)``                                   :16-24
* ``center_of_mass(part_list, st_x, st_y, st_z, st_mass)``             :26-43
* ``CM_velocity(M, part_list, st_vx, st_vy, st_vz, st_mass)``          :45-60
* ``furthest_particle(cx, cy, cz, part_list, st_x, st_y, st_z)``       :98-111
* ``half_mass_radius(cx, cy, cz, M, part_list, st_x, st_y, st_z, st_mass)`` :365-392
* ``sigma_effective(part_list, R05, st_x, ..., vx, vy, vz)``           :607-625

* ``escape_velocity_unbinding_fortran(rete, L, ncoarse, grid_data, gas_data, masclet_dm_data,
  cx, cy, cz, vx, vy, vz, Rmax, part_list, st_x, ..., st_mass, factor_v, rho_B)`` :282-361,
  the single-pass stellar escape cut with the AMR gas conversion and the potential on the GPU;
  ``escape_velocity_unbinding_particles`` is the same cut with the gas and dark-matter
  particles supplied by the caller.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .halo_gas import bf_potential

RED = {k: i for i, k in enumerate(_lib.RED_FIELDS)}
N_ABOUT = 8
NAN = float("nan")


def halo_reductions(offsets, x, y, z, vx, vy, vz, m, mask=None, about=None):
    """FP64 reductions per CSR segment; returns an (n_haloes, 11) array (or device tensor)."""
    dev = _lib._is_torch(x)
    if dev:
        nh = int(offsets.shape[0]) - 1
        n = int(x.shape[0])
        out = _lib.like(x, (max(nh, 0), len(_lib.RED_FIELDS)), np.float64)
        arrs = (offsets, x, y, z, vx, vy, vz, m)
    else:
        offsets = _lib.as_host(offsets, np.int64)
        arrs = (offsets,) + tuple(_lib.as_host(a, np.float64) for a in (x, y, z, vx, vy, vz, m))
        nh = offsets.shape[0] - 1
        n = arrs[1].shape[0]
        out = np.zeros((max(nh, 0), len(_lib.RED_FIELDS)), dtype=np.float64)
        if mask is not None:
            mask = _lib.as_host(mask, np.uint8)
        if about is not None:
            about = _lib.as_host(about, np.float64).reshape(nh, N_ABOUT)
    if nh <= 0:
        return out
    _lib.check_arrays(np.int64, nh + 1, offsets=arrs[0])
    _lib.check_arrays(np.float64, n, **dict(zip(("x", "y", "z", "vx", "vy", "vz", "m"), arrs[1:])))
    _lib.check_arrays(np.uint8, n, mask=mask)
    if about is not None and (tuple(about.shape) != (nh, N_ABOUT) or str(about.dtype) not in ("float64", "torch.float64")
                              or (_lib._is_torch(about) and not about.is_contiguous())):
        raise ValueError(f"about must be a contiguous float64 ({nh}, {N_ABOUT}) array")
    st = _lib.lib().halma_halo_reductions(n, nh, *[_lib.ptr(a) for a in arrs], _lib.ptr(mask), _lib.ptr(about),
                                          _lib.ptr(out), _lib.stream_of(*arrs))
    _lib.check(st, "halma_halo_reductions")
    return out


def _one(part_list, st_x=None, st_y=None, st_z=None, st_vx=None, st_vy=None, st_vz=None, st_mass=None,
         about=None):
    pl = np.asarray(part_list, dtype=np.int64)

    def g(a, fill):
        if a is None:
            return np.full(len(pl), fill)
        return np.ascontiguousarray(np.asarray(a, dtype=np.float64)[pl])

    ab = None if about is None else np.array([about], dtype=np.float64)
    row = halo_reductions(np.array([0, len(pl)], dtype=np.int64), g(st_x, 0.0), g(st_y, 0.0), g(st_z, 0.0),
                          g(st_vx, 0.0), g(st_vy, 0.0), g(st_vz, 0.0), g(st_mass, 1.0), about=ab)
    return row[0]


def total_mass(part_list, st_mass):
    return float(_one(part_list, st_mass=st_mass)[RED["mass"]])


def center_of_mass(part_list, st_x, st_y, st_z, st_mass):
    r = _one(part_list, st_x, st_y, st_z, st_mass=st_mass)
    if r[RED["mass"]] > 0:
        return float(r[RED["cx"]]), float(r[RED["cy"]]), float(r[RED["cz"]]), float(r[RED["mass"]])
    return 0., 0., 0., 0.


def CM_velocity(M, part_list, st_vx, st_vy, st_vz, st_mass):
    if not M > 0.:
        return 0., 0., 0.
    r = _one(part_list, st_vx=st_vx, st_vy=st_vy, st_vz=st_vz, st_mass=st_mass)
    # the kernel divides by its own sum of masses; the reference divides by the caller's M
    s = r[RED["mass"]] / M
    return float(r[RED["vx"]] * s), float(r[RED["vy"]] * s), float(r[RED["vz"]] * s)


def furthest_particle(cx, cy, cz, part_list, st_x, st_y, st_z):
    if len(part_list) == 0:
        return 0.
    r = _one(part_list, st_x, st_y, st_z, about=[cx, cy, cz, NAN, NAN, NAN, NAN, NAN])
    return float(r[RED["rmax"]])


def half_mass_radius(cx, cy, cz, M, part_list, st_x, st_y, st_z, st_mass):
    r = _one(part_list, st_x, st_y, st_z, st_mass=st_mass, about=[cx, cy, cz, NAN, NAN, NAN, M, NAN])
    return float(r[RED["r05"]])


def sigma_effective(part_list, R05, st_x, st_y, st_z, st_vx, st_vy, st_vz, cx, cy, cz, vx, vy, vz):
    if len(part_list) == 0:
        return 0.
    r = _one(part_list, st_x, st_y, st_z, st_vx, st_vy, st_vz, about=[cx, cy, cz, vx, vy, vz, NAN, R05])
    return float(r[RED["sigma"]])


def escape_velocity_unbinding_fortran(rete, L, ncoarse, grid_data, gas_data, masclet_dm_data, cx, cy, cz, vx, vy, vz,
                                      Rmax, part_list, st_x, st_y, st_z, st_vx, st_vy, st_vz, st_mass, factor_v,
                                      rho_B):
    """halo_properties.py:282-361, same signature and result (bool per halo star, True =
    bound), with the AMR conversion and the potential on the GPU.

    Sources: the gas cells of the refined patches inside Rmax (``halo_gas.AMRgrid_to_particles``,
    masses times rete**3), the halo's stars, and the DM particles inside Rmax (masses times
    ``halo_gas.MASS_TO_SUN``, the reference's units.mass_to_sun), concatenated in that order
    (:333-336); the float32 potential of the f2py kernel (halma_bf_potential_f32, bit-identical
    to the Fortran loop in the default reference mode); E = 1/2 |v - v_bulk|^2 - G phi
    factor_v^2 with G = 4.3e-9; bound = E <= 0.  The host arithmetic around the kernel is the
    reference's, in its order and dtypes, so the result is the reference's bit for bit.  With
    ``grid_data=None``, ``gas_data`` is taken as gas particles (x, y, z, vx, vy, vz, mass, temp)
    already converted (comoving masses)."""
    from .halo_gas import AMRgrid_to_particles, MASS_TO_SUN, brute_force_binding_energy_fortran
    dm_x, dm_y, dm_z = (np.asarray(masclet_dm_data[k]) for k in range(3))
    dm_mass = np.asarray(masclet_dm_data[3]) * MASS_TO_SUN
    inside = np.sqrt((dm_x - cx) ** 2 + (dm_y - cy) ** 2 + (dm_z - cz) ** 2) < Rmax
    dm_x, dm_y, dm_z, dm_mass = dm_x[inside], dm_y[inside], dm_z[inside], dm_mass[inside]
    st_x_halo, st_y_halo, st_z_halo = st_x[part_list], st_y[part_list], st_z[part_list]
    st_vx_halo, st_vy_halo, st_vz_halo = st_vx[part_list], st_vy[part_list], st_vz[part_list]
    st_mass_halo = st_mass[part_list]
    if grid_data is not None:
        gas = AMRgrid_to_particles(L, ncoarse, grid_data, gas_data, Rmax, cx, cy, cz, rho_B)
    else:
        gas = tuple(np.asarray(a) for a in gas_data)
    gas_x, gas_y, gas_z, gas_mass = gas[0], gas[1], gas[2], gas[6]
    inside = np.sqrt((gas_x - cx) ** 2 + (gas_y - cy) ** 2 + (gas_z - cz) ** 2) < Rmax
    gas_x, gas_y, gas_z, gas_mass = gas_x[inside], gas_y[inside], gas_z[inside], gas_mass[inside]
    gas_mass *= rete ** 3
    total_x = np.concatenate((gas_x, st_x_halo, dm_x))
    total_y = np.concatenate((gas_y, st_y_halo, dm_y))
    total_z = np.concatenate((gas_z, st_z_halo, dm_z))
    total_mass = np.concatenate((gas_mass, st_mass_halo, dm_mass))
    binding_energy = brute_force_binding_energy_fortran(total_mass, total_x, total_y, total_z,
                                                        st_x_halo, st_y_halo, st_z_halo)
    binding_energy = -binding_energy
    G_const = 4.3 * 1e-3
    G_const *= 1e-6
    binding_energy *= G_const
    binding_energy *= factor_v ** 2
    st_v2 = 0.5 * ((st_vx_halo - vx) ** 2 + (st_vy_halo - vy) ** 2 + (st_vz_halo - vz) ** 2)
    total_energy = st_v2 + binding_energy
    return total_energy <= 0.


def escape_velocity_unbinding_particles(cx, cy, cz, vx, vy, vz, Rmax, part_list, st_x, st_y, st_z, st_vx, st_vy,
                                        st_vz, st_mass, factor_v, gas_x=(), gas_y=(), gas_z=(), gas_mass=(),
                                        dm_x=(), dm_y=(), dm_z=(), dm_mass=()):
    """Single-pass escape cut (halo_properties.py:320-361) on gas and DM given as particles:
    sources are the gas cells, the halo's stars and the DM particles inside Rmax
    (concatenated in that order, :333-336); E = 1/2 |v - v_bulk|^2 - G phi factor_v^2;
    returns ``E <= 0`` per halo star.  Unlike escape_velocity_unbinding_fortran, the masses
    are used as given: the caller applies the reference's two unit conversions, DM masses
    times units.mass_to_sun (:292) and gas masses times rete**3 (comoving to physical, :326).
    The selection of gas and DM inside Rmax is host bookkeeping; the potential runs on the GPU."""
    gx, gy, gz, gm = (np.asarray(a, dtype=np.float64) for a in (gas_x, gas_y, gas_z, gas_mass))
    dmx, dmy, dmz, dmm = (np.asarray(a, dtype=np.float64) for a in (dm_x, dm_y, dm_z, dm_mass))
    if dmx.size:
        inside = np.sqrt((dmx - cx) ** 2 + (dmy - cy) ** 2 + (dmz - cz) ** 2) < Rmax
        dmx, dmy, dmz, dmm = dmx[inside], dmy[inside], dmz[inside], dmm[inside]
    if gx.size:
        inside = np.sqrt((gx - cx) ** 2 + (gy - cy) ** 2 + (gz - cz) ** 2) < Rmax
        gx, gy, gz, gm = gx[inside], gy[inside], gz[inside], gm[inside]
    pl = np.asarray(part_list)
    sx, sy, sz = st_x[pl], st_y[pl], st_z[pl]
    if len(sx) == 0:
        return np.array([], dtype=bool)
    tx = np.concatenate((gx, sx, dmx))
    ty = np.concatenate((gy, sy, dmy))
    tz = np.concatenate((gz, sz, dmz))
    tm = np.concatenate((gm, st_mass[pl], dmm))
    e = -bf_potential(tm, tx, ty, tz, sx, sy, sz)
    G_const = 4.3 * 1e-3
    G_const *= 1e-6
    e *= G_const
    e *= factor_v ** 2
    ek = 0.5 * ((st_vx[pl] - vx) ** 2 + (st_vy[pl] - vy) ** 2 + (st_vz[pl] - vz) ** 2)
    return (ek + e) <= 0.


# ---------------------------------------------------------------------------------------
# the O(N) part of the main script's property loop (pyHALMA.py:930-1016)
# ---------------------------------------------------------------------------------------
PROP = {k: i for i, k in enumerate(_lib.PROP_FIELDS)}
# main-script array name -> field (pyHALMA.py:945-1013)
DRIVER_NAMES = {"rad05": "r05", "rad05_x": "r05x", "rad05_y": "r05y", "rad05_z": "r05z", "velocities_x": "vx",
                "velocities_y": "vy", "velocities_z": "vz", "specific_angular_momentum_x": "jx",
                "specific_angular_momentum_y": "jy", "specific_angular_momentum_z": "jz",
                "specific_angular_momentum": "j", "tully_fisher_velocities": "v_tf",
                "kinematic_morphologies": "k_co", "s_axis_major": "a", "s_axis_intermediate": "b",
                "s_axis_minor": "c", "sig_3D": "sig_3d", "sig_1D_x": "sig_1d_x", "sig_1D_y": "sig_1d_y",
                "sig_1D_z": "sig_1d_z", "vsigma": "v_sigma", "lambda_ensellem": "lambda"}


def halo_property_table(offsets, members, st_x, st_y, st_z, st_vx, st_vy, st_vz, st_mass, centre, LL):
    """C ABI ``halma_halo_properties``: groups as CSR over particle indices, centre rows
    (cx, cy, cz, mass, rmax); returns an (n_groups, len(PROP_FIELDS)) float64 table."""
    offsets = _lib.as_host(offsets, np.int64)
    members = _lib.as_host(members, np.int32)
    arrs = tuple(_lib.as_host(a, np.float64) for a in (st_x, st_y, st_z, st_vx, st_vy, st_vz, st_mass))
    centre = _lib.as_host(centre, np.float64).reshape(-1, 5)
    G = offsets.shape[0] - 1
    if centre.shape[0] != G:
        raise ValueError("one centre row (cx, cy, cz, mass, rmax) per group")
    _lib.check_arrays(np.float64, arrs[0].shape[0], **dict(zip(("st_x", "st_y", "st_z", "st_vx", "st_vy", "st_vz",
                                                               "st_mass"), arrs)))
    if G > 0 and not 0 <= offsets[-1] <= members.shape[0]:
        raise ValueError(f"the offsets cover {offsets[-1]} members, {members.shape[0]} given")
    out = np.zeros((max(G, 1), len(_lib.PROP_FIELDS)), dtype=np.float64)
    if G > 0:
        st = _lib.lib().halma_halo_properties(arrs[0].shape[0], *[_lib.ptr(a) for a in arrs], G, _lib.ptr(offsets),
                                              _lib.ptr(members), _lib.ptr(centre), float(LL), _lib.ptr(out), None)
        _lib.check(st, "halma_halo_properties")
    return out[:G]


def property_loop(new_groups, st_x, st_y, st_z, st_vx, st_vy, st_vz, st_mass, center_x, center_y, center_z, masses,
                  rmax, LL):
    """The O(N) properties the main script's loop computes per halo (pyHALMA.py:930-1016), for all
    haloes at once.  Inputs as the phase-space cleaning leaves them; returns a dict keyed by the
    main script's array names (rad05, rad05_x, ..., sig_3D, sig_1D_x, vsigma, lambda_ensellem)."""
    lens = np.fromiter((len(g) for g in new_groups), dtype=np.int64, count=len(new_groups))
    offsets = np.zeros(len(new_groups) + 1, dtype=np.int64)
    np.cumsum(lens, out=offsets[1:])
    members = np.concatenate([np.asarray(g, dtype=np.int64) for g in new_groups]) if offsets[-1] > 0 \
        else np.zeros(0, dtype=np.int64)
    if members.size and (members.min() < 0 or members.max() >= len(st_x)):
        raise ValueError("group members must be indices into the particle arrays")
    centre = np.stack([np.asarray(a, dtype=np.float64) for a in (center_x, center_y, center_z, masses, rmax)], 1) \
        if len(new_groups) else np.zeros((0, 5))
    t = halo_property_table(offsets, members, st_x, st_y, st_z, st_vx, st_vy, st_vz, st_mass, centre, LL)
    return {name: t[:, PROP[f]].copy() for name, f in DRIVER_NAMES.items()}
