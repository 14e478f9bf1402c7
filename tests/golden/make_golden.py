"""Generate golden fixtures by running pyHALMA's own Python code in this container.

Run from the repository root:
    python tests/golden/make_golden.py --reference DIR      (or PYHALMA_REFERENCE=DIR)

DIR is a checkout of pyHALMA; it is read in place and never modified.  Modules
that are absent here are replaced by stubs in ``sys.modules`` before the import:

* ``numba``: ``njit`` returns the function unchanged, ``prange`` is ``range`` and
  ``get_num_threads`` returns 1, so the numba kernels run as plain Python;
* ``masclet_framework``, ``matplotlib``: empty namespaces except ``units.mass_to_sun`` (1.0:
  masses are generated in Msun) and two third-party helpers of ``tools`` that the AMR
  conversion calls (halo_gas.py:90-91), restated: ``create_vector_levels`` (patch 0 is the
  base grid, then npatch[1] patches of level 1, ...) and ``which_patches_inside_box`` (the
  base grid plus every patch whose extent [r - res, r - res + n*res] per axis overlaps the
  box; the conversion re-tests every cell, so any superset gives the same particles);
* ``fortran_modules.particle``: ``particle.brute_force_binding_energy`` maps onto the
  oracle's float32 restatement of particle_subroutines.f90:466-514 (gfortran is absent).

Fixtures written to tests/golden/ (all seeds fixed):

* fof_cases.npz   — reference ``fof.friends_of_friends_serial`` on small synthetic and
  adversarial inputs (positions stored exactly; canonical labels = min index, -1 alone);
* fof_config1.npz — the same on the 1e5-particle Plummer snapshot (positions stored; the
  SHA-256 of the positions regenerated from the seed here is stored as well);
* predicate.npz   — adversarial two-point pairs at nextafter distances and whether the
  reference's KDTree links them (pins the pair predicate);
* halo_props.npz  — reference reductions (halo_properties.py) on a few haloes;
* rps.npz         — reference ``halo_gas.RPS`` / ``most_bound_particle`` outputs with
  ``np.random.seed`` fixed before each call (pins the sub-sampling and energy logic);
* substructure.npz — the main script's inline substructure block (pyHALMA.py:703-766) exec'd
  from the reference's own source on bridged snapshots (input and output groups stored);
* ball.npz        — reference ``halo_gas.st_gas_dm_particles_inside`` with its MASCLET AMR
  conversion replaced by a pass-through of gas particles (inputs and the 17 outputs stored);
* psc.npz         — the main script's phase-space cleaning block (pyHALMA.py:774-877) exec'd from
  the reference's own source on FoF groups of contaminated Plummer snapshots;
* amr.npz         — reference ``halo_gas.AMRgrid_to_particles`` (with its numba kernel
  patch_to_particles) on synthetic refined patches, several boxes;
* escape.npz      — reference ``halo_properties.escape_velocity_unbinding_fortran`` with the
  same AMR grids, DM particles and a stellar halo (two factor_v, two Rmax);
* properties.npz  — the reference's O(N) per-halo property functions (half-mass radii, bulk
  velocity, angular momentum, Tully-Fisher velocity, kappa_co, shape, sigma_effective,
  sigma projections) called as the main script's property loop calls them; the f2py routines
  halo_shape / sigma_projections map onto the C restatement of the Fortran.
"""
from __future__ import annotations

import argparse
import hashlib
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from pyhalma_gb300 import synth  # noqa: E402


def install_stubs():
    nb = types.ModuleType("numba")

    def njit(*a, **k):
        if a and callable(a[0]) and not k:
            return a[0]
        return lambda f: f

    nb.njit = njit
    nb.jit = njit
    nb.prange = range
    nb.get_num_threads = lambda: 1
    nb.set_num_threads = lambda n: None
    sys.modules["numba"] = nb

    mf = types.ModuleType("masclet_framework")
    for sub in ("units", "tools", "particles", "particle2grid", "read_masclet", "read_asohf",
                "cosmo_tools"):
        m = types.ModuleType("masclet_framework." + sub)
        setattr(mf, sub, m)
        sys.modules["masclet_framework." + sub] = m
    mf.units.mass_to_sun = 1.0

    def create_vector_levels(npatch):
        out = [0]
        for lev, cnt in enumerate(list(npatch)[1:], start=1):
            out += [lev] * int(cnt)
        return np.array(out)

    def which_patches_inside_box(box, patchnx, patchny, patchnz, patchrx, patchry, patchrz, npatch, size, nmax):
        levels = create_vector_levels(npatch)
        keep = [0]
        for p in range(1, len(patchnx)):
            res = size / nmax / 2 ** levels[p]
            lo = [patchrx[p] - res, patchry[p] - res, patchrz[p] - res]
            hi = [lo[0] + patchnx[p] * res, lo[1] + patchny[p] * res, lo[2] + patchnz[p] * res]
            if all(box[2 * q] < hi[q] and box[2 * q + 1] > lo[q] for q in range(3)):
                keep.append(p)
        return keep

    mf.tools.create_vector_levels = create_vector_levels
    mf.tools.which_patches_inside_box = which_patches_inside_box
    sys.modules["masclet_framework"] = mf

    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    mpl.pyplot = plt
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = plt

    fm = types.ModuleType("fortran_modules")
    part = types.ModuleType("fortran_modules.particle")

    class _P:
        @staticmethod
        def brute_force_binding_energy(ncores, ntotal, m, x, y, z, ntest, tx, ty, tz):
            assert m.dtype == np.float32 and tx.dtype == np.float32
            assert int(ntotal) == len(m) and int(ntest) == len(tx)
            return oracle.bf_potential_f32(m, x, y, z, tx, ty, tz, ncores=max(int(ncores), 1))

        serial_brute_force_binding_energy = None

        @staticmethod
        def halo_shape(ncore, npart, x, y, z, mass):
            from oracle import properties as op
            assert x.dtype == np.float32 and int(npart) == len(x)
            out = np.zeros(3, dtype=np.float32)
            op.lib().oracle_halo_shape(int(npart), op._p(x), op._p(y), op._p(z), op._p(mass), op._p(out))
            return out

        @staticmethod
        def sigma_projections(ncore, npart, grid, n_cell, part_list, st_x, st_y, st_z, st_vx, st_vy, st_vz,
                              st_mass, cx, cy, cz, R05x, R05y, R05z, ll):
            from oracle import properties as op
            assert grid.dtype == np.float32 and st_vx.dtype == np.float32
            pl = np.ascontiguousarray(part_list.astype(np.int64) - 1)          # Fortran indices start at 1
            out = np.zeros(5, dtype=np.float32)
            arrs = [np.ascontiguousarray(a) for a in (st_x, st_y, st_z, st_vx, st_vy, st_vz, st_mass)]
            op.lib().oracle_sigma_projections(int(npart), op._p(grid), int(n_cell), op._p(pl),
                                              *[op._p(a) for a in arrs],
                                              *[float(v) for v in (cx, cy, cz, R05x, R05y, R05z, ll)], op._p(out))
            return tuple(out)

    part.particle = _P
    fm.particle = part
    sys.modules["fortran_modules"] = fm
    sys.modules["fortran_modules.particle"] = part


def import_reference(refdir):
    install_stubs()
    sys.path.insert(0, refdir)
    from python_scripts import fof, halo_gas, halo_properties  # noqa
    return fof, halo_gas, halo_properties


def sha(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def fof_cases(fof):
    cases = {}
    rng = np.random.default_rng(11)
    # 1) small clustered snapshot
    s = synth.plummer_snapshot(4000, 8, seed=3, box_mpc=0.5)
    cases["plummer4k"] = (np.stack([s.x, s.y, s.z], 1), 0.0015)
    # 2) lattice with spacing exactly the linking length (ties at d == r), jittered by ulps
    cases["lattice_tie"] = (synth.lattice_points(9, 0.0015, origin=(0.3, -0.2, 0.1)), 0.0015)
    cases["lattice_jitter"] = (synth.lattice_points(9, 0.0015, origin=(1.7, 2.3, -4.1),
                                                    jitter_ulps=2, seed=5), 0.0015)
    # 3) duplicates, chains and isolated points
    base = rng.uniform(0, 0.05, (600, 3))
    dup = np.concatenate([base, base[:100], base[50:60]])
    cases["duplicates"] = (dup, 0.002)
    chain = np.zeros((400, 3))
    chain[:, 0] = np.arange(400) * 0.0015
    chain[:, 1] = 0.25
    cases["chain"] = (chain, 0.0015)
    cases["sparse"] = (rng.uniform(-1, 1, (500, 3)), 0.01)
    cases["single"] = (np.array([[0.1, 0.2, 0.3]]), 0.0015)
    cases["pair_at_r"] = (np.array([[0.0, 0.0, 0.0], [0.0015, 0.0, 0.0]]), 0.0015)
    big = rng.normal(0, 0.004, (3000, 3))
    cases["blob"] = (big, 0.0004)
    out = {}
    for name, (data, ll) in cases.items():
        groups = fof.friends_of_friends_serial(data[:, 0], data[:, 1], data[:, 2], ll)
        lab = oracle.groups_to_labels(groups, data.shape[0])
        out[f"{name}__xyz"] = data
        out[f"{name}__ll"] = np.float64(ll)
        out[f"{name}__labels"] = lab
        out[f"{name}__ngroups"] = np.int64(len(groups))
        print(f"  fof {name}: n={data.shape[0]} groups={len(groups)}")
    np.savez_compressed(os.path.join(HERE, "fof_cases.npz"), **out)


def fof_config1(fof):
    s = synth.plummer_snapshot(100_000, 50, seed=0, box_mpc=10.0)
    groups = fof.friends_of_friends_serial(s.x, s.y, s.z, 0.0015)
    lab = oracle.groups_to_labels(groups, s.n)
    # positions are stored too: NumPy's transcendental kernels differ across platforms, so
    # another machine may regenerate a slightly different snapshot from the same seed
    np.savez_compressed(os.path.join(HERE, "fof_config1.npz"), labels=lab, x=s.x, y=s.y, z=s.z,
                        sha256=np.array(sha(s.x, s.y, s.z)), ll=np.float64(0.0015),
                        n=np.int64(s.n), seed=np.int64(0), n_spheres=np.int64(50),
                        box_mpc=np.float64(10.0), ngroups=np.int64(len(groups)))
    print(f"  fof config1: n={s.n} groups={len(groups)}")


def predicate_pairs(fof):
    from scipy.spatial import KDTree
    rng = np.random.default_rng(7)
    a_all, b_all, r_all, hit_all = [], [], [], []
    for r in (0.0015, 1.5, 0.7):
        found, tries = 0, 0
        while found < 400 and tries < 200_000:
            tries += 1
            a = rng.uniform(-4 * r, 4 * r, 3)
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            b = a + d * r
            for k in range(3):
                for _ in range(rng.integers(0, 3)):
                    b[k] = np.nextafter(b[k], np.inf if rng.random() < 0.5 else -np.inf)
            dx, dy, dz = a - b
            seq = (dx * dx + dy * dy) + dz * dz <= r * r
            alt = np.sqrt(dx * dx + dy * dy + dz * dz) <= r
            alt2 = dx * dx + (dy * dy + dz * dz) <= r * r
            if seq == alt and seq == alt2:
                continue  # keep only pairs where plausible predicates disagree
            hit = 1 in KDTree(np.array([a, b])).query_ball_point(a, r)
            found += 1
            a_all.append(a); b_all.append(b); r_all.append(r); hit_all.append(hit)
    np.savez_compressed(os.path.join(HERE, "predicate.npz"), a=np.array(a_all),
                        b=np.array(b_all), r=np.array(r_all), hit=np.array(hit_all))
    print(f"  predicate pairs: {len(r_all)}")


def halo_props(hp):
    s = synth.plummer_snapshot(20_000, 6, seed=4, box_mpc=1.0)
    out = {"x": s.x, "y": s.y, "z": s.z, "vx": s.vx, "vy": s.vy, "vz": s.vz, "m": s.mass}
    res = []
    for h in range(6):
        pl = np.nonzero(s.sphere == h)[0].astype(np.int64)
        cx, cy, cz, M = hp.center_of_mass(pl, s.x, s.y, s.z, s.mass)
        tm = hp.total_mass(pl, s.mass)
        vx, vy, vz = hp.CM_velocity(M, pl, s.vx, s.vy, s.vz, s.mass)
        rmax = hp.furthest_particle(cx, cy, cz, pl, s.x, s.y, s.z)
        r05 = hp.half_mass_radius(cx, cy, cz, M, pl, s.x, s.y, s.z, s.mass)
        sig = hp.sigma_effective(pl, r05, s.x, s.y, s.z, s.vx, s.vy, s.vz, cx, cy, cz, vx, vy, vz)
        res.append([tm, cx, cy, cz, M, vx, vy, vz, rmax, r05, sig])
        out[f"pl{h}"] = pl
    out["results"] = np.array(res)
    np.savez_compressed(os.path.join(HERE, "halo_props.npz"), **out)
    print("  halo properties: 6 haloes")


def rps_cases(hg):
    out = {}
    n = 0
    for k, (ngas, ndm, nst, lim) in enumerate([(800, 300, 400, 5000), (7000, 6000, 5500, 5000),
                                               (1200, 9000, 300, 1000)]):
        g = synth.nfw_gas_halo(ngas, nst, seed=20 + k, r_vir_kpc=60.0)
        rng = np.random.default_rng(40 + k)
        dm = rng.normal(0, 0.02, (ndm, 3))
        mass_dm_part = 1e7
        dm_m = np.where(rng.random(ndm) < 0.3, mass_dm_part / 8, mass_dm_part / 64)
        vb = g.bulk
        gas = [g.gas_x.astype(np.float64), g.gas_y.astype(np.float64), g.gas_z.astype(np.float64),
               g.gas_vx, g.gas_vy, g.gas_vz, g.gas_mass, g.gas_temp]
        oripa = np.arange(nst) + 1000 * k
        for nspec in (1, 2):
            np.random.seed(1234 + k)
            r = hg.RPS(*gas, dm[:, 0], dm[:, 1], dm[:, 2], dm_m, g.st_x, g.st_y, g.st_z,
                       g.st_mass, vb[0], vb[1], vb[2], lim, mass_dm_part, nspec)
            out[f"c{k}_rps{nspec}"] = np.array(r, dtype=np.float64)
        np.random.seed(999 + k)
        mb = hg.most_bound_particle(gas[0], gas[1], gas[2], gas[6], dm[:, 0], dm[:, 1], dm[:, 2],
                                    dm_m, g.st_x, g.st_y, g.st_z, g.st_mass, oripa, lim,
                                    mass_dm_part)
        out[f"c{k}_mb"] = np.array(mb, dtype=np.float64)
        for name, arr in (("gx", gas[0]), ("gy", gas[1]), ("gz", gas[2]), ("gvx", gas[3]),
                          ("gvy", gas[4]), ("gvz", gas[5]), ("gm", gas[6]), ("gt", gas[7]),
                          ("dx", dm[:, 0]), ("dy", dm[:, 1]), ("dz", dm[:, 2]), ("dm", dm_m),
                          ("sx", g.st_x), ("sy", g.st_y), ("sz", g.st_z), ("sm", g.st_mass),
                          ("oripa", oripa), ("bulk", vb)):
            out[f"c{k}_{name}"] = arr
        out[f"c{k}_params"] = np.array([lim, mass_dm_part], dtype=np.float64)
        n += 1
    np.savez_compressed(os.path.join(HERE, "rps.npz"), ncase=np.int64(n), **out)
    print(f"  rps/most-bound: {n} cases")


def _reference_block(refdir, start_marker, end_marker, extra_lines=1):
    """Source of an inline block of pyHALMA.py (from the line holding start_marker to the line
    holding end_marker, plus extra_lines), dedented so that it can be exec'd on its own."""
    import textwrap
    src = open(os.path.join(refdir, "pyHALMA.py")).read().split("\n")
    i0 = next(i for i, line in enumerate(src) if start_marker in line)
    i1 = next(i for i in range(i0, len(src)) if end_marker in src[i])
    return textwrap.dedent("\n".join(src[i0:i1 + 1 + extra_lines])), i0 + 1, i1 + 1 + extra_lines


def substructure_cases(fof, hp, refdir):
    """The main script's substructure block (pyHALMA.py:703-766) run as written: its source is
    exec'd with the reference's fof / halo_properties modules, the main script's good_groups and
    the FoF groups of a bridged snapshot (after good_groups(MINP), as at pyHALMA.py:592)."""
    block, b0, b1 = _reference_block(refdir, "if SUBSTRUCTURE_FLAG:", "Substructures / Cut FoF bridges")
    gg, _, _ = _reference_block(refdir, "def good_groups(groups, minp):", "def good_groups(groups, minp):")
    out = {"block_lines": np.array([b0, b1], dtype=np.int64)}
    cases = [("one_level", 1, 0.0015, 25, 2.0, 0.0005, 0.75, 50),
             ("three_levels", 2, 0.0015, 25, 2.0, 0.0001, 0.75, 50),
             ("dec1p5", 3, 0.0015, 10, 1.5, 0.0004, 0.5, 30)]
    for name, seed, LL, MINP_SUB, DEC_FACTOR, MIN_LL, DIST_FACTOR, MINP in cases:
        s = synth.bridged_snapshot(8, 4, seed=seed, box_mpc=1.0, n_hi=2500)
        groups = fof.friends_of_friends_serial(s.x, s.y, s.z, LL)
        ns = {"np": np, "fof": fof, "halo_properties": hp, "tqdm": lambda it: it, "print": lambda *a, **k: None}
        exec(gg, ns)
        groups = np.array(groups, dtype=object)
        groups = groups[ns["good_groups"](groups, MINP)]
        groups_in = [list(g) for g in groups]
        ns.update(dict(SUBSTRUCTURE_FLAG=True, PYFOF_FLAG=False, groups=groups, st_x=s.x, st_y=s.y, st_z=s.z,
                       st_mass=s.mass, LL=LL, MINP_SUB=MINP_SUB, DEC_FACTOR=DEC_FACTOR, MIN_LL=MIN_LL,
                       DIST_FACTOR=DIST_FACTOR, MINP=MINP))
        exec(block, ns)
        res = [list(map(int, g)) for g in ns["groups"]]
        lens_in = np.array([len(g) for g in groups_in], dtype=np.int64)
        lens_out = np.array([len(g) for g in res], dtype=np.int64)
        out[f"{name}__x"], out[f"{name}__y"], out[f"{name}__z"], out[f"{name}__m"] = s.x, s.y, s.z, s.mass
        out[f"{name}__params"] = np.array([LL, MINP_SUB, DEC_FACTOR, MIN_LL, DIST_FACTOR, MINP], dtype=np.float64)
        out[f"{name}__in_off"] = np.concatenate(([0], np.cumsum(lens_in)))
        out[f"{name}__in_mem"] = np.concatenate([np.asarray(g, dtype=np.int64) for g in groups_in])
        out[f"{name}__out_off"] = np.concatenate(([0], np.cumsum(lens_out)))
        out[f"{name}__out_mem"] = np.concatenate([np.asarray(g, dtype=np.int64) for g in res]) if res \
            else np.zeros(0, dtype=np.int64)
        out[f"{name}__counter_sub"] = np.int64(ns["counter_sub"])
        print(f"  substructure {name}: n={s.n} groups in={len(groups_in)} out={len(res)} "
              f"cut={ns['counter_sub']}")
    np.savez_compressed(os.path.join(HERE, "substructure.npz"), **out)


def ball_cases(hg):
    """The reference's st_gas_dm_particles_inside (halo_gas.py:223-277) run as written, with its
    AMR-grid conversion (halo_gas.py:56-141, needs MASCLET grids) replaced by a pass-through of
    gas particles; the KD-trees are built as the main script builds them (pyHALMA.py:543-545)."""
    from scipy.spatial import KDTree
    out = {}
    orig = hg.AMRgrid_to_particles
    try:
        for k, (ngas, ndm, nst) in enumerate([(3000, 8000, 6000), (1500, 4000, 10000)]):
            rng = np.random.default_rng(60 + k)
            c = rng.uniform(-1, 1, 3)
            gas = [c[q] + rng.normal(0, 0.01, ngas) for q in range(3)] + \
                  [rng.normal(0, 100, ngas) for _ in range(3)] + [rng.lognormal(11, 1, ngas), rng.uniform(1e3, 1e6, ngas)]
            dm = [c[q] + rng.normal(0, 0.02, ndm) for q in range(3)] + [rng.uniform(1e6, 1e7, ndm)]
            st = [c[q] + rng.normal(0, 0.008, nst) for q in range(3)]
            st_data = st + [np.zeros(nst) for _ in range(3)] + [rng.uniform(1e5, 1e6, nst),
                                                                        np.zeros(nst), np.zeros(nst),
                                                                        np.arange(nst) + 10_000 * k]
            st_tree = KDTree(np.array((st[0], st[1], st[2])).T)
            dm_tree = KDTree(np.array((dm[0], dm[1], dm[2])).T)
            hg.AMRgrid_to_particles = lambda L, ncoarse, grid_data, gas_data, R, cx, cy, cz, rho_B: \
                tuple(np.copy(a) for a in gas_data)
            for j, R in enumerate((0.004, 0.015)):
                res = hg.st_gas_dm_particles_inside(0.5, 40.0, 128, None, gas, dm, st_data, st_tree, dm_tree,
                                                    c[0], c[1], c[2], R, 1.0)
                for q, a in enumerate(res):
                    out[f"c{k}r{j}_out{q}"] = np.asarray(a)
                out[f"c{k}r{j}_R"] = np.float64(R)
            for q, a in enumerate(gas):
                out[f"c{k}_gas{q}"] = a
            for q, a in enumerate(dm):
                out[f"c{k}_dm{q}"] = a
            for q, a in enumerate(st_data):
                out[f"c{k}_st{q}"] = a
            out[f"c{k}_centre"] = c
            print(f"  ball gather case {k}: gas={ngas} dm={ndm} stars={nst}")
    finally:
        hg.AMRgrid_to_particles = orig
    np.savez_compressed(os.path.join(HERE, "ball.npz"), ncase=np.int64(2), rete=np.float64(0.5), **out)


def _store_grid(out, key, g):
    """A synthetic AMR grid as flat arrays: patch table and every field's cells concatenated
    patch by patch, each patch x-major (tests/test_amr_escape.py rebuilds the lists)."""
    gd = g.grid_data
    out[key + "_npatch"] = np.asarray(gd[5])
    out[key + "_patchn"] = np.stack([gd[6], gd[7], gd[8]], 1)
    out[key + "_patchr"] = np.stack([gd[12], gd[13], gd[14]], 1)
    for j, f in enumerate(g.gas_data):   # float32 values (exact) and flags
        flat = np.concatenate([np.ravel(a) for a in f])
        out[key + f"_f{j}"] = flat.astype(np.float32) if j < 5 else flat.astype(bool)
    out[key + "_scalars"] = np.array([g.L, g.ncoarse, g.rho_B], dtype=np.float64)
    out[key + "_centre"] = g.centre


def amr_cases(hg):
    """The reference's AMRgrid_to_particles on two synthetic grids, three boxes each."""
    out = {}
    for k in range(2):
        g = synth.amr_grid(seed=70 + k, centre_mpc=(1.3 + k, -0.7, 2.2 - k))
        _store_grid(out, f"g{k}", g)
        for j, (R, shift) in enumerate(((0.01, 0.0), (0.03, 0.004), (0.2, -0.01))):
            c = g.centre + shift
            res = hg.AMRgrid_to_particles(g.L, g.ncoarse, g.grid_data, g.gas_data, R, c[0], c[1], c[2], g.rho_B)
            for q, a in enumerate(res):
                out[f"g{k}b{j}_out{q}"] = np.asarray(a, dtype=np.float64)
            out[f"g{k}b{j}_box"] = np.array([R, *c], dtype=np.float64)
            print(f"  AMR grid {k} box {j}: {len(res[0])} gas particles")
    np.savez_compressed(os.path.join(HERE, "amr.npz"), ngrid=np.int64(2), nbox=np.int64(3), **out)


def escape_cases(hp):
    """The reference's escape_velocity_unbinding_fortran (halo_properties.py:282-361): gas from
    the AMR grids of amr.npz, DM particles, and a Plummer stellar halo with a hot tail, two
    factor_v and two Rmax per grid."""
    out = {}
    for k in range(2):
        g = synth.amr_grid(seed=70 + k, centre_mpc=(1.3 + k, -0.7, 2.2 - k))
        rng = np.random.default_rng(90 + k)
        c = g.centre
        nst, ndm, nfield = 3000 + 1000 * k, 8000, 1500
        a = 0.004
        u = rng.uniform(1e-6, 0.999, nst)
        r = a / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
        d = rng.normal(size=(nst, 3))
        d /= np.linalg.norm(d, axis=1)[:, None]
        st = c + r[:, None] * d
        bulk = rng.normal(0, 150, 3)
        sig = np.where(rng.random(nst) < 0.2, 400.0, 60.0)
        stv = bulk + rng.normal(size=(nst, 3)) * sig[:, None]
        field = c + rng.uniform(-0.2, 0.2, (nfield, 3))
        fv = rng.normal(0, 200, (nfield, 3))
        allp = np.concatenate([field, st])
        allv = np.concatenate([fv, stv])
        st_x, st_y, st_z = (np.ascontiguousarray(allp[:, q]) for q in range(3))
        st_vx, st_vy, st_vz = (np.ascontiguousarray(allv[:, q]) for q in range(3))
        st_mass = rng.uniform(5e5, 2e6, nfield + nst)
        part_list = np.arange(nfield, nfield + nst)
        dm = c + rng.normal(0, 0.015, (ndm, 3))
        dm_data = [np.ascontiguousarray(dm[:, q]) for q in range(3)] + [rng.uniform(5e6, 2e7, ndm)]
        for q, arr in enumerate(dm_data):
            out[f"g{k}_dm{q}"] = arr
        for name, arr in (("st_x", st_x), ("st_y", st_y), ("st_z", st_z), ("st_vx", st_vx), ("st_vy", st_vy),
                          ("st_vz", st_vz), ("st_mass", st_mass), ("part_list", part_list)):
            out[f"g{k}_{name}"] = arr
        for j, (Rmax, fv_) in enumerate(((0.02, 1.0), (0.05, 1.3))):
            bound = hp.escape_velocity_unbinding_fortran(0.5, g.L, g.ncoarse, g.grid_data, g.gas_data, dm_data,
                                                         c[0], c[1], c[2], bulk[0], bulk[1], bulk[2], Rmax,
                                                         part_list, st_x, st_y, st_z, st_vx, st_vy, st_vz,
                                                         st_mass, fv_, g.rho_B)
            out[f"g{k}e{j}_bound"] = np.asarray(bound)
            out[f"g{k}e{j}_params"] = np.array([0.5, Rmax, fv_, *bulk], dtype=np.float64)
            print(f"  escape grid {k} case {j}: {int(np.sum(bound))} of {len(bound)} bound")
    np.savez_compressed(os.path.join(HERE, "escape.npz"), ngrid=np.int64(2), ncase=np.int64(2), **out)


def psc_cases(fof, hp, refdir):
    """The main script's phase-space cleaning block (pyHALMA.py:774-877: calc_cell / clean_cell per
    group, the reset for small groups, the MINP cut and the sort by size) run as written on the
    FoF groups of contaminated Plummer snapshots."""
    block, b0, b1 = _reference_block(refdir, "print('---> Phase-space cleaning begins <---')",
                                     "which_cell_list_z = which_cell_list_z[sort_indices]", 0)
    gg, _, _ = _reference_block(refdir, "def good_groups(groups, minp):", "def good_groups(groups, minp):")
    out = {"block_lines": np.array([b0, b1], dtype=np.int64)}
    cases = [("psc_on", 31, 0.0015, 1.0, 3.0, True, 50), ("psc_q2", 32, 0.0015, 2.0, 2.0, True, 40),
             ("psc_aggr", 34, 0.0015, 3.0, 1.0, True, 30), ("psc_off", 33, 0.0015, 1.0, 3.0, False, 50)]
    for name, seed, LL, Q_FIL, SIG_FIL, PSC_FLAG, MINP in cases:
        s = synth.plummer_snapshot(12_000, 8, seed=seed, box_mpc=0.5, contaminant_frac=0.15, m_hi=3e10)
        groups = fof.friends_of_friends_serial(s.x, s.y, s.z, LL)
        ns = {"np": np, "halo_properties": hp, "tqdm": lambda it: it, "print": lambda *a, **k: None}
        exec(gg, ns)
        groups = np.array(groups, dtype=object)
        groups = groups[ns["good_groups"](groups, MINP)]
        groups_in = [list(g) for g in groups]
        ns.update(dict(groups=groups, st_x=s.x, st_y=s.y, st_z=s.z, st_vx=s.vx, st_vy=s.vy, st_vz=s.vz,
                       st_mass=s.mass, LL=LL, Q_FIL=Q_FIL, SIG_FIL=SIG_FIL, PSC_FLAG=PSC_FLAG, MINP=MINP))
        exec(block, ns)
        for k in ("x", "y", "z", "vx", "vy", "vz"):
            out[f"{name}__{k}"] = getattr(s, k)
        out[f"{name}__m"] = s.mass
        out[f"{name}__params"] = np.array([LL, Q_FIL, SIG_FIL, float(PSC_FLAG), MINP], dtype=np.float64)
        lens = [len(g) for g in groups_in]
        out[f"{name}__in_off"] = np.concatenate(([0], np.cumsum(lens))).astype(np.int64)
        out[f"{name}__in_mem"] = np.concatenate([np.asarray(g, dtype=np.int64) for g in groups_in])
        ng = ns["new_groups"]
        out[f"{name}__out_off"] = np.concatenate(([0], np.cumsum([len(g) for g in ng]))).astype(np.int64)
        out[f"{name}__out_mem"] = np.concatenate([np.asarray(g, dtype=np.int64) for g in ng])
        for k in ("center_x", "center_y", "center_z", "masses", "rmax", "num_particles", "num_cells"):
            out[f"{name}__{k}"] = np.asarray(ns[k])
        for a in "xyz":
            wl = ns[f"which_cell_list_{a}"]
            out[f"{name}__which_{a}_off"] = np.concatenate(([0], np.cumsum([len(w) for w in wl]))).astype(np.int64)
            out[f"{name}__which_{a}"] = np.concatenate([np.asarray(w, dtype=np.int64) for w in wl])
        print(f"  phase-space cleaning {name}: n={s.n} groups in={len(groups_in)} out={len(ng)} "
              f"particles {sum(lens)} -> {int(np.sum(ns['num_particles']))}")
    np.savez_compressed(os.path.join(HERE, "psc.npz"), **out)


def property_cases(hp):
    """The O(N) per-halo properties of the main script's property loop (pyHALMA.py:930-1016), called
    as the main script calls them, on the groups and centres that phase-space cleaning leaves for a
    contaminated Plummer snapshot.  The Fortran routines (halo_shape, sigma_projections) run
    through the reference's Python wrappers on the C restatement of the Fortran."""
    from oracle import phase_space as ops
    s = synth.plummer_snapshot(16_000, 10, seed=51, box_mpc=0.6, contaminant_frac=0.1, m_hi=3e10)
    groups = [g for g in oracle.labels_to_groups(oracle.fof_labels(s.x, s.y, s.z, 0.0015)) if len(g) >= 50]
    LL = 0.0015
    cl = ops.phase_space_cleaning(groups, s.x, s.y, s.z, s.vx, s.vy, s.vz, s.mass, LL, 1.0, 3.0, True, 50)
    rows = []
    for h, pl in enumerate(cl["new_groups"]):
        pl = np.asarray(pl, dtype=np.int64)
        cx, cy, cz, mass, rmax = (cl[k][h] for k in ("center_x", "center_y", "center_z", "masses", "rmax"))
        rad05 = hp.half_mass_radius(cx, cy, cz, mass, pl, s.x, s.y, s.z, s.mass)
        r05x, r05y, r05z = hp.half_mass_radius_proj(cx, cy, cz, mass, pl, s.x, s.y, s.z, s.mass)
        vx, vy, vz = hp.CM_velocity(mass, pl, s.vx, s.vy, s.vz, s.mass)
        jx, jy, jz = hp.angular_momentum(mass, pl, s.x, s.y, s.z, s.vx, s.vy, s.vz, s.mass, cx, cy, cz, vx, vy, vz)
        j = (jx ** 2 + jy ** 2 + jz ** 2) ** 0.5
        vtf = hp.tully_fisher_velocity(pl, cx, cy, cz, s.x, s.y, s.z, vx, vy, vz, jx, jy, jz, s.vx, s.vy, s.vz,
                                       s.mass, rad05)
        kco = hp.kinematic_morphology(pl, s.x, s.y, s.z, s.vx, s.vy, s.vz, s.mass, cx, cy, cz, vx, vy, vz, jx, jy, jz)
        sa, sb, sc = hp.halo_shape_fortran(pl, s.x, s.y, s.z, s.mass, cx, cy, cz, rad05)
        sig3 = hp.sigma_effective(pl, rad05, s.x, s.y, s.z, s.vx, s.vy, s.vz, cx, cy, cz, vx, vy, vz)
        grid = np.arange(-(rmax + LL), rmax + LL, 2 * LL)
        s1x, s1y, s1z, vsig, lam = hp.sigma_projections_fortran(grid, len(grid), pl, s.x, s.y, s.z, s.vx, s.vy,
                                                                s.vz, vx, vy, vz, s.mass, cx, cy, cz,
                                                                r05x, r05y, r05z, LL)
        rows.append([cx, cy, cz, mass, rmax, rad05, r05x, r05y, r05z, vx, vy, vz, jx, jy, jz, j, vtf, kco,
                     sa, sb, sc, sig3, s1x, s1y, s1z, vsig, lam])
    lens = [len(g) for g in cl["new_groups"]]
    out = {"x": s.x, "y": s.y, "z": s.z, "vx": s.vx, "vy": s.vy, "vz": s.vz, "m": s.mass,
           "off": np.concatenate(([0], np.cumsum(lens))).astype(np.int64),
           "mem": np.concatenate([np.asarray(g, dtype=np.int64) for g in cl["new_groups"]]),
           "rows": np.array(rows, dtype=np.float64), "ll": np.float64(LL)}
    np.savez_compressed(os.path.join(HERE, "properties.npz"), **out)
    print(f"  halo properties (O(N) set): {len(rows)} groups")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("PYHALMA_REFERENCE"),
                    help="pyHALMA checkout (default: $PYHALMA_REFERENCE)")
    ap.add_argument("--only", default="")
    args = ap.parse_args()
    if not args.reference:
        ap.error("give the pyHALMA checkout with --reference DIR or PYHALMA_REFERENCE")
    fof, hg, hp = import_reference(args.reference)
    todo = args.only.split(",") if args.only else ["fof", "config1", "pred", "props", "rps", "sub", "ball",
                                                    "psc", "prop", "amr", "escape"]
    if "fof" in todo:
        fof_cases(fof)
    if "config1" in todo:
        fof_config1(fof)
    if "pred" in todo:
        predicate_pairs(fof)
    if "props" in todo:
        halo_props(hp)
    if "rps" in todo:
        rps_cases(hg)
    if "sub" in todo:
        substructure_cases(fof, hp, args.reference)
    if "ball" in todo:
        ball_cases(hg)
    if "psc" in todo:
        psc_cases(fof, hp, args.reference)
    if "prop" in todo:
        property_cases(hp)
    if "amr" in todo:
        amr_cases(hg)
    if "escape" in todo:
        escape_cases(hp)


if __name__ == "__main__":
    main()
