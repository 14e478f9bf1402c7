"""Seeded synthetic star/gas snapshots for the halo-finding hot path.

pyHALMA reads MASCLET snapshots (``pyHALMA.py:498``); those are not available, so every
workload here is generated from closed-form profiles with ``numpy.random.default_rng``:

* Plummer spheres: r = a / sqrt(u^(-2/3) - 1) (u clipped to [1e-6, 0.999]), isotropic
  directions, scale radius a = 2 kpc * (M / 1e10 Msun)^(1/3), isotropic Gaussian velocities
  with sigma = sqrt(G M / (6 a)) plus a bulk velocity ~ N(0, 200 km/s) per sphere.
* Contaminants: uniform inside 3a, speed 3 * v_esc(r) in a random direction
  (v_esc^2 = 2 G M / sqrt(r^2 + a^2)), so the unbinding cut has work to do.
* Uniform background particles with sigma = 300 km/s.
* Power-law halo catalogues: dN/dlogN ∝ N^-alpha between n_min and n_max.
* NFW gas haloes (concentration c, virial radius r_vir) with lognormal cell masses,
  thermal dispersion plus solid-body-like rotation about a random axis.

Positions are generated in kpc and returned in Mpc (the unit the reference functions take,
``pyHALMA.py:61``); velocities are km/s and masses Msun.  G = 4.3e-3 pc (km/s)^2 / Msun as in
``python_scripts/halo_gas.py:459-462``.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

G_PC = 4.3e-3                 # (km/s)^2 pc / Msun, halo_gas.py:459
G_KPC = G_PC * 1e-3           # (km/s)^2 kpc / Msun
G_MPC = G_PC * 1e-6           # (km/s)^2 Mpc / Msun, halo_gas.py:460


@dataclass
class Snapshot:
    """Star particles of one synthetic snapshot (reference units: Mpc, km/s, Msun)."""
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    vx: np.ndarray
    vy: np.ndarray
    vz: np.ndarray
    mass: np.ndarray
    sphere: np.ndarray            # generating sphere id, -1 for background
    contaminant: np.ndarray       # True for injected unbound contaminants
    box_mpc: float
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.x.shape[0])


def plummer_scale_radius_kpc(mass_msun):
    return 2.0 * (np.asarray(mass_msun, dtype=np.float64) / 1e10) ** (1.0 / 3.0)


def _unit_vectors(rng, n):
    v = rng.normal(size=(n, 3))
    nrm = np.linalg.norm(v, axis=1)
    nrm[nrm == 0] = 1.0
    return v / nrm[:, None]


def _largest_remainder(weights, total, minimum=1):
    w = np.asarray(weights, dtype=np.float64)
    raw = w / w.sum() * total
    base = np.maximum(np.floor(raw).astype(np.int64), minimum)
    deficit = int(total - base.sum())
    if deficit > 0:
        order = np.argsort(-(raw - np.floor(raw)))
        base[order[:deficit]] += 1
    elif deficit < 0:
        order = np.argsort(-base)
        i = 0
        while deficit < 0:
            j = order[i % len(order)]
            if base[j] > minimum:
                base[j] -= 1
                deficit += 1
            i += 1
    return base


def _spheres(rng, counts, masses, centres_kpc, bulk, contaminant_frac):
    """Vectorised Plummer spheres (+ contaminants); returns kpc / km/s arrays."""
    counts = np.asarray(counts, dtype=np.int64)
    n_tot = int(counts.sum())
    sid = np.repeat(np.arange(len(counts)), counts)
    M = np.repeat(masses, counts)
    a = plummer_scale_radius_kpc(M)
    n_cont = np.floor(contaminant_frac * counts + 0.5).astype(np.int64)
    # the last n_cont members of each sphere are contaminants
    start = np.concatenate(([0], np.cumsum(counts)[:-1]))
    rank = np.arange(n_tot) - np.repeat(start, counts)
    cont = rank >= np.repeat(counts - n_cont, counts)

    u = rng.uniform(1e-6, 0.999, n_tot)
    r = a / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
    rc = 3.0 * a * rng.uniform(0.0, 1.0, n_tot) ** (1.0 / 3.0)
    r = np.where(cont, rc, r)
    pos = np.repeat(centres_kpc, counts, axis=0) + r[:, None] * _unit_vectors(rng, n_tot)

    sigma = np.sqrt(G_KPC * M / (6.0 * a))
    vel = rng.normal(size=(n_tot, 3)) * sigma[:, None]
    vesc = np.sqrt(2.0 * G_KPC * M / np.sqrt(r * r + a * a))
    vc = (3.0 * vesc)[:, None] * _unit_vectors(rng, n_tot)
    vel = np.where(cont[:, None], vc, vel) + np.repeat(bulk, counts, axis=0)
    return pos, vel, sid, cont


def plummer_snapshot(n_particles, n_spheres, *, seed=0, box_mpc=10.0, bg_frac=0.10,
                     contaminant_frac=0.0, m_lo=1e8, m_hi=1e11, bulk_sigma=200.0,
                     bg_sigma=300.0) -> Snapshot:
    """Plummer-sphere snapshot of the small/medium workloads.

    1e5 particles / 50 spheres / no contaminants is the CPU-runnable case; 2e6 particles /
    500 spheres / 15 % contaminants is the single-GPU headline case.
    """
    rng = np.random.default_rng(seed)
    box_kpc = box_mpc * 1e3
    n_bg = int(round(bg_frac * n_particles))
    n_halo = n_particles - n_bg
    masses = np.exp(rng.uniform(np.log(m_lo), np.log(m_hi), n_spheres))
    counts = _largest_remainder(masses, n_halo)
    a_max = plummer_scale_radius_kpc(masses).max()
    margin = min(20.0 * a_max, 0.25 * box_kpc)
    centres = rng.uniform(-box_kpc / 2 + margin, box_kpc / 2 - margin, (n_spheres, 3))
    bulk = rng.normal(0.0, bulk_sigma, (n_spheres, 3))
    pos, vel, sid, cont = _spheres(rng, counts, masses, centres, bulk, contaminant_frac)
    pmass = np.repeat(masses / counts, counts)

    bg_pos = rng.uniform(-box_kpc / 2, box_kpc / 2, (n_bg, 3))
    bg_vel = rng.normal(0.0, bg_sigma, (n_bg, 3))
    bg_mass = np.full(n_bg, masses.sum() / max(n_halo, 1))

    pos = np.concatenate([pos, bg_pos]) / 1e3
    vel = np.concatenate([vel, bg_vel])
    mass = np.concatenate([pmass, bg_mass])
    sid = np.concatenate([sid, np.full(n_bg, -1)])
    cont = np.concatenate([cont, np.zeros(n_bg, dtype=bool)])
    return Snapshot(np.ascontiguousarray(pos[:, 0]), np.ascontiguousarray(pos[:, 1]),
                    np.ascontiguousarray(pos[:, 2]), np.ascontiguousarray(vel[:, 0]),
                    np.ascontiguousarray(vel[:, 1]), np.ascontiguousarray(vel[:, 2]),
                    mass, sid.astype(np.int64), cont, box_mpc,
                    dict(seed=seed, n_spheres=n_spheres, bg_frac=bg_frac,
                         contaminant_frac=contaminant_frac, sphere_mass=masses,
                         sphere_counts=counts, sphere_centre_kpc=centres))


def bridged_snapshot(n_pairs, n_single, *, seed=0, box_mpc=2.0, n_lo=300, n_hi=6000, sep_lo=4.0, sep_hi=8.0,
                     bridge_step_kpc=1.1, bg_frac=0.05, particle_mass=1e6, bulk_sigma=200.0,
                     bg_sigma=300.0) -> Snapshot:
    """Pairs of Plummer spheres joined by a thin stream, for the substructure block.

    Each pair: two spheres of log-uniform particle counts in [n_lo, n_hi] whose centres are
    sep_lo..sep_hi times the sum of their scale radii apart, and a line of particles between
    the centres every bridge_step_kpc (jittered by 0.05 kpc): the line links at a linking
    length of 1.5 kpc but not at 0.75 kpc, so FoF merges the pair and the sub-FoF of the
    substructure block separates it.  Plus n_single lone spheres and a uniform background.
    Positions in Mpc; ``sphere`` is the generating sphere id, -2 for stream particles and
    -1 for background.
    """
    rng = np.random.default_rng(seed)
    box_kpc = box_mpc * 1e3
    n_sph = 2 * n_pairs + n_single
    counts = np.exp(rng.uniform(np.log(n_lo), np.log(n_hi), n_sph)).astype(np.int64)
    masses = counts * particle_mass
    a = plummer_scale_radius_kpc(masses)
    margin = 0.1 * box_kpc
    centres = rng.uniform(-box_kpc / 2 + margin, box_kpc / 2 - margin, (n_sph, 3))
    first, second = np.arange(n_pairs), np.arange(n_pairs, 2 * n_pairs)
    sep = rng.uniform(sep_lo, sep_hi, n_pairs) * (a[first] + a[second])
    centres[second] = centres[first] + _unit_vectors(rng, n_pairs) * sep[:, None]
    bulk = rng.normal(0.0, bulk_sigma, (n_sph, 3))
    pos, vel, sid, _ = _spheres(rng, counts, masses, centres, bulk, 0.0)
    streams_p, streams_v = [], []
    for k in range(n_pairs):
        c0, c1 = centres[first[k]], centres[second[k]]
        steps = max(int(np.linalg.norm(c1 - c0) / bridge_step_kpc), 1)
        t = (np.arange(1, steps) / steps)[:, None]
        streams_p.append(c0 + t * (c1 - c0) + rng.normal(0.0, 0.05, (steps - 1, 3)))
        streams_v.append(0.5 * (bulk[first[k]] + bulk[second[k]]) + rng.normal(0.0, 30.0, (steps - 1, 3)))
    sp = np.concatenate(streams_p) if streams_p else np.zeros((0, 3))
    sv = np.concatenate(streams_v) if streams_v else np.zeros((0, 3))
    n_in = pos.shape[0] + sp.shape[0]
    n_bg = int(round(bg_frac * n_in / (1.0 - bg_frac)))
    bg_pos = rng.uniform(-box_kpc / 2, box_kpc / 2, (n_bg, 3))
    bg_vel = rng.normal(0.0, bg_sigma, (n_bg, 3))
    pos = np.concatenate([pos, sp, bg_pos]) / 1e3
    vel = np.concatenate([vel, sv, bg_vel])
    n = pos.shape[0]
    sid = np.concatenate([sid, np.full(sp.shape[0], -2), np.full(n_bg, -1)])
    return Snapshot(np.ascontiguousarray(pos[:, 0]), np.ascontiguousarray(pos[:, 1]),
                    np.ascontiguousarray(pos[:, 2]), np.ascontiguousarray(vel[:, 0]),
                    np.ascontiguousarray(vel[:, 1]), np.ascontiguousarray(vel[:, 2]),
                    np.full(n, particle_mass), sid.astype(np.int64), np.zeros(n, dtype=bool), box_mpc,
                    dict(seed=seed, n_pairs=n_pairs, n_single=n_single, stream_particles=int(sp.shape[0]),
                         background=n_bg))


def powerlaw_counts(rng, n_haloes, alpha=1.0, n_min=50, n_max=200_000):
    """Halo sizes with dN/dlogN ∝ N^-alpha on [n_min, n_max] (inverse CDF in log N)."""
    u = rng.uniform(0.0, 1.0, n_haloes)
    if abs(alpha) < 1e-12:
        logn = np.log(n_min) + u * (np.log(n_max) - np.log(n_min))
        n = np.exp(logn)
    else:
        lo, hi = n_min ** (-alpha), n_max ** (-alpha)
        n = (lo - u * (lo - hi)) ** (-1.0 / alpha)
    return np.clip(np.floor(n + 0.5).astype(np.int64), n_min, n_max)


@dataclass
class HaloCatalogue:
    """Haloes already grouped: members of halo h are rows offsets[h]:offsets[h+1]."""
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    vx: np.ndarray
    vy: np.ndarray
    vz: np.ndarray
    mass: np.ndarray
    offsets: np.ndarray
    contaminant: np.ndarray
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    @property
    def n_haloes(self) -> int:
        return int(self.offsets.shape[0] - 1)


def powerlaw_catalogue(n_haloes, *, seed=0, alpha=1.0, n_min=50, n_max=200_000,
                       particle_mass=1e6, box_mpc=100.0, contaminant_frac=0.15,
                       bulk_sigma=200.0) -> HaloCatalogue:
    """Batched-unbinding workload: independent Plummer haloes of power-law sizes."""
    rng = np.random.default_rng(seed)
    counts = powerlaw_counts(rng, n_haloes, alpha, n_min, n_max)
    masses = counts * particle_mass
    box_kpc = box_mpc * 1e3
    centres = rng.uniform(-box_kpc / 2, box_kpc / 2, (n_haloes, 3))
    bulk = rng.normal(0.0, bulk_sigma, (n_haloes, 3))
    pos, vel, _, cont = _spheres(rng, counts, masses, centres, bulk, contaminant_frac)
    pos = pos / 1e3
    offsets = np.concatenate(([0], np.cumsum(counts))).astype(np.int64)
    return HaloCatalogue(np.ascontiguousarray(pos[:, 0]), np.ascontiguousarray(pos[:, 1]),
                         np.ascontiguousarray(pos[:, 2]), np.ascontiguousarray(vel[:, 0]),
                         np.ascontiguousarray(vel[:, 1]), np.ascontiguousarray(vel[:, 2]),
                         np.full(pos.shape[0], particle_mass), offsets, cont,
                         dict(seed=seed, alpha=alpha, n_min=n_min, n_max=n_max,
                              total=int(counts.sum()), sum_n2=float((counts.astype(np.float64) ** 2).sum())))


def powerlaw_mean(alpha, n_min=50, n_max=200_000):
    """Mean halo size of dN/dlogN ∝ N^-alpha on [n_min, n_max] (closed form)."""
    a = float(alpha)
    if abs(a) < 1e-9:
        return (n_max - n_min) / np.log(n_max / n_min)
    if abs(a - 1.0) < 1e-9:
        return np.log(n_max / n_min) / (1.0 / n_min - 1.0 / n_max)
    return (a / (a - 1.0)) * (n_min ** (1 - a) - n_max ** (1 - a)) / (n_min ** (-a) - n_max ** (-a))


def alpha_for_mean(mean, n_min=50, n_max=200_000):
    """The slope whose mean halo size is `mean` (bisection; the mean falls as alpha grows)."""
    lo, hi = -1.0, 3.0
    for _ in range(100):
        mid = 0.5 * (lo + hi)
        if powerlaw_mean(mid, n_min, n_max) > mean:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def full_snapshot(n_total=200_000_000, n_haloes=200_000, *, seed=0, box_mpc=100.0, bg_frac=0.20,
                  bridge_frac=0.05, alpha=None, n_min=50, n_max=200_000, particle_mass=1e6,
                  bulk_sigma=200.0, bg_sigma=300.0, contaminant_frac=0.0, chunk=20_000):
    """Large snapshot: power-law Plummer haloes (a fraction placed in pairs within 2a of a
    partner to form FoF bridges) plus a uniform background.  With alpha=None the slope is
    chosen so that haloes hold (1 - bg_frac) of n_total on average; the background fills the
    rest up to n_total.  ``contaminant_frac`` of each halo's members are contaminants (uniform
    inside 3a at 3 v_esc).  Returns float64 arrays in Mpc, km/s, Msun and the per-particle
    generating halo id (-1 background)."""
    rng = np.random.default_rng(seed)
    n_bg_target = int(round(bg_frac * n_total))
    if alpha is None:
        alpha = alpha_for_mean((n_total - n_bg_target) / n_haloes, n_min, n_max)
    counts = powerlaw_counts(rng, n_haloes, alpha, n_min, n_max)
    masses = counts * particle_mass
    a = plummer_scale_radius_kpc(masses)
    box_kpc = box_mpc * 1e3
    centres = rng.uniform(-box_kpc / 2, box_kpc / 2, (n_haloes, 3))
    n_pair = int(bridge_frac * n_haloes) // 2 * 2
    pick = rng.choice(n_haloes, n_pair, replace=False)
    first, second = pick[: n_pair // 2], pick[n_pair // 2:]
    offs = _unit_vectors(rng, len(first)) * (rng.uniform(0, 2.0, len(first)) * a[first])[:, None]
    centres[second] = np.clip(centres[first] + offs, -box_kpc / 2, box_kpc / 2)
    bulk = rng.normal(0.0, bulk_sigma, (n_haloes, 3))
    n_halo = int(counts.sum())
    n_bg = max(n_total - n_halo, 0)
    n = n_halo + n_bg
    out = {k: np.empty(n) for k in ("x", "y", "z", "vx", "vy", "vz")}
    hid = np.empty(n, dtype=np.int32)
    cont = np.zeros(n, dtype=bool)
    pos = 0
    for h0 in range(0, n_haloes, chunk):
        sl = slice(h0, min(h0 + chunk, n_haloes))
        p, v, sid, c = _spheres(rng, counts[sl], masses[sl], centres[sl], bulk[sl], contaminant_frac)
        k = p.shape[0]
        for d, key in enumerate(("x", "y", "z")):
            out[key][pos:pos + k] = p[:, d] / 1e3
        for d, key in enumerate(("vx", "vy", "vz")):
            out[key][pos:pos + k] = v[:, d]
        hid[pos:pos + k] = sid + h0
        cont[pos:pos + k] = c
        pos += k
    for q0 in range(0, n_bg, 10_000_000):
        k = min(10_000_000, n_bg - q0)
        for key in ("x", "y", "z"):
            out[key][pos:pos + k] = rng.uniform(-box_kpc / 2, box_kpc / 2, k) / 1e3
        for key in ("vx", "vy", "vz"):
            out[key][pos:pos + k] = rng.normal(0.0, bg_sigma, k)
        hid[pos:pos + k] = -1
        pos += k
    mass = np.full(n, particle_mass)
    return Snapshot(out["x"], out["y"], out["z"], out["vx"], out["vy"], out["vz"], mass, hid, cont, box_mpc,
                    dict(seed=seed, alpha=alpha, n_haloes=n_haloes, halo_particles=n_halo, background=n_bg,
                         bridged_pairs=n_pair // 2, contaminant_frac=contaminant_frac,
                         halo_counts=counts))


def _nfw_radius(rng, n, c, r_vir):
    """Inverse-CDF sampling of the NFW enclosed-mass profile inside r_vir (tabulated)."""
    rs = r_vir / c
    xs = np.concatenate(([0.0], np.geomspace(1e-5, c, 4096)))
    mu = np.log1p(xs) - xs / (1.0 + xs)
    u = rng.uniform(0.0, mu[-1], n)
    return rs * np.interp(u, mu, xs)


@dataclass
class GasHalo:
    gas_x: np.ndarray
    gas_y: np.ndarray
    gas_z: np.ndarray
    gas_vx: np.ndarray
    gas_vy: np.ndarray
    gas_vz: np.ndarray
    gas_mass: np.ndarray
    gas_temp: np.ndarray
    st_x: np.ndarray
    st_y: np.ndarray
    st_z: np.ndarray
    st_mass: np.ndarray
    bulk: np.ndarray
    meta: dict = field(default_factory=dict)


def nfw_gas_halo(n_gas, n_stars, *, seed=0, c=8.0, r_vir_kpc=150.0, mass_mu=np.log(1e5),
                 mass_sigma=1.0, sigma_th=100.0, v_rot=150.0, star_mass=1e5,
                 centre_mpc=(0.0, 0.0, 0.0)) -> GasHalo:
    """Gas cells on an NFW profile plus a Plummer stellar body (float32 gas positions)."""
    rng = np.random.default_rng(seed)
    centre = np.asarray(centre_mpc, dtype=np.float64) * 1e3
    r = _nfw_radius(rng, n_gas, c, r_vir_kpc)
    gpos = r[:, None] * _unit_vectors(rng, n_gas)
    axis = _unit_vectors(rng, 1)[0]
    tang = np.cross(axis[None, :], gpos)
    tn = np.linalg.norm(tang, axis=1)
    tn[tn == 0] = 1.0
    bulk = rng.normal(0.0, 200.0, 3)
    gvel = rng.normal(size=(n_gas, 3)) * sigma_th + v_rot * tang / tn[:, None] + bulk
    gmass = np.exp(rng.normal(mass_mu, mass_sigma, n_gas))
    gtemp = np.exp(rng.normal(np.log(3e4), 1.5, n_gas))
    m_st = n_stars * star_mass
    a = plummer_scale_radius_kpc(m_st)
    u = rng.uniform(1e-6, 0.999, n_stars)
    rs = a / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
    spos = rs[:, None] * _unit_vectors(rng, n_stars)
    gpos = ((gpos + centre) / 1e3).astype(np.float32)
    spos = (spos + centre) / 1e3
    return GasHalo(np.ascontiguousarray(gpos[:, 0]), np.ascontiguousarray(gpos[:, 1]),
                   np.ascontiguousarray(gpos[:, 2]), gvel[:, 0].copy(), gvel[:, 1].copy(),
                   gvel[:, 2].copy(), gmass, gtemp, np.ascontiguousarray(spos[:, 0]),
                   np.ascontiguousarray(spos[:, 1]), np.ascontiguousarray(spos[:, 2]),
                   np.full(n_stars, star_mass), bulk,
                   dict(seed=seed, c=c, r_vir_kpc=r_vir_kpc))


def lattice_points(n_side, spacing, *, origin=(0.0, 0.0, 0.0), jitter_ulps=0, seed=0):
    """Cubic lattice (adversarial FoF input: neighbour distances sit exactly at the spacing)."""
    rng = np.random.default_rng(seed)
    g = np.arange(n_side, dtype=np.float64)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1) * spacing + np.asarray(origin)
    for _ in range(int(jitter_ulps)):
        d = rng.integers(-1, 2, pts.shape)
        pts = np.where(d > 0, np.nextafter(pts, np.inf), np.where(d < 0, np.nextafter(pts, -np.inf), pts))
    return pts


@dataclass
class AMRGrid:
    """A MASCLET-like AMR gas grid in the reference's tuple layout: ``grid_data[2]`` nl,
    ``[5]`` npatch (patches per level, npatch[0] = 0), ``[6:9]`` patchnx/ny/nz, ``[12:15]``
    patchrx/ry/rz (the centre of each patch's first cell of the parent level, Mpc);
    ``gas_data`` = [delta, vx, vy, vz, temp, cr0amr, solapst], each a list of per-patch 3-D
    arrays indexed [ix, iy, iz] (velocities in units of c).  Patch 0 is the base grid; the
    conversion never reads its cells, so it is stored as a single cell."""
    grid_data: list
    gas_data: list
    L: float
    ncoarse: int
    rho_B: float
    centre: np.ndarray


def amr_grid(*, seed=0, L=40.0, ncoarse=128, levels=(1, 2, 3, 4, 5, 6, 7), per_level=2, n_lo=6, n_hi=14,
             centre_mpc=(1.3, -0.7, 2.2), rho_B=5e10, sigma_v_kms=120.0):
    """Synthetic refined patches around a halo centre: per level `per_level` patches of
    n_lo..n_hi cells a side placed over the centre with random offsets, lognormal overdensity
    rising towards the centre, Gaussian velocities, about 25 % refined / 15 % overlapped
    cells (cr0amr / solapst false).  Cell values are float32 numbers (MASCLET writes float32
    fields) held in float64 arrays."""
    rng = np.random.default_rng(seed)
    c = np.asarray(centre_mpc, dtype=np.float64)
    cell0 = L / ncoarse
    nx, ny, nz, rx, ry, rz, lev = [1], [1], [1], [0.0], [0.0], [0.0], [0]
    fields = [[np.zeros((1, 1, 1))] for _ in range(5)] + [[np.zeros((1, 1, 1), dtype=bool)] for _ in range(2)]
    npatch = [0] * (max(levels) + 1)
    for lvl in levels:
        res = cell0 / 2 ** lvl
        for _ in range(per_level):
            n = rng.integers(n_lo, n_hi + 1, 3)
            off = (n / 2.0 + rng.uniform(-0.3, 0.3, 3) * n) * res
            r0 = c - off + res / 2.0          # centre of the first cell of the parent level
            nx.append(int(n[0]))
            ny.append(int(n[1]))
            nz.append(int(n[2]))
            rx.append(float(r0[0]))
            ry.append(float(r0[1]))
            rz.append(float(r0[2]))
            lev.append(lvl)
            npatch[lvl] += 1
            ix, iy, iz = np.meshgrid(np.arange(n[0]), np.arange(n[1]), np.arange(n[2]), indexing="ij")
            px = r0[0] - res / 2 + ix * res - c[0]
            py = r0[1] - res / 2 + iy * res - c[1]
            pz = r0[2] - res / 2 + iz * res - c[2]
            rr = np.sqrt(px * px + py * py + pz * pz) * 1e3   # kpc
            shape = tuple(int(v) for v in n)
            f32 = lambda a: a.astype(np.float32).astype(np.float64)
            fields[0].append(f32(np.exp(rng.normal(np.log(2e3 / (1.0 + rr / 5.0) ** 2), 0.8, shape))))
            for k in (1, 2, 3):
                fields[k].append(f32(rng.normal(0.0, sigma_v_kms / 3e5, shape)))
            fields[4].append(f32(np.exp(rng.normal(np.log(3e4), 1.0, shape))))
            fields[5].append(rng.random(shape) > 0.25)
            fields[6].append(rng.random(shape) > 0.15)
    grid = [None] * 15
    grid[2] = max(levels)
    grid[5] = np.array(npatch, dtype=np.int64)
    grid[6], grid[7], grid[8] = (np.array(a, dtype=np.int64) for a in (nx, ny, nz))
    grid[12], grid[13], grid[14] = (np.array(a, dtype=np.float64) for a in (rx, ry, rz))
    return AMRGrid(grid, fields, float(L), int(ncoarse), float(rho_B), c)
