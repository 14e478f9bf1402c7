"""GPU per-halo FP64 reductions against the reference's numba kernels (golden) and the
NumPy oracle (relative 1e-12; half-mass radius exact up to summation-order ties)."""
import numpy as np
import pytest

from oracle import reductions as ref
from pyhalma_gb300 import halo_properties as hp, synth

pytestmark = pytest.mark.gpu


def test_single_halo_dropins_match_reference(golden, cuda):
    d = golden("halo_props.npz")
    x, y, z, vx, vy, vz, m = (d[k] for k in ("x", "y", "z", "vx", "vy", "vz", "m"))
    for h, row in enumerate(d["results"]):
        pl = d[f"pl{h}"]
        tm, cx, cy, cz, M, ux, uy, uz, rmax, r05, sig = row
        assert np.isclose(hp.total_mass(pl, m), tm, rtol=1e-12)
        assert np.allclose(hp.center_of_mass(pl, x, y, z, m), (cx, cy, cz, M), rtol=1e-12, atol=0)
        assert np.allclose(hp.CM_velocity(M, pl, vx, vy, vz, m), (ux, uy, uz), rtol=1e-11, atol=1e-9)
        assert np.isclose(hp.furthest_particle(cx, cy, cz, pl, x, y, z), rmax, rtol=1e-12)
        assert np.isclose(hp.half_mass_radius(cx, cy, cz, M, pl, x, y, z, m), r05, rtol=1e-12)
        assert np.isclose(hp.sigma_effective(pl, r05, x, y, z, vx, vy, vz, cx, cy, cz, ux, uy, uz), sig, rtol=1e-11)


def test_batched_reductions_with_mask(cuda):
    cat = synth.powerlaw_catalogue(300, seed=8, n_min=50, n_max=20_000)
    rng = np.random.default_rng(1)
    mask = (rng.random(cat.n) < 0.8).astype(np.uint8)
    out = hp.halo_reductions(cat.offsets, cat.x, cat.y, cat.z, cat.vx, cat.vy, cat.vz, cat.mass, mask=mask)
    for h in range(0, 300, 7):
        pl = np.arange(cat.offsets[h], cat.offsets[h + 1])
        pl = pl[mask[pl] == 1]
        cx, cy, cz, M = ref.center_of_mass(pl, cat.x, cat.y, cat.z, cat.mass)
        ux, uy, uz = ref.CM_velocity(M, pl, cat.vx, cat.vy, cat.vz, cat.mass)
        r05 = ref.half_mass_radius(cx, cy, cz, M, pl, cat.x, cat.y, cat.z, cat.mass)
        row = out[h]
        assert np.allclose(row[:7], (M, cx, cy, cz, ux, uy, uz), rtol=1e-12, atol=1e-12)
        assert np.isclose(row[7], ref.furthest_particle(cx, cy, cz, pl, cat.x, cat.y, cat.z), rtol=1e-12)
        assert np.isclose(row[8], r05, rtol=1e-12)
        # same centre as the GPU: members at d == R05 split identically (d < R05 is strict)
        sig = ref.sigma_effective(pl, row[8], cat.x, cat.y, cat.z, cat.vx, cat.vy, cat.vz, *row[1:7])
        assert np.isclose(row[9], sig, rtol=1e-11)
        assert row[10] == len(pl)


def test_empty_and_tiny_segments(cuda):
    off = np.array([0, 0, 1, 3], dtype=np.int64)
    x = np.array([1.0, 2.0, 4.0])
    m = np.array([1.0, 1.0, 3.0])
    out = hp.halo_reductions(off, x, x, x, x, x, x, m)
    assert out[0, 0] == 0 and out[0, 10] == 0
    assert out[1, 0] == 1 and out[1, 1] == 1.0 and out[1, 8] == 0.0
    assert out[2, 0] == 4 and np.isclose(out[2, 1], 3.5)


def _walk_cases():
    """Mass sequences whose running FP64 sum rounds in every way a sequential walk can:
    non-dyadic equal masses (rounding at every step), ties of exactly half an ulp, binade
    crossings, masses far above or below the running sum, zeros, subnormals, and a negative
    mass (plain FP64 adds)."""
    rng = np.random.default_rng(12)
    u = 2.0 ** -53
    cases = [
        np.full(20_001, 0.1), np.full(20_000, 0.1), np.full(5000, 1.0), np.full(3000, 1e6 / 3),
        np.concatenate([[1.0], np.tile([u, 3 * u, u / 2, 5 * u, 2 * u], 4000)]),      # ties at 1.0's ulp
        np.concatenate([[1.0], np.full(20_000, u)]),                                   # every step a tie
        np.concatenate([[3.0], np.tile([2 * u, 6 * u, u], 3000), [1.0, 7.0]]),
        np.exp(rng.uniform(np.log(1e-30), np.log(1e30), 4000)),                        # binade jumps
        rng.uniform(0.5, 2.0, 30_000) * 1e7, rng.integers(1, 9, 10_000).astype(np.float64) * 2.0 ** -1070,
        np.concatenate([[0.0, 0.0, 5e-324], rng.uniform(0, 1, 5000), [0.0]]),
        np.concatenate([rng.uniform(0, 1, 3000), [-0.25], rng.uniform(0, 1, 3000)]),
        np.concatenate([[1e300], rng.uniform(0, 1, 2000)]), np.array([2.5]),
    ]
    cases += [rng.permutation(c) for c in cases[4:8]]
    return cases


def test_half_mass_walk_is_the_sequential_sum(cuda):
    """R05 from the integer-emulated walk against numpy's sequential cumsum walk, bit for bit,
    with the caller's centre and reference mass (about) so that only the walk is compared;
    the reference mass is the exact sum plus or minus a few ulps so that M/2 lands on the
    values the walk passes through."""
    cases = _walk_cases()
    sizes = [len(c) for c in cases]
    off = np.zeros(len(cases) * 3 + 1, dtype=np.int64)
    ms, xs, about = [], [], []
    for c in cases:
        x = np.arange(1, len(c) + 1, dtype=np.float64) * 1e-3      # walk order = index order
        cm = np.cumsum(c)
        for Mref in (cm[-1], 2 * cm[len(c) // 2], np.nextafter(2 * cm[len(c) // 3], np.inf)):
            ms.append(c)
            xs.append(x)
            a = np.full(hp.N_ABOUT, np.nan)
            a[:3] = 0.0
            a[6] = Mref
            about.append(a)
    for k, mm in enumerate(ms):
        off[k + 1] = off[k] + len(mm)
    m = np.concatenate(ms)
    x = np.concatenate(xs)
    z0 = np.zeros_like(x)
    out = hp.halo_reductions(off, x, z0, z0, z0, z0, z0, m, about=np.array(about))
    for k in range(len(ms)):
        pl = np.arange(off[k], off[k + 1])
        r05 = ref.half_mass_radius(0.0, 0.0, 0.0, about[k][6], pl, x, z0, z0, m)
        assert out[k, 8] == r05, (k, sizes[k // 3], out[k, 8], r05)


def test_device_offsets_outside_the_rows_are_refused(cuda):
    import torch
    x = torch.zeros(4, dtype=torch.float64, device=cuda)
    with pytest.raises(ValueError, match="offsets"):
        hp.halo_reductions(torch.tensor([0, 2, 5], device=cuda), *[x] * 7)
    with pytest.raises(ValueError, match="offsets"):
        hp.halo_reductions(torch.tensor([0, 3, 2, 4], device=cuda), *[x] * 7)
    out = hp.halo_reductions(torch.tensor([0, 1, 4], device=cuda), *[x] * 6, torch.ones(4, dtype=torch.float64,
                                                                                              device=cuda))
    assert out[:, 0].cpu().tolist() == [1.0, 3.0]
