"""GPU FoF parity: bit-exact partition and labels against the reference (golden fixtures)
and against the exact C oracle at the single-GPU workload size."""
import hashlib

import numpy as np
import pytest

import oracle
from pyhalma_gb300 import fof, synth

pytestmark = pytest.mark.gpu


def _cases(d):
    return sorted(set(k.split("__")[0] for k in d.files))


def test_reference_cases_bit_exact(golden, cuda):
    d = golden("fof_cases.npz")
    for name in _cases(d):
        xyz = d[name + "__xyz"]
        ll = float(d[name + "__ll"])
        lab = fof.fof_labels(xyz[:, 0].copy(), xyz[:, 1].copy(), xyz[:, 2].copy(), ll)
        assert np.array_equal(lab, d[name + "__labels"]), name
        groups = fof.friends_of_friends(xyz, ll)
        assert groups == oracle.labels_to_groups(d[name + "__labels"]), name


def test_reference_config1_bit_exact(golden, cuda):
    c = golden("fof_config1.npz")
    x, y, z = c["x"], c["y"], c["z"]          # the exact positions the reference saw
    groups = fof.friends_of_friends_serial(x, y, z, float(c["ll"]))
    assert len(groups) == int(c["ngroups"])
    assert np.array_equal(oracle.groups_to_labels(groups, len(x)), c["labels"])


def test_two_million_particles_match_oracle(cuda):
    s = synth.plummer_snapshot(2_000_000, 500, seed=1, box_mpc=10.0, contaminant_frac=0.15)
    lab = fof.fof_labels(s.x, s.y, s.z, 0.0015)
    ref = oracle.fof_labels(s.x, s.y, s.z, 0.0015)
    assert np.array_equal(lab, ref)
    # CSR groups: reference order, strict minp filter of the "parallel" variant
    off, mem = fof.fof_groups(lab, 50)
    ref_groups = [g for g in oracle.labels_to_groups(ref) if len(g) >= 50]
    assert len(off) - 1 == len(ref_groups)
    for g in (0, len(ref_groups) // 2, len(ref_groups) - 1):
        assert mem[off[g]:off[g + 1]].tolist() == ref_groups[g]


def test_device_tensors_in_place(cuda):
    import torch
    s = synth.plummer_snapshot(50_000, 20, seed=9, box_mpc=2.0)
    x, y, z = (torch.from_numpy(a).to(cuda) for a in (s.x, s.y, s.z))
    lab = fof.fof_labels(x, y, z, 0.0015)
    assert lab.is_cuda and lab.dtype == torch.int32
    assert np.array_equal(lab.cpu().numpy(), oracle.fof_labels(s.x, s.y, s.z, 0.0015))


def test_edge_cases(cuda):
    e = np.zeros(0)
    assert fof.friends_of_friends_serial(e, e, e, 0.0015) == []
    assert fof.friends_of_friends_serial(np.array([1.0]), np.array([2.0]), np.array([3.0]), 0.0015) == []
    # zero linking length links coincident points only
    p = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 0.0], [1e-12, 0.0, 0.0], [5.0, 5.0, 5.0], [5.0, 5.0, 5.0]])
    assert fof.friends_of_friends(p, 0.0) == [[0, 1], [3, 4]]
    # a linking length larger than the box puts everything in one group
    rng = np.random.default_rng(3)
    q = rng.uniform(0, 1, (1000, 3))
    assert fof.friends_of_friends(q, 10.0) == [list(range(1000))]
    with pytest.raises(ValueError):
        fof.friends_of_friends(np.array([[0.0, np.nan, 0.0], [0.0, 0.0, 0.0]]), 1.0)
    with pytest.raises(ValueError):
        fof.friends_of_friends(q, -1.0)


def test_parallel_variants_filter_strictly(cuda):
    s = synth.plummer_snapshot(30_000, 12, seed=2, box_mpc=1.0)
    groups = fof.friends_of_friends_parallel(s.x, s.y, s.z, 0.0015, 1.0, 50, s.mass)
    ref = [g for g in oracle.labels_to_groups(oracle.fof_labels(s.x, s.y, s.z, 0.0015)) if len(g) > 50]
    assert [g.tolist() for g in groups] == ref
    assert [g.tolist() for g in fof.pyfof_friends_of_friends_parallel(s.x, s.y, s.z, 0.0015, 1.0, 50, s.mass)] == ref


def test_dense_lattices_and_random_clusters_property(cuda):
    rng = np.random.default_rng(17)
    for trial in range(6):
        n = int(rng.integers(2_000, 40_000))
        pts = rng.normal(0, rng.uniform(0.001, 0.02), (n, 3)) + rng.uniform(-50, 50, 3)
        ll = float(rng.uniform(0.0002, 0.002))
        lab = fof.fof_labels(pts[:, 0].copy(), pts[:, 1].copy(), pts[:, 2].copy(), ll)
        assert np.array_equal(lab, oracle.fof_labels(pts[:, 0], pts[:, 1], pts[:, 2], ll)), trial
    # ties: lattice spacing equal to the linking length at large coordinates
    pts = synth.lattice_points(24, 0.0015, origin=(37.1, -12.3, 4.4), jitter_ulps=1, seed=4)
    lab = fof.fof_labels(pts[:, 0].copy(), pts[:, 1].copy(), pts[:, 2].copy(), 0.0015)
    assert np.array_equal(lab, oracle.fof_labels(pts[:, 0], pts[:, 1], pts[:, 2], 0.0015))


def test_far_offsets_and_elongated_boxes(cuda):
    """Cell keys stay exact far from the origin (a cloud 3e4 Mpc away) and on grids millions of
    cells long on one axis (a chain of particles 0.5-1.2 LL apart)."""
    rng = np.random.default_rng(23)
    pts = rng.normal(0, 0.003, (20_000, 3)) + np.array([1.0e4, -2.5e4, 7.5e3])
    lab = fof.fof_labels(pts[:, 0].copy(), pts[:, 1].copy(), pts[:, 2].copy(), 0.0007)
    assert np.array_equal(lab, oracle.fof_labels(pts[:, 0], pts[:, 1], pts[:, 2], 0.0007))
    n = 6000
    chain = np.zeros((n, 3))
    chain[:, 0] = 3.0e3 + np.cumsum(rng.uniform(0.5, 1.2, n)) * 0.001
    chain[:, 1] = rng.normal(0, 2e-5, n)
    chain[:, 2] = -4.0e2 + rng.normal(0, 2e-5, n)
    chain = np.concatenate([chain, chain[::7] + np.array([0.0, 1.0, 0.0])])   # a second, sparser line
    lab = fof.fof_labels(chain[:, 0].copy(), chain[:, 1].copy(), chain[:, 2].copy(), 0.001)
    assert np.array_equal(lab, oracle.fof_labels(chain[:, 0], chain[:, 1], chain[:, 2], 0.001))


def test_flat_and_thin_grids(cuda):
    """Grids one cell thick on one or two axes (planes and lines of particles): the neighbour
    keys of the padded key grid wrap across a row or column end there on every cell, and must
    land on the pad, never on a cell of the next row."""
    rng = np.random.default_rng(29)
    ll = 0.001
    cases = []
    # planes z = const (one cell in z), y = const (one cell in y)
    pl = rng.uniform(0, 0.2, (20_000, 3))
    cases.append((pl[:, 0], pl[:, 1], np.full(len(pl), 0.5)))
    cases.append((pl[:, 0], np.full(len(pl), -0.25), pl[:, 1]))
    # lines along x, y and z with steps of 0.5-1.2 LL and a parallel line 1.5 LL away
    for axis in range(3):
        t = np.cumsum(rng.uniform(0.5, 1.2, 5000)) * ll
        a = [np.full(len(t), 0.3), np.full(len(t), 0.3), np.full(len(t), 0.3)]
        a[axis] = t
        b = [v.copy() for v in a]
        b[(axis + 1) % 3] = b[(axis + 1) % 3] + 1.5 * ll
        cases.append(tuple(np.concatenate([u, v]) for u, v in zip(a, b)))
    for k, (x, y, z) in enumerate(cases):
        x, y, z = (np.ascontiguousarray(v, dtype=np.float64) for v in (x, y, z))
        lab = fof.fof_labels(x, y, z, ll)
        assert np.array_equal(lab, oracle.fof_labels(x, y, z, ll)), k


def test_integer_and_fma_key_maps(cuda):
    """Both maps from coordinates to quarter cells: the integer one (coordinates and grid within
    2^37 quarter cells) on a cloud straddling zero with signed zeros, subnormals and points on
    multiples of the linking length, and the FP64 FMA one on a cloud 1e8 length units from the
    origin (4e11 quarter cells), each against the oracle."""
    rng = np.random.default_rng(31)
    ll = 0.001
    pts = rng.normal(0, 0.004, (30_000, 3))
    special = np.array([[0.0, -0.0, 5e-324], [-5e-324, 0.0, -0.0], [2.2e-308, -2.2e-308, 0.0],
                        [ll, -ll, 0.0], [2 * ll, 0.0, -3 * ll], [-ll, -ll, -ll], [0.5 * ll, 0.5 * ll, 0.0]])
    grid = np.stack(np.meshgrid(*(np.arange(-4, 5) * ll,) * 3, indexing="ij"), axis=-1).reshape(-1, 3)
    pts = np.concatenate([pts, special, grid, grid + np.array([ll * (1 + 2 ** -40), 0.0, 0.0])])
    lab = fof.fof_labels(pts[:, 0].copy(), pts[:, 1].copy(), pts[:, 2].copy(), ll)
    assert np.array_equal(lab, oracle.fof_labels(pts[:, 0], pts[:, 1], pts[:, 2], ll))
    far = rng.normal(0, 0.004, (20_000, 3)) + np.array([1.0e8, -3.0e7, 2.0e8])
    lab = fof.fof_labels(far[:, 0].copy(), far[:, 1].copy(), far[:, 2].copy(), ll)
    assert np.array_equal(lab, oracle.fof_labels(far[:, 0], far[:, 1], far[:, 2], ll))


def test_groups_reject_labels_that_are_not_particle_indices(cuda):
    """Labels index the per-group counters; one outside [-1, n) is refused by the kernel that
    reads it (host and device labels), and the next call works as before."""
    import torch
    for bad in (np.array([0, 0, 5, -1, 2], dtype=np.int32), np.array([0, 0, -2, -1, 2], dtype=np.int32)):
        with pytest.raises(ValueError, match="labels"):
            fof.fof_groups(bad)
        with pytest.raises(ValueError, match="labels"):
            fof.fof_groups(torch.from_numpy(bad).to(cuda))
    off, mem = fof.fof_groups(np.array([0, 0, -1, 3, 3, 3], dtype=np.int32))
    assert off.tolist() == [0, 2, 5] and mem.tolist() == [0, 1, 3, 4, 5]
