"""Periodic friends-of-friends (opt-in ``boxsize``): groups that cross the box's faces.

The reference's FoF (fof.py:18-79) builds ``KDTree(data)`` without a box size; the periodic
option is what the same flood fill gives with ``KDTree(data, boxsize=L)``.  The oracle's
restatement takes that box size; a CPU test pins it against a brute-force nearest-image
union-find, and the GPU tests check ``halma_fof_periodic`` against it, bit for bit in the
partition, on clouds straddling faces, edges and corners and on a chain that wraps around.
"""
import numpy as np
import pytest

import oracle
from oracle import fof_kdtree

BOX, LL = 1.0, 0.01


def _periodic_cloud(seed, n_blob=600, n_bg=4000):
    rng = np.random.default_rng(seed)
    parts = []
    # blobs centred on a face, an edge and a corner, and one inside
    for c in ((0.0, 0.5, 0.5), (0.999, 0.0, 0.3), (0.0, 0.0, 0.0), (0.4, 0.6, 0.7)):
        parts.append(np.asarray(c) + rng.normal(0.0, 0.012, (n_blob, 3)))
    # a chain along x through the x = 0 face, steps of 0.8 LL
    t = np.arange(-20, 20) * 0.8 * LL
    parts.append(np.stack([t, np.full_like(t, 0.2), np.full_like(t, 0.8)], axis=1))
    parts.append(rng.uniform(0.0, BOX, (n_bg, 3)))
    p = np.mod(np.concatenate(parts), BOX)
    p[p >= BOX] = 0.0   # np.mod of a tiny negative value can round up to BOX
    return p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy()


def _brute_periodic_labels(x, y, z, ll, box):
    """Nearest-image pairs by brute force (image coordinate x +- box, then the same rounded
    distance as the non-periodic predicate), union-find, smallest index per component."""
    n = len(x)
    p = np.stack([x, y, z], axis=1)
    parent = np.arange(n)

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    shifts = np.array([[sx, sy, sz] for sx in (-box, 0.0, box) for sy in (-box, 0.0, box)
                       for sz in (-box, 0.0, box)])
    has = np.zeros(n, dtype=bool)
    for i in range(n):
        best = None
        for s in shifts:
            q = p + s
            d = q - p[i]
            d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
            best = d2 if best is None else np.minimum(best, d2)
        best[i] = np.inf
        for j in np.nonzero(best <= ll * ll)[0]:
            has[i] = has[j] = True
            a, b = find(i), find(int(j))
            if a != b:
                parent[max(a, b)] = min(a, b)
    lab = np.array([find(i) for i in range(n)], dtype=np.int32)
    lab[~has] = -1
    return lab


def test_oracle_periodic_flood_fill_matches_brute_force():
    x, y, z = _periodic_cloud(3, n_blob=150, n_bg=500)
    ref = _brute_periodic_labels(x, y, z, LL, BOX)
    groups = fof_kdtree.friends_of_friends_serial(x, y, z, LL, boxsize=BOX)
    assert np.array_equal(oracle.groups_to_labels(groups, len(x)), ref)
    # groups really cross the faces: the non-periodic partition differs
    flat = oracle.fof_labels(x, y, z, LL)
    assert not np.array_equal(flat, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [1, 2])
def test_gpu_periodic_matches_oracle(cuda, seed):
    from pyhalma_gb300 import fof
    x, y, z = _periodic_cloud(seed)
    ref = oracle.groups_to_labels(fof_kdtree.friends_of_friends_serial(x, y, z, LL, boxsize=BOX), len(x))
    lab = fof.fof_labels(x, y, z, LL, boxsize=BOX)
    assert np.array_equal(lab, ref)
    # the reference-signature wrapper with the box option returns the same groups
    groups = fof.friends_of_friends_serial(x, y, z, LL, boxsize=BOX)
    assert np.array_equal(oracle.groups_to_labels(groups, len(x)), ref)


@pytest.mark.gpu
def test_gpu_periodic_device_arrays_and_interior_data(cuda):
    import torch
    from pyhalma_gb300 import fof, synth
    # data far from every face: periodic and non-periodic partitions are the same
    s = synth.plummer_snapshot(50_000, 40, seed=4, box_mpc=1.0, contaminant_frac=0.0)
    keep = (np.minimum.reduce([s.x, s.y, s.z]) > 0.05) & (np.maximum.reduce([s.x, s.y, s.z]) < 0.95)
    x, y, z = s.x[keep], s.y[keep], s.z[keep]
    flat = fof.fof_labels(x, y, z, 0.0015)
    d = [torch.tensor(a, device=cuda) for a in (x, y, z)]
    per = fof.fof_labels(*d, 0.0015, boxsize=1.0).cpu().numpy()
    assert np.array_equal(per, flat)


@pytest.mark.gpu
def test_gpu_periodic_rejects_bad_boxes(cuda):
    from pyhalma_gb300 import fof
    x = np.array([0.1, 0.2, 1.5]); y = np.array([0.1, 0.2, 0.3]); z = np.array([0.5, 0.5, 0.5])
    with pytest.raises(ValueError):
        fof.fof_labels(x, y, z, 0.01, boxsize=1.0)      # a position outside [0, box)
    with pytest.raises(ValueError):
        fof.fof_labels(x[:2], y[:2], z[:2], 0.5, boxsize=1.0)   # box under 3 linking lengths
    assert fof.fof_labels(x[:0], y[:0], z[:0], 0.01, boxsize=1.0).shape == (0,)
