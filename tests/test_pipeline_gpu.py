"""One-call snapshot pipeline (FoF -> groups >= minp -> batched unbinding) against the
oracle composition on the 1e5-particle Plummer snapshot.

FoF labels and groups are compared exactly; the unbinding stage must give exactly what
unbind_batched gives on the gathered groups (whose every pass is checked against the FP64
oracle in test_unbind_gpu.py); against the oracle's own FP64 iteration a handful of
particles may differ.
"""
import numpy as np
import pytest

import oracle
from oracle.unbind import unbind_halo
from pyhalma_gb300 import synth
from pyhalma_gb300.unbinding import UnbindOptions, find_haloes, unbind_batched

pytestmark = pytest.mark.gpu


def test_find_haloes_matches_oracle_composition(cuda):
    s = synth.plummer_snapshot(100_000, 50, seed=0, box_mpc=10.0, contaminant_frac=0.15)
    cat = find_haloes(s.x, s.y, s.z, s.vx, s.vy, s.vz, s.mass, 0.0015, minp=50,
                      options=UnbindOptions(eps=1e-4, max_iter=50))
    lab = oracle.fof_labels(s.x, s.y, s.z, 0.0015)
    assert np.array_equal(cat.labels, lab)
    groups = [g for g in oracle.labels_to_groups(lab) if len(g) >= 50]
    assert cat.n_haloes == len(groups)
    expect = np.zeros(s.n, dtype=np.uint8)
    for h, g in enumerate(groups):
        g = np.array(g)
        assert np.array_equal(cat.members[cat.offsets[h]:cat.offsets[h + 1]], g)
        b, _ = unbind_halo(s.x[g], s.y[g], s.z[g], s.vx[g], s.vy[g], s.vz[g], s.mass[g], eps=1e-4, max_iter=50)
        expect[g] = b
    mem = cat.members
    bound, halo, _ = unbind_batched(cat.offsets, *(np.ascontiguousarray(a[mem]) for a in
                                                   (s.x, s.y, s.z, s.vx, s.vy, s.vz, s.mass)),
                                    UnbindOptions(eps=1e-4, max_iter=50))
    assert np.array_equal(cat.bound[mem], bound)
    assert np.array_equal(cat.haloes, halo)
    outside = np.ones(s.n, dtype=bool)
    outside[mem] = False
    assert not cat.bound[outside].any()
    assert (cat.bound != expect).sum() <= 5
    assert cat.haloes.shape == (cat.n_haloes, 11)
