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


def test_find_haloes_device_arrays_and_capacity(cuda):
    """The one-call path from device arrays gives what it gives from host arrays (where the
    first pass starts before the velocities have arrived, and a second call replays the
    captured passes with their wait on the velocities); through the C ABI, a halo capacity
    below the groups found returns HALMA_ERR_CAPACITY with the count set and the labels and
    bound flags filled (the early label copy is not started then)."""
    import ctypes
    import torch
    from pyhalma_gb300 import _lib
    s = synth.plummer_snapshot(60_000, 30, seed=7, box_mpc=10.0, contaminant_frac=0.15)
    cols = (s.x, s.y, s.z, s.vx, s.vy, s.vz, s.mass)
    opt = UnbindOptions(eps=1e-4, max_iter=50)
    host = find_haloes(*cols, 0.0015, minp=50, options=opt)
    dev = find_haloes(*(torch.tensor(a, device=cuda) for a in cols), 0.0015, minp=50, options=opt)
    assert np.array_equal(dev.labels.cpu().numpy(), host.labels)
    assert np.array_equal(dev.bound.cpu().numpy(), host.bound)
    assert np.array_equal(dev.offsets.cpu().numpy(), host.offsets)
    assert np.array_equal(dev.members.cpu().numpy(), host.members)
    assert np.array_equal(dev.haloes.cpu().numpy(), host.haloes)
    assert host.n_haloes >= 2
    again = find_haloes(*cols, 0.0015, minp=50, options=opt)
    assert np.array_equal(again.bound, host.bound)
    assert np.array_equal(again.haloes, host.haloes)
    n = s.n
    labels = np.empty(n, dtype=np.int32)
    bound = np.empty(n, dtype=np.uint8)
    offsets = np.empty(2, dtype=np.int64)
    members = np.empty(n, dtype=np.int32)
    table = np.empty((1, len(_lib.UB_FIELDS)), dtype=np.float64)
    nh = ctypes.c_int64(0)
    p = opt.params()
    st = _lib.lib().halma_find_haloes(n, *[_lib.ptr(np.ascontiguousarray(a)) for a in cols], 0.0015, 50,
                                      ctypes.byref(p), _lib.ptr(labels), _lib.ptr(bound), ctypes.byref(nh), 1,
                                      _lib.ptr(offsets), _lib.ptr(members), _lib.ptr(table), None)
    assert st == _lib.ERR_CAPACITY
    assert nh.value == host.n_haloes
    assert np.array_equal(labels, host.labels)
    assert np.array_equal(bound, host.bound)
