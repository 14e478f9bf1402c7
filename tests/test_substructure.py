"""Substructure identification (pyHALMA.py:703-766): the batched sub-FoF and the bridge
splitting against the reference's own block (golden fixtures made by exec'ing its source)
and against the oracle's group-by-group restatement.

CPU tests pin the oracle to the fixtures; GPU tests check the CUDA path bit for bit: the
segmented FoF against one oracle FoF per segment, and the whole block's output groups (and
``counter_sub``) against the reference's.
"""
import numpy as np
import pytest

import oracle
from oracle.substructure import identify_substructure as oracle_identify
from pyhalma_gb300 import synth

CASES = ("one_level", "three_levels", "dec1p5")


def _case(d, name):
    LL, MINP_SUB, DEC, MIN_LL, DF, MINP = d[name + "__params"]
    io, im = d[name + "__in_off"], d[name + "__in_mem"]
    oo, om = d[name + "__out_off"], d[name + "__out_mem"]
    groups = [im[io[g]:io[g + 1]].tolist() for g in range(len(io) - 1)]
    ref = [om[oo[g]:oo[g + 1]].tolist() for g in range(len(oo) - 1)]
    xyzm = tuple(d[name + k] for k in ("__x", "__y", "__z", "__m"))
    params = (float(LL), int(MINP_SUB), float(DEC), float(MIN_LL), float(DF), int(MINP))
    return groups, xyzm, params, ref, int(d[name + "__counter_sub"])


def test_fixture_comes_from_the_reference_block(golden):
    d = golden("substructure.npz")
    assert d["block_lines"].tolist() == [703, 766]
    for name in CASES:
        groups, _, _, ref, cut = _case(d, name)
        assert cut > 0 and len(ref) > 0, name      # every case cuts bridges


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_block(golden, name):
    groups, (x, y, z, m), params, ref, cut = _case(golden("substructure.npz"), name)
    out, n_cut = oracle_identify(groups, x, y, z, m, *params)
    assert out == ref
    assert n_cut == cut


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_reference_block(golden, cuda, name):
    from pyhalma_gb300 import substructure
    groups, (x, y, z, m), params, ref, cut = _case(golden("substructure.npz"), name)
    out, n_cut = substructure.identify_substructure(groups, x, y, z, m, *params)
    assert [list(g) for g in out] == ref
    assert n_cut == cut


@pytest.mark.gpu
def test_segmented_fof_matches_per_segment_oracle(cuda):
    """Random index lists over one snapshot, including empty, single-particle and repeated
    (spatially identical) segments: each segment's labels equal a separate FoF of its rows."""
    from pyhalma_gb300 import substructure
    s = synth.plummer_snapshot(60_000, 20, seed=6, box_mpc=1.0)
    rng = np.random.default_rng(3)
    lists = []
    for k in range(40):
        size = int(rng.choice([0, 1, 2, 50, 400, 3000, 12_000]))
        lists.append(np.sort(rng.choice(s.n, size, replace=False)))
    lists.append(lists[5].copy())            # the same particles again: must not link across
    lists.append(lists[5].copy())
    ll = 0.00075
    got = substructure.sub_friends_of_friends(s.x, s.y, s.z, lists, ll)
    for k, pl in enumerate(lists):
        lab = oracle.fof_labels(s.x[pl], s.y[pl], s.z[pl], ll)
        assert got[k] == oracle.labels_to_groups(lab), k


@pytest.mark.gpu
def test_segmented_fof_labels_and_device_tensors(cuda):
    import torch
    from pyhalma_gb300 import substructure
    s = synth.bridged_snapshot(6, 3, seed=9, box_mpc=1.0, n_hi=2000)
    lab_all = oracle.fof_labels(s.x, s.y, s.z, 0.0015)
    groups = [g for g in oracle.labels_to_groups(lab_all) if len(g) >= 50]
    off = np.concatenate(([0], np.cumsum([len(g) for g in groups]))).astype(np.int64)
    mem = np.concatenate(groups)
    gx, gy, gz = (np.ascontiguousarray(a[mem]) for a in (s.x, s.y, s.z))
    ref = np.full(len(mem), -1, dtype=np.int32)
    for g in range(len(groups)):
        lab = oracle.fof_labels(gx[off[g]:off[g + 1]], gy[off[g]:off[g + 1]], gz[off[g]:off[g + 1]], 0.00075)
        ref[off[g]:off[g + 1]] = np.where(lab >= 0, lab + off[g], -1)
    host = substructure.fof_segmented_labels(gx, gy, gz, off, 0.00075)
    assert np.array_equal(host, ref)
    dev = substructure.fof_segmented_labels(*(torch.from_numpy(a).to(cuda) for a in (gx, gy, gz, off)), 0.00075)
    assert dev.is_cuda and np.array_equal(dev.cpu().numpy(), ref)


@pytest.mark.gpu
def test_bridged_snapshot_against_oracle(cuda):
    """A larger bridged snapshot end to end: GPU FoF groups -> GPU bridge splitting, against
    the oracle's group-by-group restatement on the same groups."""
    from pyhalma_gb300 import fof, substructure
    s = synth.bridged_snapshot(60, 60, seed=11, box_mpc=3.0)
    groups = [g for g in fof.friends_of_friends_serial(s.x, s.y, s.z, 0.0015) if len(g) >= 50]
    for params in ((0.0015, 25, 2.0, 0.0005, 0.75, 50), (0.0015, 10, 2.0, 0.0001, 0.5, 20)):
        out, cut = substructure.identify_substructure(groups, s.x, s.y, s.z, s.mass, *params)
        ref, rcut = oracle_identify(groups, s.x, s.y, s.z, s.mass, *params)
        assert cut == rcut and cut > 0
        assert [list(g) for g in out] == ref


@pytest.mark.gpu
def test_edge_cases(cuda):
    from pyhalma_gb300 import substructure
    x = np.linspace(0, 1, 100)
    y = np.zeros(100)
    # no groups, no levels (MIN_LL above LL/DEC), empty groups in the input
    out, cut = substructure.identify_substructure([], x, y, y, np.ones(100), 0.0015, 25, 2.0, 0.0005, 0.75, 50)
    assert len(out) == 0 and cut == 0
    g = [list(range(0, 60)), [], list(range(60, 100))]
    out, cut = substructure.identify_substructure(g, x, y, y, np.ones(100), 0.0015, 25, 2.0, 0.01, 0.75, 30)
    assert [list(a) for a in out] == [list(range(0, 60)), list(range(60, 100))] and cut == 0
    with pytest.raises(ValueError):
        substructure.identify_substructure([[3, 2, 1]], x, y, y, np.ones(100), 0.0015, 25, 2.0, 0.0005, 0.75, 1)
    with pytest.raises(ValueError):
        substructure.fof_segmented_labels(x, y, y, np.array([0, 50], dtype=np.int64), 0.001)   # does not cover n
