"""Phase-space cleaning (halo_properties.py:113-278 calc_cell / clean_cell and the main script's loop
pyHALMA.py:774-877): the oracle and the CUDA path against the reference's own block (golden
fixture made by exec'ing its source).

Compared exactly: the kept groups (members and order), num_particles, num_cells and the
which_cell arrays.  Centres, masses and furthest-particle radii are FP64 sums whose order is
unspecified in the reference (numba fastmath), compared at 1e-11 relative.
"""
import numpy as np
import pytest

import oracle.phase_space as ops

CASES = ("psc_on", "psc_q2", "psc_aggr", "psc_off")
RTOL = 1e-11


def _case(d, name):
    LL, Q, SIG, FLAG, MINP = d[name + "__params"]
    io, im = d[name + "__in_off"], d[name + "__in_mem"]
    groups = [im[io[g]:io[g + 1]] for g in range(len(io) - 1)]
    arrays = [d[name + "__" + k] for k in ("x", "y", "z", "vx", "vy", "vz", "m")]
    return groups, arrays, (float(LL), float(Q), float(SIG), bool(FLAG), int(MINP))


def _check(d, name, res):
    oo, om = d[name + "__out_off"], d[name + "__out_mem"]
    ref = [om[oo[g]:oo[g + 1]].tolist() for g in range(len(oo) - 1)]
    assert [list(map(int, g)) for g in res["new_groups"]] == ref
    for k in ("num_particles", "num_cells"):
        assert np.array_equal(np.asarray(res[k]), d[name + "__" + k]), k
    for k in ("center_x", "center_y", "center_z", "masses", "rmax"):
        np.testing.assert_allclose(np.asarray(res[k], dtype=np.float64), d[name + "__" + k], rtol=RTOL, atol=1e-15)
    for a in "xyz":
        wo, w = d[name + "__which_" + a + "_off"], d[name + "__which_" + a]
        assert [list(map(int, q)) for q in res["which_" + a]] == [w[wo[g]:wo[g + 1]].tolist() for g in range(len(wo) - 1)]


def test_fixture_comes_from_the_reference_block(golden):
    d = golden("psc.npz")
    assert d["block_lines"].tolist() == [774, 877]
    # the aggressive case removes most particles over several passes
    assert d["psc_aggr__num_particles"].sum() < 0.5 * (len(d["psc_aggr__in_mem"]))


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_block(golden, name):
    d = golden("psc.npz")
    groups, arrays, params = _case(d, name)
    _check(d, name, ops.phase_space_cleaning(groups, *arrays, *params))


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_reference_block(golden, cuda, name):
    from pyhalma_gb300 import phase_space
    d = golden("psc.npz")
    groups, arrays, params = _case(d, name)
    _check(d, name, phase_space.phase_space_cleaning(groups, *arrays, *params))


@pytest.mark.gpu
def test_gpu_matches_oracle_on_fof_groups(cuda):
    """FoF groups of a 200k-particle contaminated snapshot, cleaning on and aggressive."""
    from pyhalma_gb300 import fof, phase_space, synth
    s = synth.plummer_snapshot(200_000, 60, seed=41, box_mpc=2.0, contaminant_frac=0.15)
    groups = [g for g in fof.friends_of_friends_serial(s.x, s.y, s.z, 0.0015) if len(g) >= 50]
    arrays = (s.x, s.y, s.z, s.vx, s.vy, s.vz, s.mass)
    for params in ((0.0015, 1.0, 3.0, True, 50), (0.0015, 3.0, 1.0, True, 30)):
        got = phase_space.phase_space_cleaning(groups, *arrays, *params)
        ref = ops.phase_space_cleaning(groups, *arrays, *params)
        assert [g.tolist() for g in got["new_groups"]] == [g.tolist() for g in ref["new_groups"]]
        for k in ("num_particles", "num_cells"):
            assert list(got[k]) == list(ref[k])
        for k in ("which_x", "which_y", "which_z"):
            assert all(np.array_equal(a, b) for a, b in zip(got[k], ref[k]))
        for k in ("center_x", "masses", "rmax"):
            np.testing.assert_allclose(got[k], ref[k], rtol=RTOL, atol=1e-15)


@pytest.mark.gpu
def test_edge_groups(cuda):
    from pyhalma_gb300 import phase_space
    rng = np.random.default_rng(8)
    n = 500
    x, y, z = rng.normal(0, 0.002, (3, n))
    vx, vy, vz = rng.normal(0, 50, (3, n))
    m = np.ones(n)
    groups = [np.arange(0, 300), np.array([], dtype=np.int64), np.array([300]), np.arange(301, 340),
              np.arange(340, 500)]
    for flag in (True, False):
        got = phase_space.phase_space_cleaning(groups, x, y, z, vx, vy, vz, m, 0.0015, 1.0, 3.0, flag, 1)
        ref = ops.phase_space_cleaning(groups, x, y, z, vx, vy, vz, m, 0.0015, 1.0, 3.0, flag, 1)
        assert [g.tolist() for g in got["new_groups"]] == [g.tolist() for g in ref["new_groups"]]
        assert list(got["num_cells"]) == list(ref["num_cells"])
        for k in ("which_x", "which_y", "which_z"):
            assert all(np.array_equal(a, b) for a, b in zip(got[k], ref[k]))
    with pytest.raises(ValueError):
        phase_space.phase_space_cleaning([np.array([0, n])], x, y, z, vx, vy, vz, m, 0.0015, 1.0, 3.0, True, 1)


@pytest.mark.gpu
def test_groups_that_clean_away(cuda):
    """Q_FIL above every cell count drops every particle in the first sweep (remaining 0:
    empty final grid), and SIG_FIL 0 drops particles in later sweeps too; both paths against
    the oracle."""
    from pyhalma_gb300 import phase_space
    rng = np.random.default_rng(12)
    n = 3000
    x, y, z = rng.normal(0, 0.003, (3, n))
    vx, vy, vz = rng.normal(0, 80, (3, n))
    m = rng.uniform(0.5, 2.0, n)
    groups = [np.arange(0, 1200), np.arange(1200, 3000)]
    for q_fil, sig_fil in ((1e9, 3.0), (1.0, 0.0), (2.0, 0.3)):
        got = phase_space.phase_space_cleaning(groups, x, y, z, vx, vy, vz, m, 0.0015, q_fil, sig_fil, True, 1)
        ref = ops.phase_space_cleaning(groups, x, y, z, vx, vy, vz, m, 0.0015, q_fil, sig_fil, True, 1)
        assert [g.tolist() for g in got["new_groups"]] == [g.tolist() for g in ref["new_groups"]]
        assert list(got["num_particles"]) == list(ref["num_particles"])
        for k in ("which_x", "which_y", "which_z"):
            assert all(np.array_equal(a, b) for a, b in zip(got[k], ref[k]))


def _sequential(v):
    """The reference's loop: s = 0.0, then s += v[i] in order, each addition rounded."""
    with np.errstate(over="ignore", invalid="ignore"):     # the infinite and NaN cases are meant
        return float(np.add.accumulate(np.concatenate([[0.0], np.asarray(v, dtype=np.float64)]))[-1])


@pytest.mark.gpu
def test_sequential_sums_are_the_scalar_loop(cuda):
    """The building block of the per-cell sums against the scalar FP64 loop, bit for bit:
    sums that change sign, cancel to zero, cross binades, meet ties of half an ulp, hold
    subnormals, infinities and NaN; segments of 0 to 3000 values."""
    from pyhalma_gb300 import phase_space
    rng = np.random.default_rng(31)
    u = 2.0 ** -53
    segs = [np.zeros(0), np.array([-0.0]), np.array([1.0, -1.0]), np.array([5e-324, -5e-324, 5e-324]),
            np.array([1e308, 1e308, -1e308]), np.array([1.0, np.inf, -np.inf]), np.array([np.nan, 1.0]),
            np.concatenate([[1.0], rng.integers(-8, 9, 3000) * u]),
            np.concatenate([[1e300, -1e300], rng.normal(0, 1, 500)])]
    for kind in range(40):
        n = int(rng.integers(1, 3000))
        if kind % 5 == 0:
            v = rng.normal(0, 1, n)
        elif kind % 5 == 1:
            v = rng.normal(250, 60, n) * rng.uniform(1e5, 1e7, n)            # mass x velocity
        elif kind % 5 == 2:
            v = rng.normal(0, 1, n) * np.exp(rng.uniform(-30, 30, n))
        elif kind % 5 == 3:
            v = np.full(n, 0.1) * np.where(rng.random(n) < 0.4, -1.0, 1.0)
        else:
            h = rng.normal(0, 1, n // 2)
            v = np.concatenate([h, -h[::-1], [0.0]])
        segs.append(v)
    off = np.zeros(len(segs) + 1, dtype=np.int64)
    np.cumsum([len(s) for s in segs], out=off[1:])
    vals = np.concatenate(segs)
    got = phase_space.sequential_sums(vals, off)
    want = np.array([_sequential(s) for s in segs])
    assert np.array_equal(got, want, equal_nan=True)
    num = ~np.isnan(want)                     # signed zeros agree too (a NaN's sign bit is not defined)
    assert np.array_equal(np.signbit(got[num]), np.signbit(want[num]))
    import torch
    T = lambda a: torch.from_numpy(a).to(cuda)
    assert np.array_equal(phase_space.sequential_sums(T(vals), T(off)).cpu().numpy(), want, equal_nan=True)
