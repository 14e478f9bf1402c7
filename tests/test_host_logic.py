"""Host-side logic on the CPU: synthetic generators, group ordering helpers, and the RPS /
most-bound host code checked against the reference's outputs with the oracle potential
standing in for the GPU kernel."""
import numpy as np
import pytest

import oracle
from pyhalma_gb300 import halo_gas, synth


def test_plummer_snapshot_counts_and_units():
    s = synth.plummer_snapshot(20_000, 10, seed=3, box_mpc=10.0, contaminant_frac=0.15)
    assert s.n == 20_000
    assert (s.sphere == -1).sum() == 2000
    assert np.abs(s.x).max() <= 5.0
    share = s.contaminant[s.sphere >= 0].mean()
    assert 0.13 < share < 0.17


def test_powerlaw_counts_distribution():
    rng = np.random.default_rng(0)
    n = synth.powerlaw_counts(rng, 200_000, alpha=1.0, n_min=50, n_max=200_000)
    assert n.min() >= 50 and n.max() <= 200_000
    # dN/dlogN ~ N^-1 -> mean = (n_min^-1 ... ) ~ 415 for [50, 2e5]
    assert 380 < n.mean() < 450
    flat = synth.powerlaw_counts(rng, 200_000, alpha=0.0, n_min=50, n_max=200_000)
    assert flat.mean() > 10 * n.mean()


def test_labels_groups_roundtrip():
    lab = np.array([-1, 1, 1, 3, -1, 3, 1], dtype=np.int32)
    groups = oracle.labels_to_groups(lab)
    assert groups == [[1, 2, 6], [3, 5]]
    assert np.array_equal(oracle.groups_to_labels(groups, 7), lab)


def test_good_groups():
    from pyhalma_gb300.fof import good_groups
    assert good_groups([[1, 2], [3], [4, 5, 6]], 2).tolist() == [True, False, True]


@pytest.fixture
def oracle_potential(monkeypatch):
    # host logic only: the GPU call is replaced by the oracle's float32 restatement
    def fake(total_mass, total_x, total_y, total_z, test_x, test_y, test_z, mode=None, eps2=0.0):
        return oracle.bf_potential_f32(total_mass, total_x, total_y, total_z, test_x, test_y, test_z)
    monkeypatch.setattr(halo_gas, "bf_potential", fake)


def test_rps_and_most_bound_host_logic_match_reference(golden, oracle_potential):
    d = golden("rps.npz")
    for k in range(int(d["ncase"])):
        g = lambda n: d[f"c{k}_{n}"]
        lim, mass_dm_part = g("params")
        gas = [g(n) for n in ("gx", "gy", "gz", "gvx", "gvy", "gvz", "gm", "gt")]
        for nspec in (1, 2):
            np.random.seed(1234 + k)
            out = halo_gas.RPS(*gas, g("dx"), g("dy"), g("dz"), g("dm"), g("sx"), g("sy"), g("sz"), g("sm"),
                               *g("bulk"), int(lim), mass_dm_part, nspec)
            assert np.array_equal(np.array(out, dtype=np.float64), g(f"rps{nspec}")), (k, nspec)
        np.random.seed(999 + k)
        mb = halo_gas.most_bound_particle(gas[0], gas[1], gas[2], gas[6], g("dx"), g("dy"), g("dz"), g("dm"),
                                          g("sx"), g("sy"), g("sz"), g("sm"), g("oripa"), int(lim), mass_dm_part)
        assert np.array_equal(np.array(mb, dtype=np.float64), g("mb")), k
