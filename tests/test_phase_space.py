"""Phase-space cleaning (halo_properties.py:113-278 calc_cell / clean_cell and the driver loop
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
