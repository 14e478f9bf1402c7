"""Bounded device-side loops run out cleanly.

Every union-find loop of the FoF kernels and the pass loop of phase-space cleaning carry an
iteration bound; reaching it returns HALMA_ERR_NOT_CONVERGED instead of spinning.  These tests
make each bound run out on purpose (a host-set cap, no GPU fault involved) and then check that
the device is still usable: the next call with the default bound returns the oracle's answer.
"""
import numpy as np
import pytest

import oracle
from pyhalma_gb300 import _lib

pytestmark = pytest.mark.gpu


def _chain(n=5000, step=0.0009):
    # particles 0.6 LL apart along a slightly wobbling line: one long component
    t = np.arange(n, dtype=np.float64)
    x = 0.31 + step * t
    y = -0.2 + 1e-5 * np.sin(t)
    z = 0.05 + 1e-5 * np.cos(t)
    return x, y, z


def test_union_find_cap_returns_not_converged(cuda):
    from pyhalma_gb300 import fof
    x, y, z = _chain()
    ll = 0.0015
    L = _lib.lib()
    try:
        # cap 0: the first step of any find walk (every non-root particle takes one) trips it
        assert L.halma_set_union_find_cap(0) == _lib.OK
        with pytest.raises(_lib.HalmaError) as e:
            fof.fof_labels(x, y, z, ll)
        assert e.value.status == _lib.ERR_NOT_CONVERGED
        assert b"union-find" in L.halma_last_error()
    finally:
        L.halma_set_union_find_cap(-1)
    lab = fof.fof_labels(x, y, z, ll)
    assert np.array_equal(lab, oracle.fof_labels(x, y, z, ll))
    assert (lab == 0).all()


def test_cleaning_pass_cap_returns_not_converged(golden, cuda):
    from pyhalma_gb300 import phase_space
    d = golden("psc.npz")
    name = "psc_aggr"   # four sweeps per group
    LL, Q, SIG, FLAG, MINP = d[name + "__params"]
    io, im = d[name + "__in_off"], d[name + "__in_mem"]
    arrays = [d[name + "__" + k] for k in ("x", "y", "z", "vx", "vy", "vz", "m")]
    with pytest.raises(_lib.HalmaError) as e:
        phase_space.clean_groups(io, im, *arrays, float(LL), float(Q), float(SIG), bool(FLAG), int(MINP),
                                 max_passes=1)
    assert e.value.status == _lib.ERR_NOT_CONVERGED
    # the same call with the default bound completes and keeps the reference's groups
    ctl, _, _, table = phase_space.clean_groups(io, im, *arrays, float(LL), float(Q), float(SIG), bool(FLAG),
                                                int(MINP))
    assert table[:, _lib.PSC_FIELDS.index("passes")].max() >= 3
