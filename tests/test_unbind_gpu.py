"""Batched unbinding parity against the FP64 oracle (oracle/unbind.py).

The iterative cut repeats the reference's single pass (halo_properties.py:282-361), so it
is checked pass by pass: the GPU's bound set after k-1 passes is the input of an FP64 oracle
pass, and the GPU's pass k must agree with it.  Tolerances written here:
* potential: |phi_gpu / phi_fp64 - 1| <= RTOL_PHI = 1e-6 for every particle a pass
  evaluates and keeps (the potential is returned for those; FP32-compensated path);
* membership: the GPU's pass may keep or remove a particle against the FP64 pass only if
  that particle's FP64 energy lies within BAND = 2e-6 * (E_kin + G*phi) of zero (the 1e-6
  potential bound with a factor-2 margin);
* halo table after every pass: FP64 mass / centre / bulk velocity of the GPU's bound set at
  1e-12 relative.
No halo is skipped: a pass that keeps or removes a particle within the band still has its
potential, its other particles and its halo row checked.
"""
import numpy as np
import pytest

from oracle.unbind import unbind_halo, unbind_pass
from pyhalma_gb300 import synth
from pyhalma_gb300.unbinding import G_MPC, UnbindOptions, unbind_batched

pytestmark = pytest.mark.gpu
RTOL_PHI = 1e-6
BAND = 2e-6
EPS = 1e-4


@pytest.fixture(scope="module")
def catalogue():
    return synth.powerlaw_catalogue(80, seed=3, n_min=50, n_max=6000, contaminant_frac=0.15, alpha=0.6)


def _arrays(cat):
    return cat.offsets, cat.x, cat.y, cat.z, cat.vx, cat.vy, cat.vz, cat.mass


def _check_halo_rows(cat, bound, halo):
    for h in range(cat.n_haloes):
        sl = slice(cat.offsets[h], cat.offsets[h + 1])
        b = bound[sl].astype(bool)
        row = halo[h]
        assert row[7] == b.sum(), h
        if not b.any():
            continue
        m = cat.mass[sl][b]
        M = m.sum()
        assert abs(row[0] / M - 1) < 1e-12, h
        for k, a in ((1, cat.x), (2, cat.y), (3, cat.z), (4, cat.vx), (5, cat.vy), (6, cat.vz)):
            ref = (m * a[sl][b]).sum() / M
            assert abs(row[k] - ref) <= 1e-12 * max(1.0, abs(ref)), (h, k)


def _check_pass_contract(cat, rtol_phi, band, **opt):
    """Runs the GPU with max_iter = 1, 2, ... until every halo has converged and checks each
    pass against one FP64 oracle pass on the GPU's own input set.  Returns the number of
    particles kept or removed against the FP64 pass (all inside the band)."""
    n = cat.n
    prev = np.ones(n, dtype=bool)
    flips = 0
    for k in range(1, 51):
        bound, halo, phi = unbind_batched(*_arrays(cat), UnbindOptions(eps=EPS, max_iter=k, **opt), want_phi=True)
        bound = bound.astype(bool)
        assert not (bound & ~prev).any(), "a removed particle came back"
        for h in range(cat.n_haloes):
            sl = slice(cat.offsets[h], cat.offsets[h + 1])
            s = prev[sl]
            if not s.any():
                continue
            sel = lambda a: a[sl][s]
            p_ref, ek, e = unbind_pass(sel(cat.x), sel(cat.y), sel(cat.z), sel(cat.vx), sel(cat.vy), sel(cat.vz),
                                       sel(cat.mass), eps=EPS)
            keep_gpu, keep_ref = bound[sl][s], e <= 0.0
            if halo[h, 8] >= k and keep_gpu.any():
                # the halo ran pass k: the potential returned for the particles it kept is the
                # one that pass evaluated (the removed ones get none)
                p = phi[sl][s][keep_gpu]
                assert np.max(np.abs(p / p_ref[keep_gpu] - 1.0)) <= rtol_phi, (k, h)
            diff = keep_gpu != keep_ref
            if diff.any():
                scale = np.abs(e) / (ek + G_MPC * np.abs(p_ref))
                assert np.all(scale[diff] <= band), (k, h, scale[diff])
                flips += int(diff.sum())
        _check_halo_rows(cat, bound, halo)
        if np.array_equal(bound, prev) and halo[:, 8].max() < k:
            break
        prev = bound
    return flips


def test_fp32c_matches_fp64_oracle(catalogue, cuda):
    flips = _check_pass_contract(catalogue, RTOL_PHI, BAND)
    assert flips <= 5
    bound, halo, phi = unbind_batched(*_arrays(catalogue), UnbindOptions(eps=EPS, max_iter=50), want_phi=True)
    assert not bound[catalogue.contaminant].any()
    # end to end against the oracle's own iteration: a handful of particles at most differ
    diff = 0
    for h in range(catalogue.n_haloes):
        sl = slice(catalogue.offsets[h], catalogue.offsets[h + 1])
        b_ref, _ = unbind_halo(catalogue.x[sl], catalogue.y[sl], catalogue.z[sl], catalogue.vx[sl],
                               catalogue.vy[sl], catalogue.vz[sl], catalogue.mass[sl], eps=EPS, max_iter=50)
        diff += int((bound[sl].astype(bool) != b_ref).sum())
    assert diff <= 5


def test_full_recompute_matches_fp64_oracle(catalogue, cuda):
    # every pass recomputes the full potential (no subtraction of the removed particles)
    assert _check_pass_contract(catalogue, RTOL_PHI, BAND, incremental=False) <= 5


def test_incremental_equals_full_recompute(catalogue, cuda):
    inc = unbind_batched(*_arrays(catalogue), UnbindOptions(eps=EPS, max_iter=50), want_phi=True)
    full = unbind_batched(*_arrays(catalogue), UnbindOptions(eps=EPS, max_iter=50, incremental=False), want_phi=True)
    assert (inc[0] != full[0]).sum() <= 2
    both = (inc[0] == 1) & (full[0] == 1)
    # each is within RTOL_PHI of FP64 (checked above); against each other likewise
    assert np.max(np.abs(inc[2][both] / full[2][both] - 1.0)) < RTOL_PHI


def test_fp64_path_matches_oracle(catalogue, cuda):
    assert _check_pass_contract(catalogue, 1e-12, 0.0, precision="fp64") == 0


def test_graph_replay_is_identical_and_deterministic(catalogue, cuda):
    a = unbind_batched(*_arrays(catalogue), UnbindOptions(eps=EPS, max_iter=12, use_graph=True), want_phi=True)
    b = unbind_batched(*_arrays(catalogue), UnbindOptions(eps=EPS, max_iter=12, use_graph=False), want_phi=True)
    c = unbind_batched(*_arrays(catalogue), UnbindOptions(eps=EPS, max_iter=12, use_graph=True), want_phi=True)
    for x, y in ((a, b), (a, c)):
        assert np.array_equal(x[0], y[0])
        assert np.array_equal(x[1], y[1])
        assert np.array_equal(x[2], y[2])


def test_tile_shapes_give_identical_results(catalogue, cuda):
    # every tile shape sums each target's sources in the same chunk order: bit-identical
    from pyhalma_gb300 import autotune
    saved = autotune.get_table()
    try:
        out = []
        for t in (1, 2, 4):
            autotune.set_table([2 ** 31 - 1], [t], 1 << 20)
            out.append(unbind_batched(*_arrays(catalogue), UnbindOptions(eps=EPS, max_iter=50), want_phi=True))
        for o in out[1:]:
            assert np.array_equal(o[0], out[0][0])
            assert np.array_equal(o[2], out[0][2])
        # source slices change the summation grouping only: same membership, phi within 1e-7
        autotune.set_table([2 ** 31 - 1], [4], 256)
        b, h, p = unbind_batched(*_arrays(catalogue), UnbindOptions(eps=EPS, max_iter=50), want_phi=True)
        assert (b != out[0][0]).sum() <= 2
        same = (b == 1) & (out[0][0] == 1)
        assert np.max(np.abs(p[same] / out[0][2][same] - 1)) < 1e-7
    finally:
        autotune.set_table(*saved)


def test_iteration_cap_and_pass_count(catalogue, cuda):
    bound1, halo1, _ = unbind_batched(*_arrays(catalogue), UnbindOptions(eps=EPS, max_iter=1))
    assert np.all(halo1[:, 8] == 1)
    bound, halo, _ = unbind_batched(*_arrays(catalogue), UnbindOptions(eps=EPS, max_iter=50))
    assert halo[:, 8].max() >= 2
    # one pass removes a subset of what the converged cut removes
    assert np.all(bound <= bound1)


def test_edge_cases(cuda):
    # empty haloes and single-particle haloes
    off = np.array([0, 0, 1, 3], dtype=np.int64)
    x = np.array([0.0, 1.0, 1.0001])
    v = np.zeros(3)
    m = np.full(3, 1e8)
    bound, halo, phi = unbind_batched(off, x, v, v, v, v, v, m, UnbindOptions(eps=EPS), want_phi=True)
    assert bound.tolist() == [1, 1, 1]     # at rest: every particle is bound (E = -G phi <= 0)
    assert halo[0, 7] == 0 and halo[1, 7] == 1 and halo[2, 7] == 2
    assert phi[0] == 0.0
    assert abs(phi[1] / (1e8 / np.sqrt(1e-8 + EPS ** 2)) - 1) < 1e-6
    # no haloes at all
    b2, h2, _ = unbind_batched(np.array([0], dtype=np.int64), np.zeros(0), *[np.zeros(0)] * 6)
    assert b2.shape == (0,) and h2.shape[0] == 0


def test_device_tensors(catalogue, cuda):
    import torch
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    bound_d, halo_d, _ = unbind_batched(*[t(a) for a in _arrays(catalogue)], UnbindOptions(eps=EPS, max_iter=50))
    bound_h, halo_h, _ = unbind_batched(*_arrays(catalogue), UnbindOptions(eps=EPS, max_iter=50))
    assert np.array_equal(bound_d.cpu().numpy(), bound_h)
    assert np.array_equal(halo_d.cpu().numpy(), halo_h)
