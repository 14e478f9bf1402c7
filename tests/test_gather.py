"""Ball gather (halo_gas.py:218-277): the CUDA range queries against the reference's own
st_gas_dm_particles_inside (golden fixture, KD-tree order) and the oracle's brute force.

The reference returns the DM and star selections in KD-tree traversal order; the GPU returns
the same particles in ascending index order, so those are compared as sets (sorted by
position).  The gas selection keeps the input order in both and is compared element by
element.  Every comparison is exact.
"""
import numpy as np
import pytest

import oracle.gather as og
from pyhalma_gb300 import synth


def _case(d, k):
    gas = [d[f"c{k}_gas{q}"] for q in range(8)]
    dm = [d[f"c{k}_dm{q}"] for q in range(4)]
    st = [d[f"c{k}_st{q}"] for q in range(10)]
    return gas, dm, st, d[f"c{k}_centre"]


def _rows(*arrays):
    a = np.stack([np.asarray(x, dtype=np.float64) for x in arrays], 1)
    return a[np.lexsort(a.T[::-1])]


def test_oracle_matches_reference_selection(golden):
    d = golden("ball.npz")
    for k in range(int(d["ncase"])):
        gas, dm, st, c = _case(d, k)
        for j in range(2):
            R = float(d[f"c{k}r{j}_R"])
            out = [d[f"c{k}r{j}_out{q}"] for q in range(17)]
            m = og.parallel_inside(gas[0], gas[1], gas[2], R, *c)
            assert np.array_equal(gas[0][m], out[0]) and np.array_equal(gas[7][m], out[7])
            assert np.array_equal(gas[6][m] * float(d["rete"]) ** 3, out[6])
            sel = og.query_ball_point(dm[0], dm[1], dm[2], c, R)
            assert np.array_equal(_rows(dm[0][sel], dm[1][sel], dm[2][sel], dm[3][sel]), _rows(*out[8:12]))
            sel = og.query_ball_point(st[0], st[1], st[2], c, R)
            assert np.array_equal(np.sort(st[9][sel]), np.sort(out[16]))
            assert len(sel) > 100


@pytest.mark.gpu
def test_gpu_matches_reference_function(golden, cuda):
    from pyhalma_gb300 import halo_gas
    d = golden("ball.npz")
    for k in range(int(d["ncase"])):
        gas, dm, st, c = _case(d, k)
        for j in range(2):
            R = float(d[f"c{k}r{j}_R"])
            ref = [d[f"c{k}r{j}_out{q}"] for q in range(17)]
            got = halo_gas.st_gas_dm_particles_inside(float(d["rete"]), 40.0, 128, None, gas, dm, st, None, None,
                                                      c[0], c[1], c[2], R, 1.0)
            for q in range(8):                       # gas: same order
                assert np.array_equal(got[q], ref[q]), (k, j, q)
            assert np.array_equal(_rows(*got[8:12]), _rows(*ref[8:12]))
            assert np.array_equal(_rows(*got[12:17]), _rows(*ref[12:17]))


@pytest.mark.gpu
def test_batched_spheres_match_oracle(cuda):
    from pyhalma_gb300 import halo_gas
    s = synth.plummer_snapshot(300_000, 40, seed=12, box_mpc=2.0)
    rng = np.random.default_rng(4)
    k = 500
    pick = rng.integers(0, s.n, k)
    cx, cy, cz = (a[pick] + rng.normal(0, 2e-3, k) for a in (s.x, s.y, s.z))
    R = np.exp(rng.uniform(np.log(1e-4), np.log(3e-2), k))
    R[:5] = 0.0                                        # zero radius: coincident points only
    cx[5:10] += 10.0                                   # spheres outside the particles' box
    R[10] = 5.0                                        # one sphere holding every particle
    for strict in (False, True):
        off, idx = halo_gas.balls_inside(s.x, s.y, s.z, cx, cy, cz, R, strict=strict)
        assert off[0] == 0 and len(idx) == off[-1]
        for b in range(k):
            got = idx[off[b]:off[b + 1]]
            if strict:
                ref = np.nonzero(og.parallel_inside(s.x, s.y, s.z, R[b], cx[b], cy[b], cz[b]))[0]
            else:
                ref = og.query_ball_point(s.x, s.y, s.z, (cx[b], cy[b], cz[b]), R[b])
            assert np.array_equal(got, ref), (strict, b)
        assert off[11] - off[10] == (s.n if not strict else off[11] - off[10])


@pytest.mark.gpu
def test_boundary_points_and_device_tensors(cuda):
    """Points at distance R from the centre, nudged by a few ulps, inside a denser cloud."""
    import torch
    from pyhalma_gb300 import halo_gas
    rng = np.random.default_rng(21)
    c = np.array([3.7, -1.2, 0.4])
    R = 0.0035
    d = rng.normal(size=(20000, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    p = c + d * R
    for q in range(3):
        p[:, q] = np.where(rng.random(len(p)) < 0.3, np.nextafter(p[:, q], np.inf), p[:, q])
        p[:, q] = np.where(rng.random(len(p)) < 0.3, np.nextafter(p[:, q], -np.inf), p[:, q])
    pts = np.concatenate([p, c + rng.normal(0, R, (30000, 3))])
    x, y, z = (np.ascontiguousarray(pts[:, q]) for q in range(3))
    got = halo_gas.query_ball_point(x, y, z, c, R)
    ref = og.query_ball_point(x, y, z, c, R)
    assert np.array_equal(got, ref)
    assert 0 < np.count_nonzero(np.isin(ref, np.arange(20000))) < 20000   # the boundary is cut
    assert np.array_equal(halo_gas.parallel_inside(x, y, z, R, *c), og.parallel_inside(x, y, z, R, *c))
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    off, idx = halo_gas.balls_inside(T(x), T(y), T(z), T([c[0]]), T([c[1]]), T([c[2]]), T([R]))
    assert idx.is_cuda and np.array_equal(idx.cpu().numpy(), ref)


@pytest.mark.gpu
def test_empty_inputs(cuda):
    from pyhalma_gb300 import halo_gas
    e = np.zeros(0)
    off, idx = halo_gas.balls_inside(e, e, e, [0.0], [0.0], [0.0], [1.0])
    assert off.tolist() == [0, 0] and len(idx) == 0
    off, idx = halo_gas.balls_inside(np.ones(3), np.ones(3), np.ones(3), e, e, e, e)
    assert off.tolist() == [0] and len(idx) == 0
    with pytest.raises(ValueError):
        halo_gas.balls_inside(np.ones(3), np.ones(3), np.ones(3), [0.0], [0.0], [0.0], [-1.0])
    with pytest.raises(ValueError):
        halo_gas.balls_inside(np.ones(3), np.ones(3), np.ones(3), [np.nan], [0.0], [0.0], [1.0])


@pytest.mark.gpu
def test_duplicates_and_zero_radius(cuda):
    """Repeated points and a zero radius centred on a particle: every copy of that particle is
    inside (d^2 = 0 <= 0), nothing else; strict mode keeps nothing at R = 0."""
    from pyhalma_gb300 import halo_gas
    rng = np.random.default_rng(5)
    base = rng.uniform(0, 0.01, (2000, 3))
    pts = np.concatenate([base, base[:300], base[:10]])
    x, y, z = (np.ascontiguousarray(pts[:, q]) for q in range(3))
    c = pts[3]
    got = halo_gas.query_ball_point(x, y, z, c, 0.0)
    assert np.array_equal(got, og.query_ball_point(x, y, z, c, 0.0)) and len(got) == 3
    off, idx = halo_gas.balls_inside(x, y, z, [c[0]], [c[1]], [c[2]], [0.0], strict=True)
    assert len(idx) == 0
    for R in (1e-4, 1e-3, 5e-3):
        assert np.array_equal(halo_gas.query_ball_point(x, y, z, c, R), og.query_ball_point(x, y, z, c, R))
