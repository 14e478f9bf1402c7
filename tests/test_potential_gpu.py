"""GPU potential parity.

* reference mode: bit-identical to the float32 restatement of particle_subroutines.f90:466-514
  (sequential sum, coordinate mask, each operation rounded);
* fast mode: float32 rsqrt pair terms + compensated sums, relative error <= 1e-6 against the
  FP64 oracle (tolerance stated here: RTOL_FAST);
* FP64 comparator path: <= 1e-12 against the FP64 oracle;
* the drop-in wrappers, RPS and most_bound_particle: equal to the reference's outputs.
"""
import numpy as np
import pytest

import oracle
from pyhalma_gb300 import _lib, halo_gas, synth

pytestmark = pytest.mark.gpu
RTOL_FAST = 1e-6


def _cloud(rng, n, scale=0.01, centre=(12.3, -4.5, 7.7)):
    p = rng.normal(0, scale, (n, 3)) + np.asarray(centre)
    m = np.exp(rng.normal(np.log(1e6), 1.0, n))
    return p, m


def test_reference_mode_bit_exact(cuda):
    rng = np.random.default_rng(0)
    for ns, nt in ((1, 1), (31, 33), (1000, 257), (5003, 1999)):
        p, m = _cloud(rng, ns)
        t, _ = _cloud(rng, nt)
        got = halo_gas.bf_potential(m, p[:, 0], p[:, 1], p[:, 2], t[:, 0], t[:, 1], t[:, 2], mode="reference")
        ref = oracle.bf_potential_f32(m, p[:, 0], p[:, 1], p[:, 2], t[:, 0], t[:, 1], t[:, 2])
        assert got.dtype == np.float32
        assert np.array_equal(got, ref), (ns, nt)


def test_reference_mode_mask_and_duplicates_bit_exact(cuda):
    # AMR-like lattice: many sources share one or two coordinates with a target, duplicates too
    g = (np.arange(12) * 0.25 + 3.0).astype(np.float32)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    src = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    src = np.concatenate([src, src[:50]])
    m = np.linspace(1.0, 2.0, len(src)).astype(np.float32)
    tgt = src[::7]
    got = halo_gas.bf_potential(m, *src.T, *tgt.T, mode="reference")
    ref = oracle.bf_potential_f32(m, *src.T, *tgt.T)
    assert np.array_equal(got, ref)
    fast = halo_gas.bf_potential(m, *src.T, *tgt.T, mode="fast")
    r64 = oracle.potential_f64(m, *src.T.astype(np.float64), *tgt.T.astype(np.float64), mask=oracle.MASK_COORD)
    assert np.max(np.abs(fast / r64 - 1)) < RTOL_FAST


def test_fast_mode_relative_error_vs_fp64(cuda):
    rng = np.random.default_rng(1)
    for ns, nt, eps in ((20_000, 3_000, 0.0), (100_000, 512, 1e-4), (64, 100_000, 1e-4)):
        p, m = _cloud(rng, ns)
        t, _ = _cloud(rng, nt)
        p32, t32, m32 = p.astype(np.float32), t.astype(np.float32), m.astype(np.float32)
        got = _lib.lib()  # noqa: F841 (library loads)
        phi = halo_gas.bf_potential(m32, *p32.T, *t32.T, mode="fast", eps2=eps * eps)
        ref = oracle.potential_f64(m32, *p32.T.astype(np.float64), *t32.T.astype(np.float64), eps2=eps * eps,
                                   mask=oracle.MASK_COORD)
        rel = np.abs(phi.astype(np.float64) / ref - 1.0)
        assert rel.max() < RTOL_FAST, (ns, nt, rel.max())


def test_wrapper_semantics(cuda):
    e = halo_gas.brute_force_binding_energy_fortran([1.0], [0.0], [0.0], [0.0], [], [], [])
    assert e.size == 0 and e.dtype == np.float64            # np.array([]) as in halo_gas.py:169-170
    out = halo_gas.brute_force_binding_energy_fortran([1.0, 2.0], [0.0, 1.0], [0.0, 1.0], [0.0, 1.0],
                                                      [3.0], [4.0], [5.0])
    assert out.dtype == np.float32
    # no sources: zero potential
    z = halo_gas.bf_potential([], [], [], [], [1.0, 2.0], [1.0, 2.0], [1.0, 2.0])
    assert np.array_equal(z, np.zeros(2, np.float32))


def test_fp64_path_vs_oracle(cuda):
    rng = np.random.default_rng(2)
    p, m = _cloud(rng, 3000)
    phi = np.empty(3000)
    for mask in (oracle.MASK_COORD, oracle.MASK_SELF, oracle.MASK_NONE):
        eps2 = 0.0 if mask != oracle.MASK_NONE else 1e-8
        st = _lib.lib().halma_potential_f64(3000, _lib.ptr(m), *[_lib.ptr(np.ascontiguousarray(p[:, k])) for k in range(3)],
                                            3000, *[_lib.ptr(np.ascontiguousarray(p[:, k])) for k in range(3)],
                                            eps2, mask, 0, _lib.ptr(phi), None)
        _lib.check(st, "halma_potential_f64")
        ref = oracle.potential_f64(m, *p.T, *p.T, eps2=eps2, mask=mask)
        assert np.max(np.abs(phi / ref - 1)) < 1e-12


def test_rps_and_most_bound_match_reference(golden, cuda):
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


def test_device_tensor_path(cuda):
    import torch
    rng = np.random.default_rng(4)
    p, m = _cloud(rng, 4000)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(cuda)
    phi = halo_gas.bf_potential(t(m), t(p[:, 0]), t(p[:, 1]), t(p[:, 2]), t(p[:, 0]), t(p[:, 1]), t(p[:, 2]),
                                mode="reference")
    assert phi.is_cuda
    ref = oracle.bf_potential_f32(m, p[:, 0], p[:, 1], p[:, 2], p[:, 0], p[:, 1], p[:, 2])
    assert np.array_equal(phi.cpu().numpy(), ref)


@pytest.mark.parametrize("nt,ns,self_mask", [(20_001, 20_001, False), (20_001, 26_000, False),
                                             (9_000, 300_000, False), (12_345, 15_000, True)])
def test_self_set_potential_symmetric_route(cuda, nt, ns, self_mask):
    """Targets that are the first sources (the same device arrays): the set's pairs go through
    the symmetric block kernel, once for both particles; the other sources through the tile
    kernel.  Against the FP64 oracle at RTOL_FAST and against the tile kernel alone (the same
    targets as separate arrays) at RTOL_FAST."""
    import torch
    from pyhalma_gb300.autograd import potential_f32
    rng = np.random.default_rng(nt + ns)
    p, m = _cloud(rng, ns, scale=0.005, centre=(0.3, -0.2, 0.1))
    f = lambda a: torch.tensor(np.ascontiguousarray(a, dtype=np.float32), device=cuda)
    sx, sy, sz, sm = f(p[:, 0]), f(p[:, 1]), f(p[:, 2]), f(m)
    eps = 1e-4
    so = 0 if self_mask else None
    phi = potential_f32(sx, sy, sz, sm, sx[:nt], sy[:nt], sz[:nt], eps, self_offset=so).cpu().numpy()
    tile = potential_f32(sx, sy, sz, sm, sx[:nt].clone(), sy[:nt].clone(), sz[:nt].clone(), eps,
                         self_offset=so).cpu().numpy()
    q = p.astype(np.float32).astype(np.float64)
    ref = oracle.potential_f64(m.astype(np.float32).astype(np.float64), *q.T, *q[:nt].T, eps2=eps * eps,
                               mask=oracle.MASK_SELF if self_mask else oracle.MASK_NONE)
    assert np.max(np.abs(phi / ref - 1.0)) <= RTOL_FAST
    assert np.max(np.abs(phi.astype(np.float64) / tile - 1.0)) <= RTOL_FAST
