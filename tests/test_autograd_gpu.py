"""Adjoint of the softened potential: the GPU backward against the FP64 reference gradient
(oracle, norm-wise relative 1e-5) and against central finite differences of the FP64
potential with h = 1e-3 kpc (relative 1e-4)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _setup(cuda, n_src=3000, n_tgt=2000, seed=0):
    import torch
    rng = np.random.default_rng(seed)
    s = rng.normal(0, 0.02, (n_src, 3))
    t = rng.normal(0, 0.02, (n_tgt, 3))
    m = np.exp(rng.normal(np.log(1e5), 1.0, n_src))
    g = rng.normal(size=n_tgt)
    T = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float32, device=cuda, requires_grad=True)
    return s.astype(np.float32).astype(np.float64), t.astype(np.float32).astype(np.float64), \
        m.astype(np.float32).astype(np.float64), g, T


def test_backward_matches_fp64_gradient(cuda):
    import torch
    from pyhalma_gb300.autograd import softened_potential
    s, t, m, g, T = _setup(cuda)
    eps = 1e-4
    sx, sy, sz, mm = T(s[:, 0]), T(s[:, 1]), T(s[:, 2]), T(m)
    tx, ty, tz = T(t[:, 0]), T(t[:, 1]), T(t[:, 2])
    phi = softened_potential(sx, sy, sz, mm, tx, ty, tz, eps)
    ref_phi = oracle.potential_f64(m, *s.T, *t.T, eps2=eps * eps, mask=oracle.MASK_NONE)
    assert np.max(np.abs(phi.detach().cpu().numpy() / ref_phi - 1)) < 1e-6
    (phi * torch.tensor(g, dtype=torch.float32, device=cuda)).sum().backward()
    gm, gs, gt = oracle.potential_grad_f64(m, *s.T, *t.T, g, eps2=eps * eps, mask=oracle.MASK_NONE)
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    assert rel(mm.grad.cpu().numpy(), gm) < 1e-5
    assert rel(np.stack([a.grad.cpu().numpy() for a in (sx, sy, sz)], 1), gs) < 1e-5
    assert rel(np.stack([a.grad.cpu().numpy() for a in (tx, ty, tz)], 1), gt) < 1e-5


def test_self_potential_against_finite_differences(cuda):
    import torch
    from pyhalma_gb300.autograd import softened_potential
    rng = np.random.default_rng(3)
    n = 1500
    p = rng.normal(0, 0.01, (n, 3)).astype(np.float32).astype(np.float64)
    m = np.exp(rng.normal(np.log(1e5), 1.0, n)).astype(np.float32).astype(np.float64)
    eps = 1e-4
    x, y, z = (torch.tensor(p[:, k], dtype=torch.float32, device=cuda, requires_grad=True) for k in range(3))
    mm = torch.tensor(m, dtype=torch.float32, device=cuda, requires_grad=True)
    # potential energy W = -1/2 sum_i m_i phi_i (G = 1): dW/dm and forces
    phi = softened_potential(x, y, z, mm, x, y, z, eps, self_offset=0)
    W = -0.5 * (mm * phi).sum()
    W.backward()
    h = 1e-6   # Mpc = 1e-3 kpc

    def W64(mv, pv):
        ph = oracle.potential_f64(mv, *pv.T, *pv.T, eps2=eps * eps, mask=oracle.MASK_SELF)
        return -0.5 * float(mv @ ph)
    for j in (0, 11, 777):
        e = np.zeros(n)
        e[j] = h
        dp = np.zeros_like(p)
        dp[j, 0] = h
        fd_x = (W64(m, p + dp) - W64(m, p - dp)) / (2 * h)
        fd_m = (W64(m + e * 1e3, p) - W64(m - e * 1e3, p)) / (2 * h * 1e3)
        # the net force is a cancelling sum of FP32 terms: 1e-3 relative
        assert abs(x.grad[j].item() - fd_x) < 1e-3 * abs(fd_x), j
        assert abs(mm.grad[j].item() - fd_m) < 1e-4 * abs(fd_m), j


@pytest.mark.slow
def test_gas_halo_adjoint_at_full_scale(cuda):
    """The gas halo of the adjoint configuration: 2e6 NFW gas cells as targets, the gas and
    5e5 stars (2.5e6) as sources, L = sum_i phi_i (g = 1: the targets' gradients are the
    accelerations / G, the sources' mass gradients dL/dm).  512 sampled targets and 512 sampled
    sources against the FP64 gradient (norm-wise relative 1e-5), 8 of each against central
    finite differences of the FP64 potential with h = 1e-3 kpc (relative 1e-3 for the
    cancelling position sums, 1e-5 for the mass gradient)."""
    import torch
    from pyhalma_gb300 import synth
    from pyhalma_gb300.autograd import softened_potential
    g = synth.nfw_gas_halo(2_000_000, 500_000, seed=3)
    f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    S = np.stack([f32(np.concatenate([g.gas_x, g.st_x])), f32(np.concatenate([g.gas_y, g.st_y])),
                  f32(np.concatenate([g.gas_z, g.st_z]))], 1)
    M = f32(np.concatenate([g.gas_mass, g.st_mass]))
    Tp = np.stack([f32(g.gas_x), f32(g.gas_y), f32(g.gas_z)], 1)
    T = lambda a: torch.tensor(np.ascontiguousarray(a), device=cuda, requires_grad=True)
    sx, sy, sz, mm = T(S[:, 0]), T(S[:, 1]), T(S[:, 2]), T(M)
    tx, ty, tz = T(Tp[:, 0]), T(Tp[:, 1]), T(Tp[:, 2])
    eps = 1e-4
    phi = softened_potential(sx, sy, sz, mm, tx, ty, tz, eps)
    phi.sum().backward()
    gt_gpu = np.stack([a.grad.cpu().numpy() for a in (tx, ty, tz)], 1).astype(np.float64)
    gs_gpu = np.stack([a.grad.cpu().numpy() for a in (sx, sy, sz)], 1).astype(np.float64)
    gm_gpu = mm.grad.cpu().numpy().astype(np.float64)
    S64, M64, T64 = S.astype(np.float64), M.astype(np.float64), Tp.astype(np.float64)
    rng = np.random.default_rng(5)
    ti = np.sort(rng.choice(len(T64), 512, replace=False))
    si = np.sort(rng.choice(len(S64), 512, replace=False))
    _, _, gt = oracle.potential_grad_f64(M64, *S64.T, *T64[ti].T, np.ones(len(ti)), eps2=eps * eps,
                                         mask=oracle.MASK_NONE)
    gm, gs, _ = oracle.potential_grad_f64(M64[si], *S64[si].T, *T64.T, np.ones(len(T64)), eps2=eps * eps,
                                          mask=oracle.MASK_NONE)
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    assert rel(gt_gpu[ti], gt) < 1e-5
    assert rel(gs_gpu[si], gs) < 1e-5
    assert rel(gm_gpu[si], gm) < 1e-5
    h = 1e-6   # Mpc = 1e-3 kpc

    def phi_at(p):        # FP64 potential of all sources at one point
        d = S64 - p
        return float((M64 / np.sqrt((d * d).sum(1) + eps * eps)).sum())

    def l_source(j, p, m):  # source j's part of L = sum_i phi_i
        d = T64 - p
        return float(m * (1.0 / np.sqrt((d * d).sum(1) + eps * eps)).sum())
    for i in ti[:8]:
        e = np.zeros(3)
        e[0] = h
        fd = (phi_at(T64[i] + e) - phi_at(T64[i] - e)) / (2 * h)
        assert abs(gt_gpu[i, 0] - fd) <= 1e-3 * np.linalg.norm(gt[np.searchsorted(ti, i)]), i
    for j in si[:8]:
        e = np.zeros(3)
        e[1] = h
        fd = (l_source(j, S64[j] + e, M64[j]) - l_source(j, S64[j] - e, M64[j])) / (2 * h)
        assert abs(gs_gpu[j, 1] - fd) <= 1e-3 * np.linalg.norm(gs[np.searchsorted(si, j)]), j
        dm = 1e-3 * M64[j]
        fdm = (l_source(j, S64[j], M64[j] + dm) - l_source(j, S64[j], M64[j] - dm)) / (2 * dm)
        assert abs(gm_gpu[j] - fdm) <= 1e-5 * abs(fdm), j
