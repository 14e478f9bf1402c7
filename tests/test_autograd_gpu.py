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
