"""Differentiable softened potential: a torch.autograd.Function over the GB300 kernels.

    phi_i = sum_j m_j (|s_j - t_i|^2 + eps^2)^-1/2        (self pair skipped when self_offset
                                                            is given: j == i + self_offset)

Forward: ``halma_potential_f32`` (float32 rsqrt pair terms, compensated sums).
Backward: ``halma_potential_grad_f32`` — the hand-written adjoint kernels — gives, for the
upstream gradient g = dL/dphi,
    dL/dm_j = sum_i g_i r^-1,   dL/ds_j = m_j sum_i g_i (t_i - s_j) r^-3,
    dL/dt_i = g_i sum_j m_j (s_j - t_i) r^-3,
so per-particle gravitational accelerations follow from the target gradient with g = 1
(a_i = G * dphi_i/dt_i) and dE/dm from the mass gradient.  Positions are passed as three
float32 CUDA tensors (SoA); passing the same tensors as sources and targets (with
self_offset=0) differentiates the self-potential, autograd summing both contributions.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib


def _ptrs(*ts):
    return [_lib.ptr(t) for t in ts]


def potential_f32(sx, sy, sz, m, tx, ty, tz, eps, self_offset=None):
    """Forward only (no graph): float32 phi on the device."""
    phi = torch.empty(tx.shape[0], dtype=torch.float32, device=tx.device)
    if tx.shape[0] == 0:
        return phi
    mask = _lib.MASK_NONE if self_offset is None else _lib.MASK_SELF
    st = _lib.lib().halma_potential_f32(int(sx.shape[0]), *_ptrs(m, sx, sy, sz), int(tx.shape[0]),
                                        *_ptrs(tx, ty, tz), float(eps) ** 2, mask, int(self_offset or 0),
                                        _lib.ptr(phi), _lib.stream_of(tx))
    _lib.check(st, "halma_potential_f32")
    return phi


class SoftenedPotential(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sx, sy, sz, m, tx, ty, tz, eps, self_offset):
        args = [a.contiguous() for a in (sx, sy, sz, m, tx, ty, tz)]
        for a in args:
            if a.dtype != torch.float32 or not a.is_cuda:
                raise ValueError("SoftenedPotential takes float32 CUDA tensors")
        _lib.check_arrays(np.float32, int(args[0].shape[0]), sx=args[0], sy=args[1], sz=args[2], m=args[3])
        _lib.check_arrays(np.float32, int(args[4].shape[0]), tx=args[4], ty=args[5], tz=args[6])
        ctx.eps = float(eps)
        ctx.self_offset = self_offset
        ctx.save_for_backward(*args)
        return potential_f32(*args, eps, self_offset)

    @staticmethod
    def backward(ctx, g):
        sx, sy, sz, m, tx, ty, tz = ctx.saved_tensors
        g = g.contiguous().to(torch.float32)
        ns, nt = int(sx.shape[0]), int(tx.shape[0])
        need_m = ctx.needs_input_grad[3]
        need_s = any(ctx.needs_input_grad[0:3])
        need_t = any(ctx.needs_input_grad[4:7])
        gm = torch.zeros(ns, dtype=torch.float32, device=sx.device) if need_m else None
        gs = torch.zeros(ns, 3, dtype=torch.float32, device=sx.device) if need_s else None
        gt = torch.zeros(nt, 3, dtype=torch.float32, device=sx.device) if need_t else None
        mask = _lib.MASK_NONE if ctx.self_offset is None else _lib.MASK_SELF
        st = _lib.lib().halma_potential_grad_f32(ns, *_ptrs(m, sx, sy, sz), nt, *_ptrs(tx, ty, tz, g),
                                                 ctx.eps ** 2, mask, int(ctx.self_offset or 0), _lib.ptr(gm),
                                                 _lib.ptr(gs), _lib.ptr(gt), _lib.stream_of(sx))
        _lib.check(st, "halma_potential_grad_f32")
        out_s = (gs[:, 0], gs[:, 1], gs[:, 2]) if need_s else (None, None, None)
        out_t = (gt[:, 0], gt[:, 1], gt[:, 2]) if need_t else (None, None, None)
        return (*out_s, gm, *out_t, None, None)


def softened_potential(sx, sy, sz, m, tx, ty, tz, eps, self_offset=None):
    return SoftenedPotential.apply(sx, sy, sz, m, tx, ty, tz, eps, self_offset)
