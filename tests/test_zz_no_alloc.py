"""The allocation-free potential entry point against the regular one.

halma_bf_potential_f32_noalloc exists for callers that cannot allocate device memory when they
need the potential: code running while its stream is captured into a CUDA graph, where
cudaMalloc is not allowed, and host applications whose own memory pool owns all device
memory.  It keeps its scratch in a static device array shared by all calls.  This test calls it
through the C ABI twice in a row (different sizes, so the second call runs over the first
call's leftover scratch) and compares each result with halma_bf_potential_f32 in
HALMA_POT_FAST mode on the same inputs, within the tolerance of the other potential tests.
The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from pyhalma_gb300 import _lib

pytestmark = pytest.mark.gpu
RTOL_FAST = 1e-6


def _case(seed, ns, nt, cuda):
    import torch
    rng = np.random.default_rng(seed)
    src = rng.normal(0, 0.01, (ns, 3)) + np.array([3.1, -2.2, 0.7])
    tgt = rng.normal(0, 0.01, (nt, 3)) + np.array([3.1, -2.2, 0.7])
    m = np.exp(rng.normal(np.log(1e6), 1.0, ns))
    f = lambda a: torch.tensor(np.ascontiguousarray(a, dtype=np.float32), device=cuda)
    return [f(m), f(src[:, 0]), f(src[:, 1]), f(src[:, 2])], [f(tgt[:, 0]), f(tgt[:, 1]), f(tgt[:, 2])]


def _call(fn, srcs, tgts, out, *extra):
    import torch
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = [ctypes.c_void_p(t.data_ptr()) for t in srcs + tgts]
    st = fn(srcs[0].numel(), *p[:4], tgts[0].numel(), *p[4:], ctypes.c_void_p(out.data_ptr()), *extra, stream)
    _lib.check(st, fn.__name__)
    torch.cuda.synchronize()


def test_noalloc_matches_regular_entry_point_twice(cuda):
    import torch
    L = _lib.lib()
    eps2 = 1e-8
    # 100 000 sources / 2 000 targets splits the sources (uses the scratch); then a smaller call
    for seed, ns, nt in ((1, 100_000, 2_000), (2, 30_000, 700)):
        srcs, tgts = _case(seed, ns, nt, cuda)
        a = torch.empty(nt, dtype=torch.float32, device=cuda)
        b = torch.empty(nt, dtype=torch.float32, device=cuda)
        _call(L.halma_bf_potential_f32_noalloc, srcs, tgts, a, ctypes.c_double(eps2))
        _call(L.halma_bf_potential_f32, srcs, tgts, b, ctypes.c_int32(_lib.POT_FAST), ctypes.c_double(eps2))
        a, b = a.cpu().numpy(), b.cpu().numpy()
        assert np.all(np.isfinite(a)) and np.all(a > 0)
        assert np.max(np.abs(a.astype(np.float64) / b - 1.0)) <= RTOL_FAST, seed


def test_noalloc_rejects_host_arrays_and_oversized_splits(cuda):
    import torch
    L = _lib.lib()
    h = np.zeros(8, dtype=np.float32)
    ph = h.ctypes.data_as(ctypes.c_void_p)
    assert L.halma_bf_potential_f32_noalloc(8, ph, ph, ph, ph, 8, ph, ph, ph, ph, 0.0, None) == _lib.ERR_INVALID
    # 1.1e6 targets against 1e5 sources would need 2 slices x 1.1e6 partial sums > 2^21
    nt, ns = 1_100_000, 100_000
    t = torch.zeros(nt, dtype=torch.float32, device=cuda)
    s = torch.zeros(ns, dtype=torch.float32, device=cuda)
    ps, pt = ctypes.c_void_p(s.data_ptr()), ctypes.c_void_p(t.data_ptr())
    st = L.halma_bf_potential_f32_noalloc(ns, ps, ps, ps, ps, nt, pt, pt, pt, pt, 0.0, None)
    assert st == _lib.ERR_CAPACITY
    assert b"partial sums" in L.halma_last_error()
