"""The allocation-free potential entry point against the regular one.

halma_bf_potential_f32_noalloc exists for callers that cannot let a library allocate device
memory: host codes (an AMR simulation calling the halo finder between its steps) whose own
pool reserves nearly all device memory, and callers that keep several streams busy, for whom
the device-wide synchronisation of a cudaFree is a stall.  It keeps its scratch in a static
device array shared by all calls.  This test calls it through the C ABI twice in a row
(different sizes, so the second call runs over the first call's leftover scratch) and compares
each result with halma_bf_potential_f32 in HALMA_POT_FAST mode on the same inputs: both split
the sources the same way and run the same kernels, so the results must be identical.
The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from pyhalma_gb300 import _lib

pytestmark = pytest.mark.gpu
SCRATCH_DOUBLES = 1 << 21   # partial sums the static scratch holds


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
        assert np.array_equal(a, b), seed


def test_noalloc_rejects_host_arrays_and_oversized_splits(cuda):
    import torch
    L = _lib.lib()
    h = np.zeros(8, dtype=np.float32)
    ph = h.ctypes.data_as(ctypes.c_void_p)
    assert L.halma_bf_potential_f32_noalloc(8, ph, ph, ph, ph, 8, ph, ph, ph, ph, 0.0, None) == _lib.ERR_INVALID
    # The source split gives 2 slices when the targets make one tile (128 targets) short of
    # 64 tiles per SM: 2 x 128 x (64 SMs - 1) partial sums, above 2^21 from 129 SMs on.
    sms = torch.cuda.get_device_properties(cuda).multi_processor_count
    nt, ns = 128 * (64 * sms - 1), 100_000
    if 2 * nt <= SCRATCH_DOUBLES:
        pytest.skip(f"{sms} SMs: no split of this shape exceeds the scratch")
    t = torch.zeros(nt, dtype=torch.float32, device=cuda)
    s = torch.zeros(ns, dtype=torch.float32, device=cuda)
    ps, pt = ctypes.c_void_p(s.data_ptr()), ctypes.c_void_p(t.data_ptr())
    st = L.halma_bf_potential_f32_noalloc(ns, ps, ps, ps, ps, nt, pt, pt, pt, pt, 0.0, None)
    assert st == _lib.ERR_CAPACITY
    assert b"partial sums" in L.halma_last_error()
