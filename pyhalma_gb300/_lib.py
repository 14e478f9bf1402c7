"""ctypes binding of libhalma_gb300.so (the C ABI declared in include/halma.h).

The library is loaded from the package directory only.  There is no CPU fallback: if the
shared library is missing the import of any compute function fails with ``ImportError``
telling the user to build it (``python -c "import pyhalma_gb300.build as b; b.build()"``).
Arrays cross the boundary as raw pointers: NumPy arrays (host memory; the library copies them
to the device and back) or CUDA torch tensors (device memory, used in place on the current
torch stream).
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhalma_gb300.so")

OK = 0
ERR_INVALID = -1
ERR_NOMEM = -2
ERR_CUDA = -3
ERR_NOT_CONVERGED = -4
ERR_TIMEOUT = -5
ERR_CAPACITY = -6
ERR_NO_DEVICE = -7

POT_REFERENCE = 0
POT_FAST = 1
MASK_COORD, MASK_SELF, MASK_NONE = 0, 1, 2
UNBIND_FP32C, UNBIND_FP64 = 0, 1

RED_FIELDS = ["mass", "cx", "cy", "cz", "vx", "vy", "vz", "rmax", "r05", "sigma", "n"]
UB_FIELDS = ["mass", "cx", "cy", "cz", "vx", "vy", "vz", "n_bound", "iterations", "e_kin", "e_pot"]


class HalmaError(RuntimeError):
    def __init__(self, status, where, detail):
        self.status = status
        super().__init__(f"{where}: {detail} (status {status})")


class UnbindParams(ctypes.Structure):
    _fields_ = [("eps", ctypes.c_double), ("G", ctypes.c_double), ("factor_v", ctypes.c_double),
                ("max_iter", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("use_graph", ctypes.c_int32), ("flags", ctypes.c_int32)]


UNBIND_FULL_RECOMPUTE = 1


class SubstructureParams(ctypes.Structure):
    _fields_ = [("linking_length", ctypes.c_double), ("dec_factor", ctypes.c_double),
                ("min_ll", ctypes.c_double), ("dist_factor", ctypes.c_double),
                ("minp_sub", ctypes.c_int32), ("minp", ctypes.c_int32)]


class PscParams(ctypes.Structure):
    _fields_ = [("linking_length", ctypes.c_double), ("q_fil", ctypes.c_double), ("sig_fil", ctypes.c_double),
                ("enabled", ctypes.c_int32), ("min_part", ctypes.c_int32), ("minp", ctypes.c_int32),
                ("max_passes", ctypes.c_int32)]


PSC_FIELDS = ["cx", "cy", "cz", "mass", "rmax", "npart", "n_cell", "kept", "passes"]


PROP_FIELDS = ["r05", "r05x", "r05y", "r05z", "vx", "vy", "vz", "jx", "jy", "jz", "j", "v_tf", "k_co", "a", "b", "c",
               "sig_3d", "sig_1d_x", "sig_1d_y", "sig_1d_z", "v_sigma", "lambda"]


_lock = threading.Lock()
_lib = None

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
_F64 = ctypes.c_double

SIGNATURES = {
    "halma_abi_version": ([], ctypes.c_int),
    "halma_status_string": ([ctypes.c_int], ctypes.c_char_p),
    "halma_last_error": ([], ctypes.c_char_p),
    "halma_release_workspace": ([], ctypes.c_int),
    "halma_kernel_launch_count": ([], ctypes.c_int64),
    "halma_set_profiling": ([_I32], ctypes.c_int),
    "halma_set_tile_table": ([_I32, _P, _P, _I32], ctypes.c_int),
    "halma_get_tile_table": ([_P, _P, _P, _P], ctypes.c_int),
    "halma_profile_stats": ([_P, _I32], ctypes.c_int),
    "halma_set_union_find_cap": ([_I32], ctypes.c_int),
    "halma_profile_fof_stages": ([_P, _I32], ctypes.c_int),
    "halma_measure_fp32_fma_rate": ([_I32, _I32, _P, _P, _P], ctypes.c_int),
    "halma_measure_pair_rate": ([_I32, _P, _P, _P], ctypes.c_int),
    "halma_measure_term_rate": ([_I32, _P, _P, _P], ctypes.c_int),
    "halma_fof": ([_I64, _P, _P, _P, _F64, _P, _P, _P], ctypes.c_int),
    "halma_fof_periodic": ([_I64, _P, _P, _P, _F64, _F64, _P, _P, _P], ctypes.c_int),
    "halma_fof_groups": ([_I64, _P, _I32, _P, _P, _P, _P], ctypes.c_int),
    "halma_fof_segmented": ([_I64, _P, _P, _P, _I64, _P, _F64, _P, _P, _P], ctypes.c_int),
    "halma_split_bridges": ([_I64, _P, _P, _P, _P, _I64, _P, _P, ctypes.POINTER(SubstructureParams), _P, _I64, _P,
                             _P, _P, _P], ctypes.c_int),
    "halma_phase_space_clean": ([_I64, _P, _P, _P, _P, _P, _P, _P, _I64, _P, _P, ctypes.POINTER(PscParams), _P, _P,
                                 _P, _P, _P], ctypes.c_int),
    "halma_halo_properties": ([_I64, _P, _P, _P, _P, _P, _P, _P, _I64, _P, _P, _P, _F64, _P, _P], ctypes.c_int),
    "halma_ball_gather": ([_I64, _P, _P, _P, _I64, _P, _P, _P, _P, _I32, _P, _P, _I64, _P, _P], ctypes.c_int),
    "halma_sequential_sum_f64": ([_I64, _P, _I64, _P, _P, _P], ctypes.c_int),
    "halma_amr_to_particles": ([_I32, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _F64, _I32, _P, _F64, _I64,
                                _P, _P, _P, _P, _P, _P, _P, _P, _P, _P], ctypes.c_int),
    "halma_bf_potential_f32": ([_I64, _P, _P, _P, _P, _I64, _P, _P, _P, _P, _I32, _F64, _P], ctypes.c_int),
    "halma_potential_f64": ([_I64, _P, _P, _P, _P, _I64, _P, _P, _P, _F64, _I32, _I64, _P, _P], ctypes.c_int),
    "halma_potential_f32": ([_I64, _P, _P, _P, _P, _I64, _P, _P, _P, _F64, _I32, _I64, _P, _P], ctypes.c_int),
    "halma_bf_potential_f32_noalloc": ([_I64, _P, _P, _P, _P, _I64, _P, _P, _P, _P, _F64, _P], ctypes.c_int),
    "halma_potential_grad_f32": ([_I64, _P, _P, _P, _P, _I64, _P, _P, _P, _P, _F64, _I32, _I64, _P, _P, _P, _P],
                                 ctypes.c_int),
    "halma_halo_reductions": ([_I64, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P], ctypes.c_int),
    "halma_unbind_batched": ([_I64, _I64, _P, _P, _P, _P, _P, _P, _P, _P, ctypes.POINTER(UnbindParams), _P, _P, _P,
                              _P], ctypes.c_int),
    "halma_find_haloes": ([_I64, _P, _P, _P, _P, _P, _P, _P, _F64, _I32, ctypes.POINTER(UnbindParams), _P, _P, _P,
                           _I64, _P, _P, _P, _P], ctypes.c_int),
}


def lib():
    """The loaded library; raises ImportError if it has not been built."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(
                    f"{LIB_PATH} is missing: build the CUDA extension first "
                    "(python -c 'import pyhalma_gb300.build as b; b.build()'); there is no CPU fallback")
            L = ctypes.CDLL(LIB_PATH)
            for name, (args, res) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.argtypes = args
                fn.restype = res
            _lib = L
    return _lib


def check(status, where):
    if status == OK:
        return
    detail = lib().halma_last_error().decode(errors="replace")
    if status == ERR_INVALID:
        raise ValueError(f"{where}: {detail}")
    raise HalmaError(status, where, detail)


def launch_count() -> int:
    return int(lib().halma_kernel_launch_count())


def set_profiling(on: bool):
    lib().halma_set_profiling(1 if on else 0)


def profile_stats():
    """Last call's measurements: dict(fof_ms, unbind_ms, passes=[(pairs, pair_kernels_ms), ...],
    sym_pairs=[pair terms of each pass evaluated by the symmetric block kernel],
    sym_ms=[milliseconds of that kernel in each pass])."""
    n = lib().halma_profile_stats(None, 0)
    buf = np.zeros(max(n, 3))
    lib().halma_profile_stats(buf.ctypes.data_as(ctypes.c_void_p), len(buf))
    k = int(buf[2])
    passes = [(float(buf[3 + 4 * i]), float(buf[4 + 4 * i])) for i in range(k)]
    sym = [float(buf[5 + 4 * i]) for i in range(k)]
    sym_ms = [float(buf[6 + 4 * i]) for i in range(k)]
    return {"fof_ms": float(buf[0]), "unbind_ms": float(buf[1]), "passes": passes, "sym_pairs": sym,
            "sym_ms": sym_ms}


FOF_STAGES = ["bbox_keys", "sort", "records", "cells", "items", "link", "labels", "groups"]


def measure_fp32_fma_rate(packed=True, iters=1 << 15):
    """(TFLOP/s, ms) of the FP32 FMA peak kernel on the current device."""
    t, ms = ctypes.c_double(0), ctypes.c_double(0)
    check(lib().halma_measure_fp32_fma_rate(1 if packed else 0, int(iters), ctypes.byref(t), ctypes.byref(ms), None),
          "halma_measure_fp32_fma_rate")
    return t.value, ms.value


def measure_pair_rate(iters=1 << 12):
    """(pairs/s, ms) of the pair-arithmetic ceiling kernel on the current device."""
    r, ms = ctypes.c_double(0), ctypes.c_double(0)
    check(lib().halma_measure_pair_rate(int(iters), ctypes.byref(r), ctypes.byref(ms), None),
          "halma_measure_pair_rate")
    return r.value, ms.value


def measure_term_rate(iters=1 << 12):
    """(pair terms/s, ms) of the tile kernel's arithmetic ceiling on the current device."""
    r, ms = ctypes.c_double(0), ctypes.c_double(0)
    check(lib().halma_measure_term_rate(int(iters), ctypes.byref(r), ctypes.byref(ms), None),
          "halma_measure_term_rate")
    return r.value, ms.value


def profile_fof_stages():
    """Milliseconds of each FoF stage of the last find_haloes call (profiling on)."""
    buf = np.zeros(len(FOF_STAGES))
    lib().halma_profile_fof_stages(buf.ctypes.data_as(ctypes.c_void_p), len(buf))
    return dict(zip(FOF_STAGES, buf.tolist()))


# ---------------------------------------------------------------------------------------
# array plumbing
# ---------------------------------------------------------------------------------------
def _is_torch(a):
    return type(a).__module__.startswith("torch")


def ptr(a):
    """Raw pointer of a contiguous NumPy array or torch tensor (None -> NULL)."""
    if a is None:
        return None
    if _is_torch(a):
        if not a.is_contiguous():
            raise ValueError("torch tensors passed to the library must be contiguous")
        return ctypes.c_void_p(a.data_ptr())
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("arrays passed to the library must be C-contiguous")
    return a.ctypes.data_as(ctypes.c_void_p)


def stream_of(*arrays):
    """The current torch stream if any argument lives on a CUDA device, else NULL."""
    for a in arrays:
        if a is not None and _is_torch(a) and a.is_cuda:
            import torch
            return ctypes.c_void_p(torch.cuda.current_stream(a.device).cuda_stream)
    return None


def as_host(a, dtype):
    """Contiguous NumPy array of the given dtype (copy only when needed)."""
    return np.ascontiguousarray(a, dtype=dtype)


_TORCH_DTYPE_NAMES = {np.float32: "float32", np.float64: "float64", np.int32: "int32", np.int64: "int64",
                      np.uint8: "uint8"}


def check_arrays(dtype, n, **arrays):
    """Raise ValueError unless every given array (None entries skipped) is one-dimensional,
    holds n entries (any number when n is None) and has exactly `dtype`; torch tensors on a
    CUDA device must also be on the current device.  The library reads n elements of that
    type through each raw pointer, so an array of another dtype or length would be read
    past its end."""
    for name, a in arrays.items():
        if a is None:
            continue
        if _is_torch(a):
            import torch
            want = getattr(torch, _TORCH_DTYPE_NAMES[np.dtype(dtype).type])
            if a.dtype != want:
                raise ValueError(f"{name} must be a {want} tensor, got {a.dtype}")
            if a.is_cuda and a.device.index != torch.cuda.current_device():
                raise ValueError(f"{name} is on {a.device}, not on the current device "
                                 f"cuda:{torch.cuda.current_device()}")
        elif not isinstance(a, np.ndarray) or a.dtype != np.dtype(dtype):
            raise ValueError(f"{name} must be a {np.dtype(dtype).name} array or tensor")
        shape = tuple(a.shape)
        if len(shape) != 1:
            raise ValueError(f"{name} must be one-dimensional, got shape {shape}")
        if n is not None and shape[0] != n:
            raise ValueError(f"{name} has {shape[0]} entries, expected {n}")


def pinned_empty(shape, dtype):
    """An uninitialised NumPy array in page-locked host memory from torch's caching pinned
    allocator (plain np.empty without torch or a CUDA device).  Device-to-host copies into it
    are DMA transfers with no CPU memcpy; a pageable destination makes the CUDA driver copy through
    staging buffers on the host and fault fresh pages in, whose cost depends on the host's
    other load.  The block goes back to torch's cache when the array is released, so repeated
    calls of the same size allocate nothing."""
    try:
        import torch
        if not torch.cuda.is_available():
            raise ImportError
    except ImportError:
        return np.empty(shape, dtype=dtype)
    tmap = {np.float32: torch.float32, np.float64: torch.float64, np.int32: torch.int32,
            np.int64: torch.int64, np.uint8: torch.uint8}
    return torch.empty(shape, dtype=tmap[np.dtype(dtype).type], pin_memory=True).numpy()


def like(a, shape, dtype):
    """An output buffer on the same side (host NumPy / device torch) as `a`."""
    if _is_torch(a):
        import torch
        tmap = {np.float32: torch.float32, np.float64: torch.float64, np.int32: torch.int32,
                np.int64: torch.int64, np.uint8: torch.uint8}
        return torch.empty(shape, dtype=tmap[np.dtype(dtype).type], device=a.device)
    return np.empty(shape, dtype=dtype)
