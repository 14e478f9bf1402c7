"""C ABI: the library loads, exports every function include/halma.h declares, and rejects bad
arguments with the documented status before touching a GPU (CPU only)."""
import ctypes
import os
import re

import numpy as np
import pytest

from pyhalma_gb300 import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "halma.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|const char \*)\s*\*?\s*(halma_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("halma_fof", "halma_fof_groups", "halma_bf_potential_f32", "halma_potential_f64",
                 "halma_potential_f32", "halma_potential_grad_f32", "halma_halo_reductions",
                 "halma_unbind_batched", "halma_find_haloes"):
        assert must in names


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    for name in declared_functions():
        assert hasattr(L, name), name
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"


def test_status_strings_and_version():
    L = _lib.lib()
    assert L.halma_abi_version() == 1
    assert L.halma_status_string(0) == b"ok"
    assert L.halma_status_string(-1) == b"invalid argument"


def test_invalid_arguments_are_rejected_before_any_device_work():
    L = _lib.lib()
    x = np.zeros(4)
    lab = np.zeros(4, dtype=np.int32)
    assert L.halma_fof(-1, _lib.ptr(x), _lib.ptr(x), _lib.ptr(x), 1.0, _lib.ptr(lab), None, None) == _lib.ERR_INVALID
    assert L.halma_fof(4, _lib.ptr(x), _lib.ptr(x), _lib.ptr(x), -1.0, _lib.ptr(lab), None, None) == _lib.ERR_INVALID
    assert b"linking length" in L.halma_last_error()
    assert L.halma_fof(4, _lib.ptr(x), _lib.ptr(x), _lib.ptr(x), float("nan"), _lib.ptr(lab), None, None) == \
        _lib.ERR_INVALID
    assert L.halma_fof(4, None, _lib.ptr(x), _lib.ptr(x), 1.0, _lib.ptr(lab), None, None) == _lib.ERR_INVALID
    f = np.zeros(3, dtype=np.float32)
    assert L.halma_bf_potential_f32(3, *[_lib.ptr(f)] * 4, 3, *[_lib.ptr(f)] * 3, _lib.ptr(f), 7, 0.0, None) == \
        _lib.ERR_INVALID
    assert L.halma_bf_potential_f32(3, *[_lib.ptr(f)] * 4, 3, *[_lib.ptr(f)] * 3, _lib.ptr(f),
                                    _lib.POT_REFERENCE, 0.5, None) == _lib.ERR_INVALID
    # no targets: nothing to do, success without a device
    assert L.halma_bf_potential_f32(3, *[_lib.ptr(f)] * 4, 0, *[_lib.ptr(f)] * 3, _lib.ptr(f),
                                    _lib.POT_FAST, 0.0, None) == _lib.OK
    p = _lib.UnbindParams(0.0, 4.3e-9, 1.0, 10, 0, 1, 0)
    off = np.array([0, 4], dtype=np.int64)
    b = np.zeros(4, dtype=np.uint8)
    assert L.halma_unbind_batched(4, 1, _lib.ptr(off), *[_lib.ptr(x)] * 7, ctypes.byref(p), _lib.ptr(b), None,
                                  None, None) == _lib.ERR_INVALID          # eps must be > 0
    p = _lib.UnbindParams(1e-4, 4.3e-9, 1.0, 0, 0, 1, 0)
    assert L.halma_unbind_batched(4, 1, _lib.ptr(off), *[_lib.ptr(x)] * 7, ctypes.byref(p), _lib.ptr(b), None,
                                  None, None) == _lib.ERR_INVALID          # max_iter >= 1
    p = _lib.UnbindParams(1e-4, 4.3e-9, 1.0, 5, 9, 1, 0)
    assert L.halma_unbind_batched(4, 1, _lib.ptr(off), *[_lib.ptr(x)] * 7, ctypes.byref(p), _lib.ptr(b), None,
                                  None, None) == _lib.ERR_INVALID          # unknown precision
    assert L.halma_potential_grad_f32(3, *[_lib.ptr(f)] * 4, 3, *[_lib.ptr(f)] * 4, 0.0, _lib.MASK_COORD, 0,
                                      None, None, None, None) == _lib.ERR_INVALID


def test_python_layer_raises_value_error():
    from pyhalma_gb300 import fof
    with pytest.raises(ValueError):
        fof.fof_labels(np.zeros(3), np.zeros(2), np.zeros(3), 1.0)
    with pytest.raises(ValueError):
        fof.friends_of_friends(np.zeros((3, 2)), 1.0)


def test_tile_table_validation_and_roundtrip():
    from pyhalma_gb300 import autotune
    saved = autotune.get_table()
    try:
        autotune.set_table([100, 5000, 2 ** 31 - 1], [1, 2, 4], 2048)
        assert autotune.get_table() == ([100, 5000, 2 ** 31 - 1], [1, 2, 4], 2048)
        with pytest.raises(ValueError):
            autotune.set_table([100], [3])            # tile shape must be 1, 2 or 4
        with pytest.raises(ValueError):
            autotune.set_table([100, 50], [1, 2])     # bounds must increase
        with pytest.raises(ValueError):
            autotune.set_table([100], [2], 100)       # slice must be a multiple of 32
    finally:
        autotune.set_table(*saved)


def test_unbind_params_layout():
    # the C struct: 3 doubles + 4 int32
    assert ctypes.sizeof(_lib.UnbindParams) == 40


def test_substructure_entry_points_reject_bad_arguments():
    L = _lib.lib()
    x = np.zeros(4)
    lab = np.zeros(4, dtype=np.int32)
    off = np.array([0, 4], dtype=np.int64)
    seg = lambda o, ll=1.0: L.halma_fof_segmented(4, *[_lib.ptr(x)] * 3, len(o) - 1, _lib.ptr(o), ll,
                                                  _lib.ptr(lab), None, None)
    assert seg(off, -1.0) == _lib.ERR_INVALID                                   # linking length
    assert seg(np.array([0, 3], dtype=np.int64)) == _lib.ERR_INVALID            # offsets do not reach n
    assert seg(np.array([0, 3, 2, 4], dtype=np.int64)) == _lib.ERR_INVALID      # decreasing offsets
    mem = np.arange(4, dtype=np.int32)
    out_off = np.zeros(8, dtype=np.int64)
    out_mem = np.zeros(4, dtype=np.int32)
    n_out = ctypes.c_int64(0)

    def split(p, o=off):
        return L.halma_split_bridges(4, *[_lib.ptr(x)] * 4, len(o) - 1, _lib.ptr(o), _lib.ptr(mem), ctypes.byref(p),
                                     ctypes.byref(n_out), 7, _lib.ptr(out_off), _lib.ptr(out_mem), None, None)
    assert split(_lib.SubstructureParams(0.0, 2.0, 0.0005, 0.75, 25, 50)) == _lib.ERR_INVALID      # LL > 0
    assert split(_lib.SubstructureParams(0.0015, 1.0, 0.0005, 0.75, 25, 50)) == _lib.ERR_INVALID   # DEC > 1
    assert split(_lib.SubstructureParams(0.0015, 2.0, -1.0, 0.75, 25, 50)) == _lib.ERR_INVALID     # MIN_LL >= 0
    assert split(_lib.SubstructureParams(0.0015, 2.0, 0.0005, 0.75, 25, 50),
                 np.array([0, 5], dtype=np.int64)) == _lib.ERR_INVALID   # more members than particles
    # the C struct: 4 doubles + 2 int32
    assert ctypes.sizeof(_lib.SubstructureParams) == 40


def test_ball_gather_rejects_bad_arguments():
    L = _lib.lib()
    x = np.zeros(4)
    c = np.zeros(2)
    n_found = ctypes.c_int64(0)
    g = lambda strict=0, nf=ctypes.byref(n_found), nb=2: L.halma_ball_gather(
        4, *[_lib.ptr(x)] * 3, nb, *[_lib.ptr(c)] * 4, strict, None, None, 0, nf, None)
    assert g(strict=2) == _lib.ERR_INVALID
    assert g(nf=None) == _lib.ERR_INVALID
    assert g(nb=-1) == _lib.ERR_INVALID
    assert L.halma_ball_gather(4, None, None, None, 2, *[_lib.ptr(c)] * 4, 0, None, None, 0, ctypes.byref(n_found),
                               None) == _lib.ERR_INVALID


def test_sequential_sum_rejects_bad_arguments():
    L = _lib.lib()
    v = np.ones(4)
    out = np.zeros(3)
    s = lambda o, n=4: L.halma_sequential_sum_f64(n, _lib.ptr(v), len(o) - 1, _lib.ptr(o), _lib.ptr(out), None)
    assert s(np.array([0, 2, 4], dtype=np.int64), n=-1) == _lib.ERR_INVALID
    assert s(np.array([0, 3], dtype=np.int64)) == _lib.ERR_INVALID                # offsets do not reach n
    assert s(np.array([0, 3, 2, 4], dtype=np.int64)) == _lib.ERR_INVALID          # decreasing offsets
    assert s(np.array([1, 2, 4], dtype=np.int64)) == _lib.ERR_INVALID             # offsets do not start at 0
    assert L.halma_sequential_sum_f64(4, None, 2, _lib.ptr(np.array([0, 2, 4], dtype=np.int64)), _lib.ptr(out),
                                      None) == _lib.ERR_INVALID


def test_halo_reductions_rejects_offsets_outside_the_rows():
    L = _lib.lib()
    x = np.zeros(4)
    out = np.zeros((2, len(_lib.RED_FIELDS)))
    r = lambda o: L.halma_halo_reductions(4, len(o) - 1, _lib.ptr(o), *[_lib.ptr(x)] * 7, None, None, _lib.ptr(out),
                                          None)
    assert r(np.array([0, 2, 5], dtype=np.int64)) == _lib.ERR_INVALID     # past the 4 rows
    assert r(np.array([0, 3, 2], dtype=np.int64)) == _lib.ERR_INVALID     # decreasing
    assert r(np.array([1, 2, 4], dtype=np.int64)) == _lib.ERR_INVALID     # does not start at 0
    assert r(np.array([0, 1, 3], dtype=np.int64)) == _lib.ERR_INVALID     # rows left outside every halo
    assert b"offsets" in L.halma_last_error()


def test_wrappers_check_dtypes_and_lengths_before_the_library_reads():
    """Raw pointers carry no type: a float32 tensor read as float64, or a short array read to
    n, would be read past its end.  The Python layer refuses both before any call."""
    torch = pytest.importorskip("torch")
    from pyhalma_gb300 import fof, halo_gas, halo_properties, phase_space, substructure, unbinding
    x64, x32 = torch.zeros(6, dtype=torch.float64), torch.zeros(6, dtype=torch.float32)
    with pytest.raises(ValueError, match="float64"):
        fof.fof_labels(x32, x32, x32, 1.0)
    with pytest.raises(ValueError, match="entries"):
        fof.fof_labels(x64, x64[:5], x64, 1.0)
    with pytest.raises(ValueError, match="int32"):
        fof.fof_groups(torch.zeros(6, dtype=torch.int64))
    with pytest.raises(ValueError, match="float32"):
        halo_gas.bf_potential(x64, x64, x64, x64, x32, x32, x32)
    with pytest.raises(ValueError, match="entries"):
        halo_gas.bf_potential(x32, x32, x32, x32[:4], x32, x32, x32)
    with pytest.raises(ValueError, match="float64"):
        halo_gas.balls_inside(x32, x32, x32, 0.0, 0.0, 0.0, 1.0)
    with pytest.raises(ValueError, match="entries"):
        halo_gas.balls_inside(np.zeros(6), np.zeros(5), np.zeros(6), 0.0, 0.0, 0.0, 1.0)
    off = np.array([0, 6], dtype=np.int64)
    with pytest.raises(ValueError, match="entries"):
        unbinding.unbind_batched(off, np.zeros(6), np.zeros(6), np.zeros(5), np.zeros(6), np.zeros(6), np.zeros(6),
                                 np.ones(6))
    with pytest.raises(ValueError, match="int64"):
        unbinding.unbind_batched(off.astype(np.int32), *[x64] * 7)
    with pytest.raises(ValueError, match="float64"):
        unbinding.find_haloes(*[x64] * 6, x32, 1.0)
    with pytest.raises(ValueError, match="entries"):
        halo_properties.halo_reductions(off, *[np.zeros(6)] * 6, np.zeros(7))
    with pytest.raises(ValueError, match="mask"):
        halo_properties.halo_reductions(off, *[np.zeros(6)] * 7, mask=np.ones(5, dtype=np.uint8))
    with pytest.raises(ValueError, match="about"):
        halo_properties.halo_reductions(off, *[x64] * 7, about=torch.zeros(8, dtype=torch.float32))
    with pytest.raises(ValueError, match="float64"):
        phase_space.sequential_sums(x32, torch.tensor([0, 6]))
    with pytest.raises(ValueError, match="int64"):
        substructure.fof_segmented_labels(x64, x64, x64, torch.tensor([0, 6], dtype=torch.int32), 1.0)


def test_group_wrappers_check_member_counts():
    from pyhalma_gb300 import halo_properties, phase_space
    z = np.zeros(6)
    off, mem = np.array([0, 4, 9], dtype=np.int64), np.arange(6, dtype=np.int32)
    with pytest.raises(ValueError, match="members"):
        phase_space.clean_groups(off, mem, *[z] * 7, 0.001, 1.0, 3.0)
    with pytest.raises(ValueError, match="members"):
        halo_properties.halo_property_table(off, mem, *[z] * 7, np.zeros((2, 5)), 0.001)
    with pytest.raises(ValueError, match="entries"):
        halo_properties.halo_property_table(off[:2], mem, *[z] * 6, np.zeros(5), np.zeros((1, 5)), 0.001)


C_CALLER = r"""
#include <stdio.h>
#include "halma.h"
int main(void) {
    double x[4] = {0, 0, 0, 0};
    int32_t lab[4];
    int64_t ng = 0;
    if (halma_abi_version() != 1) return 1;
    if (halma_fof(4, x, x, x, -1.0, lab, &ng, NULL) != HALMA_ERR_INVALID) return 2;
    printf("%s|%s\n", halma_status_string(HALMA_ERR_INVALID), halma_last_error());
    return 0;
}
"""


def test_plain_c_caller_compiles_links_and_calls(tmp_path):
    """The boundary is plain C: a C99 program (-pedantic, no C++ and no CUDA headers) includes
    halma.h, links the shared library and gets the documented status and message."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    src, exe = tmp_path / "caller.c", tmp_path / "caller"
    src.write_text(C_CALLER)
    libdir = os.path.dirname(_lib.LIB_PATH)
    _lib.lib()
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.dirname(HEADER),
                    str(src), "-L", libdir, "-lhalma_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out
    assert out.stdout.strip() == "invalid argument|linking length must be finite and >= 0"
