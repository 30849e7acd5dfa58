"""Host-side checks that need no GPU: the C ABI library loads and exports
every symbol include/edge_loops.h declares, the ctypes mirror matches the C
struct layout, argument errors come back as statuses, and the synthetic
generators produce what they promise."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "edge_loops.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(el_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(built_lib):
    from edge_loops_gb300 import _lib
    names = declared_functions()
    assert len(names) >= 15
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r" T (el_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)
    L = _lib.lib()
    for n in names:
        assert hasattr(L, n)


def test_struct_layout_matches_header(tmp_path):
    from edge_loops_gb300 import _lib
    prog = tmp_path / "layout.c"
    prog.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "edge_loops.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu\\n\", sizeof(el_csr),"
        " offsetof(el_csr, row_scale), offsetof(el_csr, value_dtype), sizeof(el_spmv_opts),"
        " offsetof(el_spmv_opts, num_threads), offsetof(el_spmv_opts, test_hooks));"
        "return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), str(prog), "-o", str(exe)],
                   check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    exp = [C.sizeof(_lib.ElCsr), _lib.ElCsr.row_scale.offset, _lib.ElCsr.value_dtype.offset,
           C.sizeof(_lib.ElSpmvOpts), _lib.ElSpmvOpts.num_threads.offset,
           _lib.ElSpmvOpts.test_hooks.offset]
    assert got == exp


def test_header_compiles_as_c_and_cpp(tmp_path):
    for lang, ext in (("c", "c"), ("c++", "cpp")):
        f = tmp_path / f"inc.{ext}"
        f.write_text('#include "edge_loops.h"\nint main(void){return el_version() > 0 ? 0 : 1;}\n')
        subprocess.run(["gcc" if lang == "c" else "g++", "-fsyntax-only", "-I",
                        os.path.join(REPO, "include"), str(f)], check=True)


def _csr(rows, cols, nnz, off=1, idx=1, val=1, dtype=0):
    from edge_loops_gb300 import _lib
    a = _lib.ElCsr()
    a.rows, a.cols, a.nnz = rows, cols, nnz
    a.offsets = off
    a.indices = idx
    a.values = val
    a.value_dtype = dtype
    return a


def test_argument_errors_without_gpu(built_lib):
    from edge_loops_gb300 import _lib
    L = _lib.lib()
    x = C.c_void_p(8)
    y = C.c_void_p(8)
    assert L.el_spmv(None, None, 0, None, x, y, None) == _lib.EL_ERR_NULL_POINTER
    a = _csr(1 << 30, 10, 1 << 30)
    assert L.el_spmv(None, C.byref(a), 0, None, x, y, None) == _lib.EL_ERR_OVERFLOW
    assert b"2^31" in L.el_last_error_string()
    # the limit keeps 2^16 of headroom below 2^31 for tile arithmetic
    a = _csr(3, 10, (1 << 31) - (1 << 16) - 3)
    assert L.el_spmv(None, C.byref(a), 0, None, x, y, None) == _lib.EL_ERR_OVERFLOW
    a = _csr(10, 10, -1)
    assert L.el_spmv(None, C.byref(a), 0, None, x, y, None) == _lib.EL_ERR_INVALID_ARGUMENT
    a = _csr(10, 10, 5, dtype=7)
    assert L.el_spmv(None, C.byref(a), 0, None, x, y, None) == _lib.EL_ERR_INVALID_ARGUMENT
    a = _csr(10, 10, 5, off=None)
    assert L.el_spmv(None, C.byref(a), 0, None, x, y, None) == _lib.EL_ERR_NULL_POINTER
    a = _csr(10, 10, 5)
    assert L.el_spmv(None, C.byref(a), 0, None, None, y, None) == _lib.EL_ERR_NULL_POINTER
    assert L.el_spmv(None, C.byref(a), _lib.EL_SCHED_BUCKETING, None, x, y, None) == \
        _lib.EL_ERR_UNSUPPORTED
    assert L.el_spmv(None, C.byref(a), 17, None, x, y, None) == _lib.EL_ERR_INVALID_ARGUMENT
    assert L.el_spmm(None, C.byref(a), 0, None, x, 0, 4, 2, y, 4, None) == \
        _lib.EL_ERR_INVALID_ARGUMENT  # ldb < n
    assert L.el_spmm(None, C.byref(a), _lib.EL_SCHED_WORK_ORIENTED, None, x, 0, 4, 4, y, 4,
                     None) == _lib.EL_ERR_UNSUPPORTED
    assert L.el_merge_path_partition(None, 10, 10, 128, 5, None, None) == \
        _lib.EL_ERR_NULL_POINTER
    assert L.el_merge_path_thread_coords(x, 10, 10, 1, 5, y, None) == \
        _lib.EL_ERR_INVALID_ARGUMENT
    assert L.el_quantize_values(x, 10, 10, x, 0, y, None, None) == \
        _lib.EL_ERR_INVALID_ARGUMENT
    assert L.el_status_string(_lib.EL_ERR_OVERFLOW) == b"EL_ERR_OVERFLOW"
    assert L.el_version() == 100


def test_num_tiles():
    from edge_loops_gb300 import _lib
    L = _lib.lib()
    assert L.el_merge_path_num_tiles(1000, 10000, 128, 5) == -(-11000 // 640)
    assert L.el_merge_path_num_tiles(0, 0, 128, 5) == 0
    assert L.el_merge_path_num_tiles(5, 5, 0, 5) == -1


def test_opts_default_zeroes():
    from edge_loops_gb300 import _lib
    o = _lib.ElSpmvOpts()
    o.items_per_thread = 9
    o.test_hooks = 4
    _lib.lib().el_spmv_opts_default(C.byref(o))
    assert o.items_per_thread == 0 and o.test_hooks == 0


def test_generators():
    import torch
    from edge_loops_gb300 import synth
    off, idx, val, x, cols = synth.uniform_rows(seed=0)
    assert off[-1] == 10000 and cols == 1000
    assert bool((idx.view(1000, 10).diff(dim=1) > 0).all())
    assert float(val.min()) >= -1 and float(val.max()) <= 1
    off2, idx2, *_ = synth.uniform_rows(seed=0)
    assert torch.equal(idx, idx2)
    # Above 2^24 cells the columns are drawn per row: no rows x cols matrix.
    off, idx, val, x, cols = synth.uniform_rows(rows=1 << 13, cols=1 << 12, per_row=7, seed=2)
    assert int(off[-1]) == 7 << 13 and int(idx.min()) >= 0 and int(idx.max()) < cols
    assert bool((idx.view(-1, 7).diff(dim=1) > 0).all())
    with pytest.raises(ValueError):
        synth.uniform_rows(rows=4, cols=3, per_row=4)
    off, idx, val, x, cols = synth.power_law(rows=1 << 12, target_nnz=60_000, cap=3000, seed=1)
    lens = off.long().diff()
    assert int(lens.min()) >= 1 and int(lens.max()) <= 3000
    assert abs(int(off[-1]) - 60_000) < 3000
    row_of = torch.repeat_interleave(torch.arange(1 << 12), lens)
    key = row_of * cols + idx.long()
    assert bool((key.diff() > 0).all())  # sorted and distinct within rows
    n = 12
    off, idx, val, x, rows = synth.stencil27(n=n)
    assert int(off[-1]) == (3 * n - 2) ** 3 and rows == n ** 3
    row_of = torch.repeat_interleave(torch.arange(rows), off.long().diff())
    diag = idx.long() == row_of
    assert bool((val[diag] == 26.5).all()) and int(diag.sum()) == rows
    assert float(val[~diag].max()) <= 0 and float(val[~diag].min()) >= -1
    assert bool(((row_of * rows + idx.long()).diff() > 0).all())


def test_batched_generator():
    from edge_loops_gb300 import synth
    R, offc, idxc, valc, xc, rs, ns = synth.batched(count=32, rows_hi=4096, seed=4)
    assert int(R.min()) >= 64 and int(R.max()) <= 4096
    assert xc.numel() == int(R.sum())
    total = 0
    for m in range(32):
        om = offc[rs[m] + m: rs[m] + m + R[m] + 1].long()
        assert int(om[0]) == 0 and bool((om.diff() >= 1).all())
        assert bool((om.diff() <= R[m]).all())
        seg = idxc[ns[m]: ns[m] + om[-1]]
        assert int(seg.max()) < int(R[m]) and int(seg.min()) >= 0
        total += int(om[-1])
    assert total == idxc.numel()
    mean = idxc.numel() / float(R.sum())
    assert 6.0 < mean < 10.0


def test_python_api_rejects_arrays_the_library_cannot_read():
    """The library reads every array as plain memory from its first element,
    so the Python face refuses what would read the wrong bytes or past an
    allocation: wrong dtypes, strided or expanded views, short arrays, mixed
    devices, and a host matrix handed to the device entry points."""
    import torch
    from edge_loops_gb300 import api
    off = torch.tensor([0, 2, 3], dtype=torch.int32)
    idx = torch.tensor([0, 2, 1], dtype=torch.int32)
    val = torch.tensor([1.0, 2.0, 3.0])
    A = api.CSR(off, idx, val, 2, 3)
    assert A.nnz == 3 and A.device.type == "cpu"
    with pytest.raises(TypeError):
        api.CSR(off.long(), idx, val, 2, 3)
    with pytest.raises(TypeError):
        api.CSR(off, idx.long(), val, 2, 3)
    with pytest.raises(TypeError):
        api.CSR(off, idx, val.double(), 2, 3)
    with pytest.raises(TypeError):
        api.CSR(off, idx, val, 2, 3, row_scale=torch.ones(2, dtype=torch.float64))
    with pytest.raises(ValueError):  # strided view
        api.CSR(off, torch.tensor([0, 9, 2, 9, 1, 9], dtype=torch.int32)[::2], val, 2, 3)
    with pytest.raises(ValueError):  # expanded (stride 0): one element of storage
        api.CSR(off, idx, torch.ones(1).expand(3), 2, 3)
    with pytest.raises(ValueError):
        api.CSR(off, idx, val, 3, 3)  # offsets too short for 3 rows
    with pytest.raises(ValueError):
        api.CSR(off, idx, val[:2], 2, 3)  # fewer values than indices
    with pytest.raises(ValueError):
        api.CSR(off, idx, val, 2, 3, row_scale=torch.ones(1))
    x = torch.ones(3)
    with pytest.raises(ValueError):  # device entry point, host matrix
        api.spmv(A, x)
    with pytest.raises(ValueError):
        api.spmm(A, torch.ones(3, 4))
    with pytest.raises(ValueError):  # x shorter than cols
        api.spmv_host(A, torch.ones(2))
    with pytest.raises(ValueError):  # expanded x
        api.spmv_host(A, torch.ones(1).expand(3))
    with pytest.raises(TypeError):
        api.spmv_host(A, torch.ones(3, dtype=torch.float64))
    with pytest.raises(ValueError):  # y strided
        api.spmv_host(A, x, torch.empty(4)[::2])
