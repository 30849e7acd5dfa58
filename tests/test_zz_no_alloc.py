"""el_spmv_static_scratch: SpMV for callers that must not allocate device
memory while they run (servers whose device memory is reserved up front,
allocation-free real-time loops, plugins inside a host that owns the
allocator).  Its scratch is a fixed array in the library's device image;
this checks, through the C ABI, that it gives the same y as el_spmv (within
the order-free FP32 bound both are held to) on two calls in a row, and that
it refuses a range count its scratch cannot hold.

Kept in its own file, collected last, so a failure here never hides the
results of the other GPU tests."""
import ctypes as C

import numpy as np
import pytest
import torch

from conftest import order_free_bound

pytestmark = pytest.mark.gpu


def _static_spmv(A, x, y, num_ranges=0, flags=True):
    from edge_loops_gb300 import _lib
    a = A.el()
    f = C.c_uint32(0xffffffff)
    st = _lib.lib().el_spmv_static_scratch(
        C.byref(a), C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), num_ranges,
        C.byref(f) if flags else None, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return st, int(f.value)


def test_static_scratch_matches_el_spmv_twice(cuda, oracle_mod):
    from edge_loops_gb300 import api, synth
    off, idx, vals, x, cols = synth.power_law(rows=1 << 15, target_nnz=600_000, cap=60_000,
                                              seed=11)
    A = api.CSR.from_arrays(off, idx, vals, cols, device=cuda)
    xt = x.to(cuda)
    y_ref = api.spmv(A, xt, schedule="merge_path_flat")
    assert api.workspace_errors() == 0
    y64, yabs = oracle_mod.spmv_f64(off.numpy(), idx.numpy(), vals.numpy(), x.numpy())
    bound = order_free_bound(off.numpy(), yabs)
    ref = y_ref.cpu().numpy().astype(np.float64)
    for call in range(2):  # the shared array keeps the previous call's contents
        y = torch.full((A.rows,), float("nan"), device=cuda)
        st, flags = _static_spmv(A, xt, y)
        assert st == 0 and flags == 0, (call, st, flags)
        got = y.cpu().numpy().astype(np.float64)
        assert np.all(np.abs(got - y64) <= bound), call
        assert np.all(np.abs(got - ref) <= 2 * bound), call


def test_static_scratch_range_limit_and_small_counts(cuda, oracle_mod):
    from edge_loops_gb300 import _lib, api, synth
    off, idx, vals, x, cols = synth.power_law(rows=1 << 12, target_nnz=50_000, cap=20_000,
                                              seed=12)
    A = api.CSR.from_arrays(off, idx, vals, cols, device=cuda).quantized(torch.bfloat16)
    xt = x.to(cuda)
    y = torch.empty(A.rows, device=cuda)
    st, _ = _static_spmv(A, xt, y, num_ranges=_lib.EL_STATIC_MAX_RANGES + 1)
    assert st == _lib.EL_ERR_INVALID_ARGUMENT
    assert b"at most" in _lib.lib().el_last_error_string()
    qv = A.values.float().cpu().numpy()
    y64, yabs = oracle_mod.spmv_f64(off.numpy(), idx.numpy(), qv, x.numpy(),
                                    row_scale=A.row_scale.cpu().numpy())
    bound = order_free_bound(off.numpy(), yabs)
    ref = api.spmv(A, xt).cpu().numpy().astype(np.float64)
    assert np.all(np.abs(ref - y64) <= bound)
    for ranges in (1, 7, _lib.EL_STATIC_MAX_RANGES):
        st, flags = _static_spmv(A, xt, y, num_ranges=ranges)
        assert st == 0 and flags == 0
        got = y.cpu().numpy().astype(np.float64)
        assert np.all(np.abs(got - y64) <= bound), ranges
        assert np.all(np.abs(got - ref) <= 2 * bound), ranges


def test_static_scratch_errors_readable_after_async_call(cuda):
    """With flags == NULL the call is asynchronous; el_spmv_static_scratch_errors
    reads the bits it raised afterwards (here: a column index past the end,
    which the kernel skips and reports), and the next call starts clean."""
    from edge_loops_gb300 import _lib, api
    L = _lib.lib()
    off = np.array([0, 2, 3, 5], dtype=np.int32)
    idx = np.array([0, 9, 1, 0, 2], dtype=np.int32)  # 9 >= cols
    vals = np.ones(5, dtype=np.float32)
    A = api.CSR.from_arrays(off, idx, vals, 3, device=cuda)
    x = torch.ones(3, device=cuda)
    y = torch.empty(3, device=cuda)
    st, _ = _static_spmv(A, x, y, flags=False)
    assert st == 0
    f = C.c_uint32(0)
    s = torch.cuda.current_stream().cuda_stream
    assert L.el_spmv_static_scratch_errors(C.c_void_p(s), C.byref(f), 1) == 0
    assert f.value & _lib.EL_FLAG_INDEX_RANGE
    good = api.CSR.from_arrays(off, np.array([0, 2, 1, 0, 2], np.int32), vals, 3, device=cuda)
    st, flags = _static_spmv(good, x, y)
    assert st == 0 and flags == 0
    np.testing.assert_array_equal(y.cpu().numpy(), [2, 1, 2])
    assert L.el_spmv_static_scratch_errors(C.c_void_p(s), C.byref(f), 0) == 0 and f.value == 0
