"""The default merge-path kernel's own split points, bit for bit.

The kernel cuts the merge of row ends and nonzeros into warp ranges at
diagonals g * R and finds each range's (row, nonzero) start and end with its
own warp search.  el_debug_range_trace makes every range write the diagonals
and the coordinates it computed; they must equal:

  * row weight 1 (the reference's equal split, and el_spmv_static_scratch):
    the oracle's restatement of the reference's search::_binary_search
    (util/search.hxx:34-60) at the same diagonals;
  * row weight 2 (the library default, a row end counted as two merge
    items): the closed form -- rows i with offsets[i+1] + 2 (i+1) <= d are
    closed, nonzero min(d - 2 x, offsets[x+1]) -- and, on small shapes, an
    item-by-item walk of the weighted merge.

A cut that still covered every nonzero once but sat elsewhere would pass the
y-within-bound checks of the other tests; these catch it."""
import ctypes as C
import functools

import numpy as np
import pytest
import torch

from conftest import load_golden, merge_coords_weighted, merge_walk_weighted, random_csr

pytestmark = pytest.mark.gpu

TILE = 256  # nonzeros per tile; range lengths are whole tiles


def _trace_run(fn, cap, cuda):
    from edge_loops_gb300 import _lib
    L = _lib.lib()
    buf = torch.full((6 * cap,), -1, dtype=torch.int64, device=cuda)
    _lib.check(L.el_debug_range_trace(C.c_void_p(buf.data_ptr()), cap), "trace on")
    try:
        fn()
        torch.cuda.synchronize()
    finally:
        _lib.check(L.el_debug_range_trace(None, 0), "trace off")
    t = buf.view(cap, 6).cpu().numpy()
    used = t[:, 0] >= 0
    n = int(used.sum())
    assert used[:n].all() and not used[n:].any(), "ranges are not numbered 0..n-1"
    return t[:n]


def _check(oracle_mod, off, tr, w):
    rows, nnz = len(off) - 1, int(off[-1])
    total = w * rows + nnz
    d0, d1 = tr[:, 0], tr[:, 1]
    R = int(d1[0] - d0[0]) if len(tr) > 1 else int(d1[0])
    assert len(tr) == 1 or R % TILE == 0
    g = np.arange(len(tr), dtype=np.int64)
    np.testing.assert_array_equal(d0, np.minimum(g * R, total))
    np.testing.assert_array_equal(d1, np.minimum(g * R + R, total))
    assert d1[-1] == total and (len(tr) == 1 or d0[-1] < total)
    for col, d in ((2, d0), (4, d1)):
        x, n = merge_coords_weighted(off, d, w)
        np.testing.assert_array_equal(tr[:, col], x)
        np.testing.assert_array_equal(tr[:, col + 1], n)
        if w == 1:  # the reference's search, restated in the oracle
            for k in range(len(d)):
                got = oracle_mod.mp_search(int(d[k]), off[1:], rows, 0, nnz)
                assert (int(tr[k, col]), int(tr[k, col + 1])) == got, (k, int(d[k]))
        if total <= 20_000:
            walk = merge_walk_weighted(off, w)
            np.testing.assert_array_equal(tr[:, col:col + 2], walk[d])


NAMES = ["chesapeake"] + ["random%d" % k for k in range(6)] + ["long_rows", "empty_rows",
                                                                 "power_law"]


@functools.lru_cache(maxsize=None)
def _case(name):
    """(offsets, indices, values, cols) of a named case, made on first use."""
    if name == "chesapeake":
        g = load_golden("chesapeake.npz")
        return g["offsets"], g["indices"], g["values"], 39
    if name.startswith("random"):
        rng = np.random.default_rng(21 + int(name[6:]))
        rows = int(rng.integers(1, 3000))
        cols = int(rng.integers(1, 4000))
        off, idx, vals, _ = random_csr(rng, rows, cols, max_len=int(rng.integers(0, 60)),
                                       empty_frac=float(rng.choice([0.0, 0.3, 0.9])))
        return off, idx, vals, cols
    if name == "long_rows":
        rng = np.random.default_rng(20)
        off, idx, vals, _ = random_csr(rng, rows=50, cols=300_000, max_len=5,
                                       long_rows=[(3, 200_000), (40, 70_000)])
        return off, idx, vals, 300_000
    if name == "empty_rows":
        return np.zeros(1001, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32), 10
    from edge_loops_gb300 import synth
    o, i, v, _, cols = synth.power_law(rows=1 << 16, target_nnz=1_500_000, cap=40_000, seed=1)
    return o.numpy(), i.numpy(), v.numpy(), cols


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("row_weight", [1, 2])
def test_el_spmv_range_splits(cuda, oracle_mod, name, row_weight):
    from edge_loops_gb300 import api
    off, idx, vals, cols = _case(name)
    A = api.CSR.from_arrays(off, idx, vals, cols, device=cuda)
    x = torch.rand(cols, device=cuda)
    for max_ctas in (0, 1, 3):
        tr = _trace_run(lambda: api.spmv(A, x, schedule="merge_path_flat",
                                         row_weight=row_weight, max_ctas=max_ctas),
                        1 << 14, cuda)
        assert len(tr) >= 1
        if max_ctas:
            assert len(tr) <= 8 * max_ctas
        _check(oracle_mod, off, tr, row_weight)
    assert api.workspace_errors() == 0


@pytest.mark.parametrize("name", NAMES[::3])
def test_static_scratch_range_splits(cuda, oracle_mod, name):
    """el_spmv_static_scratch always takes the reference's equal split."""
    from edge_loops_gb300 import _lib, api
    off, idx, vals, cols = _case(name)
    A = api.CSR.from_arrays(off, idx, vals, cols, device=cuda)
    a = A.el()
    x = torch.rand(cols, device=cuda)
    y = torch.empty(A.rows, device=cuda)
    for ranges in (0, 1, 7):
        f = C.c_uint32(0)

        def run():
            _lib.check(_lib.lib().el_spmv_static_scratch(
                C.byref(a), C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), ranges,
                C.byref(f), C.c_void_p(torch.cuda.current_stream().cuda_stream)), "static")

        tr = _trace_run(run, 1 << 13, cuda)
        assert f.value == 0
        if ranges:
            assert len(tr) <= ranges
        _check(oracle_mod, off, tr, 1)


@pytest.mark.parametrize("name", ["random3", "power_law"])
def test_range_splits_with_512_nonzero_tiles(cuda, oracle_mod, name):
    """Tiles of 16 nonzeros per lane walk the same ranges."""
    from edge_loops_gb300 import api
    off, idx, vals, cols = _case(name)
    A = api.CSR.from_arrays(off, idx, vals, cols, device=cuda)
    x = torch.rand(cols, device=cuda)
    for w in (1, 2):
        tr = _trace_run(lambda: api.spmv(A, x, schedule="merge_path_flat", row_weight=w,
                                         nz_per_lane=16), 1 << 14, cuda)
        _check(oracle_mod, off, tr, w)
    assert api.workspace_errors() == 0
