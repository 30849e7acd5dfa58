"""The edge (nonzero) partitioner and the SpMV over its tiles
(util/partitioner.hxx, schedule_edge/thread_mapped.hxx,
examples/spmv/thread_mapped_edge.cu) and the COO helpers (coo.hxx:90-122).

CPU: the oracle's partitioner equals the reference's own Partitioner
(golden fixtures made by tests/golden/make_golden.py from the reference's
header), rejects the sizes the reference rejects, and the C plan calls give
the reference's counts and argument errors.  GPU: the library's partitions
are bit-identical to the golden ones and to the oracle on larger inputs, the
COO sorts and row expansion are exact, and the edge SpMV is within the
FP32 order-free bound of FP64 with every quark processed by its tile.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden, order_free_bound

ARRAYS = ("quarks", "atom_begin", "atom_x", "atom_y", "tile_begin")


def golden_cases():
    g = load_golden("edge_partitions.npz")
    mats = {}
    for name in ("chesapeake", "random"):
        rows, cols = (int(v) for v in g[f"{name}_shape"])
        mats[name] = (rows, cols, g[f"{name}_row"], g[f"{name}_col"], g[f"{name}_val"])
    cases = []
    for i in range(int(g["num_cases"])):
        exp = {k: g[f"case{i}_{k}"] for k in ARRAYS + ("rows_sorted", "cols_sorted")}
        exp["atoms_x"], exp["atoms_y"] = int(g[f"case{i}_atoms_x"]), int(g[f"case{i}_atoms_y"])
        cases.append((str(g[f"case{i}_matrix"]), str(g[f"case{i}_mode"]),
                      tuple(int(v) for v in g[f"case{i}_sizes"]), exp))
    errors = [(str(g[f"error{i}_matrix"]), str(g[f"error{i}_mode"]),
               tuple(int(v) for v in g[f"error{i}_sizes"]))
              for i in range(int(g["num_errors"]))]
    return mats, cases, errors, g["errors_rejected"]


def oracle_partition(oracle_mod, rows, cols, ri, ci, mode, sizes):
    if mode == "coord":
        return oracle_mod.edge_partition_coordinate(rows, cols, ri, ci, *sizes)
    return oracle_mod.edge_partition_position(len(ri), *sizes)


def test_oracle_partition_equals_reference_golden(oracle_mod):
    mats, cases, _, _ = golden_cases()
    for name, mode, sizes, exp in cases:
        rows, cols, ri, ci, vv = mats[name]
        sr, sc, _ = oracle_mod.coo_sort(ri, ci, vv)
        np.testing.assert_array_equal(sr, exp["rows_sorted"])
        np.testing.assert_array_equal(sc, exp["cols_sorted"])
        got = oracle_partition(oracle_mod, rows, cols, sr, sc, mode, sizes)
        for k in ARRAYS:
            np.testing.assert_array_equal(got[k], exp[k], err_msg=f"{name} {mode} {sizes} {k}")
        assert (got["atoms_x"], got["atoms_y"]) == (exp["atoms_x"], exp["atoms_y"])


def test_oracle_rejects_what_the_reference_rejects(oracle_mod):
    mats, _, errors, rejected = golden_cases()
    assert rejected.all()
    for name, mode, sizes in errors:
        rows, cols, ri, ci, _ = mats[name]
        with pytest.raises(ValueError):
            oracle_partition(oracle_mod, rows, cols, ri, ci, mode, sizes)


def plan(L, rows, cols, nnz, mode, sizes):
    P = L.ElEdgePartition()
    if mode == "coord":
        st = L.lib().el_edge_partition_coordinate_plan(rows, cols, nnz, *sizes, C.byref(P))
    else:
        st = L.lib().el_edge_partition_position_plan(nnz, *sizes, C.byref(P))
    return st, P


def test_plan_counts_and_argument_errors(built_lib):
    """Host-only C calls: counts equal the reference's, bad sizes refused."""
    from edge_loops_gb300 import _lib as L
    mats, cases, errors, _ = golden_cases()
    for name, mode, sizes, exp in cases:
        rows, cols, ri, _, _ = mats[name]
        st, P = plan(L, rows, cols, len(ri), mode, sizes)
        assert st == L.EL_OK
        assert P.num_atoms == len(exp["atom_x"]) and P.num_tiles == len(exp["tile_begin"]) - 1
        assert (P.atoms_x, P.atoms_y) == (exp["atoms_x"], exp["atoms_y"])
    for name, mode, sizes in errors:
        rows, cols, ri, _, _ = mats[name]
        assert plan(L, rows, cols, len(ri), mode, sizes)[0] == L.EL_ERR_INVALID_ARGUMENT
    assert plan(L, 10, 10, 50, "pos", (5, 0))[0] == L.EL_ERR_INVALID_ARGUMENT
    assert plan(L, 10, 10, 50, "pos", (-1, 1))[0] == L.EL_ERR_INVALID_ARGUMENT
    assert plan(L, 0, 10, 0, "coord", (1, 1, 1, 1))[0] == L.EL_ERR_INVALID_ARGUMENT
    assert plan(L, 10, 10, 1 << 31, "pos", (5, 1))[0] == L.EL_ERR_OVERFLOW
    # more than 2^31 - 1 atoms
    assert plan(L, 1 << 20, 1 << 20, 10, "coord", (1, 1, 1, 1))[0] == L.EL_ERR_OVERFLOW


# ---- GPU -------------------------------------------------------------------

def device_coo(edge, rows, cols, ri, ci, vv):
    return edge.COO.from_arrays(rows, cols, ri, ci, vv, device="cuda")


def gpu_partition(edge, A, mode, sizes):
    part = edge.Partitioner(A)
    if mode == "coord":
        part.partition_atoms_coordinate_space(*sizes[:2])
        part.partition_tiles_coordinate_space(*sizes[2:])
    else:
        part.partition_atoms_position_space(sizes[0])
        part.partition_tiles_position_space(sizes[1])
    part.prepare_gpu()
    return part


@pytest.mark.gpu
def test_gpu_partition_equals_reference_golden(cuda):
    from edge_loops_gb300 import edge
    mats, cases, _, _ = golden_cases()
    for name, mode, sizes, exp in cases:
        A = device_coo(edge, *mats[name])
        part = gpu_partition(edge, A, mode, sizes)
        np.testing.assert_array_equal(A.row_indices.cpu().numpy(), exp["rows_sorted"])
        np.testing.assert_array_equal(A.col_indices.cpu().numpy(), exp["cols_sorted"])
        arr = part.get_work_tiles()
        for k in ARRAYS:
            np.testing.assert_array_equal(arr[k].cpu().numpy(), exp[k],
                                          err_msg=f"{name} {mode} {sizes} {k}")
        assert (part.P.atoms_x, part.P.atoms_y) == (exp["atoms_x"], exp["atoms_y"])
        assert part.get_num_tiles() == len(exp["tile_begin"]) - 1


def random_coo(rng, rows, cols, nnz, dup_every=0):
    ri = rng.integers(0, rows, nnz).astype(np.int32)
    ci = rng.integers(0, cols, nnz).astype(np.int32)
    if dup_every:
        ri[1::dup_every] = ri[0::dup_every][: len(ri[1::dup_every])]
        ci[1::dup_every] = ci[0::dup_every][: len(ci[1::dup_every])]
    return ri, ci, rng.uniform(-1, 1, nnz).astype(np.float32)


@pytest.mark.gpu
def test_gpu_partition_equals_oracle_larger(cuda, oracle_mod):
    from edge_loops_gb300 import edge
    rng = np.random.default_rng(23)
    rows, cols = 5003, 4001
    ri, ci, vv = random_coo(rng, rows, cols, 60000, dup_every=9)
    ri[:3000] = 17  # one long row
    sr, sc, _ = oracle_mod.coo_sort(ri, ci, vv)
    for mode, sizes in [("coord", (7, 9, 5, 3)), ("coord", (64, 4001, 3, 1)),
                        ("coord", (1, 1000, 97, 4)), ("coord", (5003, 1, 1, 4001)),
                        ("pos", (256, 1)), ("pos", (33, 17)), ("pos", (59999, 2))]:
        A = device_coo(edge, rows, cols, ri, ci, vv)
        part = gpu_partition(edge, A, mode, sizes)
        exp = oracle_partition(oracle_mod, rows, cols, sr, sc, mode, sizes)
        arr = part.get_work_tiles()
        for k in ARRAYS:
            np.testing.assert_array_equal(arr[k].cpu().numpy(), exp[k],
                                          err_msg=f"{mode} {sizes} {k}")


@pytest.mark.gpu
def test_gpu_partition_errors(cuda):
    from edge_loops_gb300 import _lib as L, edge
    mats, _, errors, _ = golden_cases()
    for name, mode, sizes in errors:
        A = device_coo(edge, *mats[name])
        part = edge.Partitioner(A)
        with pytest.raises(L.ElError) as e:
            if mode == "coord":
                part.partition_atoms_coordinate_space(*sizes[:2])
                part.partition_tiles_coordinate_space(*sizes[2:])
            else:
                part.partition_atoms_position_space(sizes[0])
                part.partition_tiles_position_space(sizes[1])
        assert e.value.status == L.EL_ERR_INVALID_ARGUMENT
    # arrays planned for other sizes are refused
    rows, cols, ri, ci, vv = mats["random"]
    A = device_coo(edge, rows, cols, ri, ci, vv)
    st, P = plan(L, rows, cols, len(ri), "coord", (16, 16, 3, 2))
    part = edge.Partitioner(A)
    part._alloc(P)
    c = A.el()
    assert L.lib().el_edge_partition_coordinate(None, C.byref(c), 16, 16, 2, 2, C.byref(P),
                                                None) == L.EL_ERR_INVALID_ARGUMENT
    # an entry outside the matrix
    bad = device_coo(edge, rows, cols, np.where(np.arange(len(ri)) == 5, rows, ri), ci, vv)
    part = edge.Partitioner(bad, sort=False)
    part.partition_atoms_coordinate_space(16, 16)
    with pytest.raises(L.ElError) as e:
        part.partition_tiles_coordinate_space(3, 2)
    assert e.value.status == L.EL_ERR_MALFORMED_CSR


@pytest.mark.gpu
def test_gpu_coo_sort(cuda, oracle_mod):
    import torch
    from edge_loops_gb300 import edge
    rng = np.random.default_rng(31)
    for rows, cols, nnz in [(1000, 700, 20000), (1, 5, 40), (3000, 1, 500), (7, 9, 1)]:
        ri, ci, vv = random_coo(rng, rows, cols, nnz, dup_every=4)
        for by_column in (False, True):
            A = device_coo(edge, rows, cols, ri, ci, vv)
            (A.sort_by_column if by_column else A.sort_by_row)()
            er, ec, ev = oracle_mod.coo_sort(ri, ci, vv, by_column=by_column)
            np.testing.assert_array_equal(A.row_indices.cpu().numpy(), er)
            np.testing.assert_array_equal(A.col_indices.cpu().numpy(), ec)
            np.testing.assert_array_equal(A.values.cpu().numpy(), ev)
    empty = edge.COO(5, 5, torch.zeros(0, dtype=torch.int32, device="cuda"),
                     torch.zeros(0, dtype=torch.int32, device="cuda"),
                     torch.zeros(0, dtype=torch.float32, device="cuda"))
    empty.sort_by_row()


@pytest.mark.gpu
def test_gpu_csr_row_indices(cuda):
    from conftest import random_csr
    from edge_loops_gb300 import api, edge
    rng = np.random.default_rng(37)
    for off, idx, vals, x in [random_csr(rng, rows=3000, cols=2000, max_len=30, empty_frac=0.4,
                                         long_rows=[(5, 1900)]),
                              random_csr(rng, rows=50, cols=10, max_len=0)]:
        A = api.CSR.from_arrays(off, idx, vals, len(x), device="cuda")
        coo = edge.COO.from_csr(A)
        np.testing.assert_array_equal(coo.row_indices.cpu().numpy(),
                                      np.repeat(np.arange(len(off) - 1), np.diff(off)))


def quark_tiles(arr):
    """The tile each quark belongs to, from the partition arrays."""
    q, ab, tb = (arr[k].cpu().numpy() for k in ("quarks", "atom_begin", "tile_begin"))
    out = np.full(len(q), -1, dtype=np.int64)
    for t in range(len(tb) - 1):
        out[q[ab[tb[t]]:ab[tb[t + 1]]]] = t
    return out


@pytest.mark.gpu
def test_gpu_spmv_edge(cuda, oracle_mod):
    import torch
    from edge_loops_gb300 import edge
    rng = np.random.default_rng(43)
    rows, cols = 4000, 3000
    ri, ci, vv = random_coo(rng, rows, cols, 50000, dup_every=11)
    ri[:4000] = 123  # a long row
    ri[ri == 7] = 8  # an empty row
    x = rng.uniform(-1, 1, cols).astype(np.float32)
    sr, sc, sv = oracle_mod.coo_sort(ri, ci, vv)
    off = np.searchsorted(sr, np.arange(rows + 1)).astype(np.int32)
    y64, yabs = oracle_mod.spmv_f64(off, sc, sv, x)
    bound = order_free_bound(off, yabs, extra=8)
    xd = torch.from_numpy(x).cuda()
    for mode, sizes in [("coord", (16, 64, 4, 2)), ("coord", (1, 3000, 1, 1)),
                        ("coord", (4000, 3000, 1, 1)), ("pos", (32, 1)), ("pos", (500, 3))]:
        A = device_coo(edge, rows, cols, ri, ci, vv)
        part = gpu_partition(edge, A, mode, sizes)
        y = torch.full((rows,), float("nan"), device="cuda")
        y, qt = edge.spmv_edge(A, part, xd, y, track=True)
        got = y.cpu().numpy().astype(np.float64)
        assert np.all(np.abs(got - y64) <= bound), (mode, sizes)
        np.testing.assert_array_equal(qt.cpu().numpy(), quark_tiles(part.get_work_tiles()))
    # no nonzeros: y is zero
    A0 = edge.COO(6, 4, torch.zeros(0, dtype=torch.int32, device="cuda"),
                  torch.zeros(0, dtype=torch.int32, device="cuda"),
                  torch.zeros(0, dtype=torch.float32, device="cuda"))
    p0 = gpu_partition(edge, A0, "coord", (2, 2, 1, 1))
    y0 = edge.spmv_edge(A0, p0, torch.ones(4, device="cuda"),
                        torch.full((6,), 5.0, device="cuda"))
    assert torch.count_nonzero(y0).item() == 0
