"""The device-side load-balanced loop API (include/edge_loops_device.cuh):
a user driver written with it compiles (CPU, cross-compiled for sm_103a),
and on the GPU its merge ranges visit every nonzero once and close every
row once, its warp search equals the sequential search at every diagonal,
its thread-mapped SpMV equals the reference's CPU loop bit for bit, and its
merge-range SpMV (partial rows by atomics) is within the FP32 bound."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import REPO, order_free_bound, random_csr

NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def build_driver(out_dir):
    exe = os.path.join(out_dir, "device_api_driver")
    subprocess.run([NVCC] + ARCH + ["-std=c++17", "-O2", "--extended-lambda",
                                    "-I", os.path.join(REPO, "include"),
                                    os.path.join(REPO, "tests", "cpp", "device_api_driver.cu"),
                                    "-o", exe], check=True)
    return exe


def test_device_api_driver_compiles(tmp_path):
    assert os.path.exists(build_driver(str(tmp_path)))


def run_driver(exe, tmp_path, off, idx, vals, x):
    inp = tmp_path / "in.bin"
    rows = len(off) - 1
    with open(inp, "wb") as f:
        np.array([rows, len(x), len(idx)], dtype=np.int64).tofile(f)
        off.astype(np.int32).tofile(f)
        idx.astype(np.int32).tofile(f)
        vals.astype(np.float32).tofile(f)
        np.array([len(x)], dtype=np.int64).tofile(f)
        x.astype(np.float32).tofile(f)
    out = tmp_path / "out.bin"
    subprocess.run([exe, str(inp), str(out)], check=True)
    raw = np.fromfile(out, dtype=np.uint8)
    n = 4 * rows
    y = raw[0:n].view(np.float32)
    count = raw[n:2 * n].view(np.int32)
    ends = raw[2 * n:3 * n].view(np.int32)
    y_rows = raw[3 * n:4 * n].view(np.float32)
    mis = int(raw[4 * n:4 * n + 4].view(np.int32)[0])
    return y, count, ends, y_rows, mis


@pytest.mark.gpu
def test_device_api_loops(tmp_path, cuda, oracle_mod):
    exe = build_driver(str(tmp_path))
    rng = np.random.default_rng(41)
    cases = [random_csr(rng, rows=5000, cols=3000, max_len=40, empty_frac=0.3,
                        long_rows=[(17, 2500), (4999, 1800)]),
             random_csr(rng, rows=1, cols=100000, max_len=0, long_rows=[(0, 90000)]),
             random_csr(rng, rows=300, cols=10, max_len=0)]  # no nonzeros at all
    for off, idx, vals, x in cases:
        y, count, ends, y_rows, mis = run_driver(exe, tmp_path, off, idx, vals, x)
        np.testing.assert_array_equal(count, np.diff(off))
        np.testing.assert_array_equal(ends, np.ones(len(off) - 1, dtype=np.int32))
        assert mis == 0
        np.testing.assert_array_equal(y_rows, oracle_mod.spmv_f32(off, idx, vals, x))
        y64, yabs = oracle_mod.spmv_f64(off, idx, vals, x)
        bound = order_free_bound(off, yabs, extra=64)
        assert np.all(np.abs(y.astype(np.float64) - y64) <= bound)


def build_edge_driver(out_dir):
    exe = os.path.join(out_dir, "edge_tiles_driver")
    subprocess.run([NVCC] + ARCH + ["-std=c++17", "-O2", "--extended-lambda",
                                    "-I", os.path.join(REPO, "include"),
                                    os.path.join(REPO, "tests", "cpp", "edge_tiles_driver.cu"),
                                    "-o", exe], check=True)
    return exe


def test_edge_tiles_driver_compiles(tmp_path):
    assert os.path.exists(build_edge_driver(str(tmp_path)))


@pytest.mark.gpu
def test_edge_tiles_loop(tmp_path, cuda, oracle_mod):
    """for_each_tile_quark over partitions the library built: every quark
    visited once, by its own tile; y within the FP32 bound."""
    from edge_loops_gb300 import edge
    exe = build_edge_driver(str(tmp_path))
    rng = np.random.default_rng(47)
    rows, cols, nnz = 2000, 1500, 30000
    ri = rng.integers(0, rows, nnz).astype(np.int32)
    ci = rng.integers(0, cols, nnz).astype(np.int32)
    vv = rng.uniform(-1, 1, nnz).astype(np.float32)
    x = rng.uniform(-1, 1, cols).astype(np.float32)
    for mode, sizes in [("coord", (32, 100, 3, 2)), ("pos", (40, 5))]:
        A = edge.COO.from_arrays(rows, cols, ri, ci, vv, device="cuda")
        part = edge.Partitioner(A)
        if mode == "coord":
            part.partition_atoms_coordinate_space(*sizes[:2])
            part.partition_tiles_coordinate_space(*sizes[2:])
        else:
            part.partition_atoms_position_space(sizes[0])
            part.partition_tiles_position_space(sizes[1])
        arr = {k: v.cpu().numpy() for k, v in part.get_work_tiles().items()}
        sr, sc, sv = (t.cpu().numpy() for t in (A.row_indices, A.col_indices, A.values))
        inp = tmp_path / "edge_in.bin"
        with open(inp, "wb") as f:
            np.array([rows, cols, nnz, len(arr["atom_x"]), len(arr["tile_begin"]) - 1],
                     dtype=np.int64).tofile(f)
            for a in (sr, sc, sv, x, arr["quarks"], arr["atom_begin"], arr["tile_begin"]):
                a.tofile(f)
        out = tmp_path / "edge_out.bin"
        subprocess.run([exe, str(inp), str(out)], check=True)
        raw = np.fromfile(out, dtype=np.uint8)
        y = raw[:4 * rows].view(np.float32)
        tile = raw[4 * rows:4 * rows + 4 * nnz].view(np.int32)
        visits = raw[4 * rows + 4 * nnz:].view(np.int32)
        np.testing.assert_array_equal(visits, np.ones(nnz, dtype=np.int32))
        exp = np.empty(nnz, dtype=np.int64)
        q, ab, tb = arr["quarks"], arr["atom_begin"], arr["tile_begin"]
        for t in range(len(tb) - 1):
            exp[q[ab[tb[t]]:ab[tb[t + 1]]]] = t
        np.testing.assert_array_equal(tile, exp)
        off = np.searchsorted(sr, np.arange(rows + 1)).astype(np.int32)
        y64, yabs = oracle_mod.spmv_f64(off, sc, sv, x)
        assert np.all(np.abs(y.astype(np.float64) - y64) <= order_free_bound(off, yabs, extra=8))
