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
