"""The reference's device-side schedule API (include/edge_loops_schedule.cuh):
a user driver written the way the reference documents its load-balancing
API (loops::schedule::setup for thread_mapped, work_oriented, warp_mapped,
block_mapped and merge_path_flat, grid_stride_range) compiles against this
header, and the very same source compiles against the reference's own
schedule headers (where their sources are present), so the two interfaces
agree (CPU: nvcc cross-compiles for sm_103a).  On a GPU the driver runs and
its outputs are checked against the oracle."""
import os
import shutil
import subprocess

import pytest

from conftest import REPO
from oracle.ref import sources as ref_sources

NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
REF = ref_sources()
DRIVER = os.path.join(REPO, "tests", "cpp", "schedule_compat_driver.cu")


def test_driver_compiles_against_this_header(tmp_path):
    exe = tmp_path / "schedule_compat_driver"
    subprocess.run([NVCC] + ARCH + ["-std=c++17", "-O2", "-I", os.path.join(REPO, "include"),
                                    DRIVER, "-o", str(exe)], check=True)
    assert exe.exists()


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "include", "loops")),
                    reason="reference sources not present")
def test_same_driver_compiles_against_the_reference_headers(tmp_path):
    # a header of the same name that pulls in the reference's schedule API
    shim = tmp_path / "inc"
    shim.mkdir()
    (shim / "edge_loops_schedule.cuh").write_text(
        "#pragma once\n#include <thrust/device_vector.h>\n#include <loops/error.hxx>\n"
        "#include <loops/util/math.hxx>\n#include <loops/util/launch.hxx>\n"
        "#include <loops/stride_ranges.hxx>\n#include <loops/schedule.hxx>\n")
    subprocess.run([NVCC] + ARCH + ["-std=c++17", "--expt-extended-lambda",
                                    "--expt-relaxed-constexpr", "-w", "-c",
                                    "-I", str(shim), "-I", os.path.join(REF, "include"),
                                    DRIVER, "-o", str(tmp_path / "drv.o")], check=True)


def _write_case(path, off, idx, vals, x, cols):
    import numpy as np
    with open(path, "wb") as f:
        np.array([len(off) - 1, cols, len(idx)], dtype=np.int64).tofile(f)
        np.asarray(off, np.int32).tofile(f)
        np.asarray(idx, np.int32).tofile(f)
        np.asarray(vals, np.float32).tofile(f)
        np.array([cols], dtype=np.int64).tofile(f)
        np.asarray(x, np.float32).tofile(f)


def _gpu_cases():
    import numpy as np
    from conftest import load_golden, random_csr
    g = load_golden("chesapeake.npz")
    rng = np.random.default_rng(5)
    yield "chesapeake", g["offsets"], g["indices"], g["values"], \
        rng.integers(1, 9, 39).astype(np.float32), 39
    # empty rows, one long row, a row count that is not a multiple of 128
    off, idx, vals, x = random_csr(rng, rows=1001, cols=50_000, max_len=30, empty_frac=0.3,
                                   long_rows=[(17, 40_000), (600, 3_000)])
    yield "edge_rows", off, idx, vals, x, 50_000
    from edge_loops_gb300 import synth
    o, i, v, xx, cols = synth.power_law(rows=5000, target_nnz=120_000, cap=20_000, seed=9)
    yield "power_law", o.numpy(), i.numpy(), v.numpy(), xx.numpy(), cols


@pytest.fixture(scope="module")
def driver_exe(tmp_path_factory):
    exe = tmp_path_factory.mktemp("drv") / "schedule_compat_driver"
    subprocess.run([NVCC] + ARCH + ["-std=c++17", "-O2", "-I", os.path.join(REPO, "include"),
                                    DRIVER, "-o", str(exe)], check=True)
    return str(exe)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["chesapeake", "edge_rows", "power_law"])
def test_driver_runs_on_gpu(tmp_path, cuda, oracle_mod, driver_exe, name):
    """The user kernels of the driver, run: every schedule's y within the
    order-free FP32 bound of the FP64 oracle, every nonzero visited once by
    block_mapped, z = 2 x + 1 exactly, and every merge_path_flat thread's
    start point from init() equal to the reference's per-thread split
    (schedule/merge_path_flat.hxx:321-385, restated in the oracle) bit for
    bit."""
    import numpy as np
    from conftest import order_free_bound
    off, idx, vals, x, cols = next(c[1:] for c in _gpu_cases() if c[0] == name)
    rows, nnz = len(off) - 1, len(idx)
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    _write_case(inp, off, idx, vals, x, cols)
    subprocess.run([driver_exe, str(inp), str(out)], check=True, timeout=120)
    raw = np.fromfile(out, dtype=np.uint8)
    pos = 0

    def take(n, dt):
        nonlocal pos
        a = raw[pos: pos + 4 * n].view(dt)
        pos += 4 * n
        return a

    ys = [take(rows, np.float32) for _ in range(4)]
    visits = take(nnz, np.int32)
    z = take(cols, np.float32)
    ys.append(take(rows, np.float32))
    tiles = -(-(rows + nnz) // 640)
    coords = take(tiles * 128 * 2, np.uint32).reshape(tiles, 128, 2)
    assert pos == len(raw)
    y64, yabs = oracle_mod.spmv_f64(off, idx, vals, x)
    bound = order_free_bound(off, yabs)
    for k, y in zip(("thread_mapped", "work_oriented", "warp_mapped", "block_mapped",
                     "merge_path_flat"), ys):
        err = np.abs(y.astype(np.float64) - y64)
        assert np.all(err <= bound), (k, int(np.argmax(err - bound)))
    np.testing.assert_array_equal(visits, np.ones(nnz, np.int32))
    np.testing.assert_array_equal(z, (np.float32(2) * x + np.float32(1)).astype(np.float32))
    exp = oracle_mod.merge_path_thread_coords(off, nnz, 128, 5)
    np.testing.assert_array_equal(coords, exp)
