"""The drop-in C++ header (include/edge_loops.hpp): compiles against the
reference's own container types (CPU; needs the reference sources, skipped
without them), and a reference-style C++ caller gives the oracle's results
on the GPU."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import REPO, load_golden
from oracle.ref import sources as ref_sources

NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
REF = ref_sources()


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "include", "loops")),
                    reason="reference sources not present")
def test_header_accepts_reference_containers(tmp_path):
    subprocess.run([NVCC] + ARCH + ["-std=c++17", "--expt-extended-lambda",
                                    "--expt-relaxed-constexpr", "-w", "-c",
                                    "-I", os.path.join(REF, "include"),
                                    "-I", os.path.join(REPO, "include"),
                                    os.path.join(REPO, "tests", "cpp", "reference_types.cu"),
                                    "-o", str(tmp_path / "rt.o")], check=True)


def build_driver(out_dir, built_lib):
    exe = os.path.join(out_dir, "compat_driver")
    subprocess.run([NVCC] + ARCH + ["-std=c++17", "-O2", "-I", os.path.join(REPO, "include"),
                                    os.path.join(REPO, "tests", "cpp", "compat_driver.cu"),
                                    built_lib, "-Xlinker",
                                    "-rpath=" + os.path.dirname(built_lib), "-o", exe],
                   check=True)
    return exe


def test_driver_compiles(tmp_path, built_lib):
    assert os.path.exists(build_driver(str(tmp_path), built_lib))


@pytest.mark.gpu
def test_driver_runs_reference_style_calls(tmp_path, built_lib, cuda, oracle_mod):
    g = load_golden("chesapeake.npz")
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        np.array([g["rows"], g["cols"], g["nnz"]], dtype=np.int64).tofile(f)
        g["offsets"].astype(np.int32).tofile(f)
        g["indices"].astype(np.int32).tofile(f)
        g["values"].astype(np.float32).tofile(f)
        np.array([len(g["x"])], dtype=np.int64).tofile(f)
        g["x"].astype(np.float32).tofile(f)
    exe = build_driver(str(tmp_path), built_lib)
    out = tmp_path / "out.bin"
    subprocess.run([exe, str(inp), str(out)], check=True)
    rows = int(g["rows"])
    data = np.fromfile(out, dtype=np.float32)
    ys = data[: 5 * rows].reshape(5, rows)
    for y in ys:
        np.testing.assert_array_equal(y, g["y_exact"].astype(np.float32))
    Cm = data[5 * rows:].reshape(rows, 3)
    for c in range(3):
        np.testing.assert_array_equal(Cm[:, c], g["y_exact"].astype(np.float32) * (c + 1))
