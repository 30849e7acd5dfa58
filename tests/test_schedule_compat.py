"""The reference's device-side schedule API (include/edge_loops_schedule.cuh):
a user driver written the way the reference documents its load-balancing
API (loops::schedule::setup for thread_mapped, work_oriented, warp_mapped
and block_mapped, grid_stride_range) compiles against this header, and the
very same source compiles against the reference's own schedule headers
(where their sources are present), so the two interfaces agree.  CPU only:
nvcc cross-compiles for sm_103a."""
import os
import shutil
import subprocess

import pytest

from conftest import REPO

NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
REF = os.environ.get("LOOPS_REF", "/root/reference")
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
