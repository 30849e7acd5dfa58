"""The reference's own SpMV kernels, compiled from its headers into a cubin
(oracle/ref/build_ref.sh) and run on the GPU (oracle/ref/ref_gpu.py), against
this library on the same inputs: every reference kernel and every schedule
of the library lands within the FP32 order-free bound of the FP64 oracle, so
the two agree within twice that bound.  Skipped where the cubin was not
built (it needs the reference sources)."""
import numpy as np
import pytest

from conftest import order_free_bound, random_csr


@pytest.mark.gpu
def test_reference_kernels_agree_with_the_library(cuda, oracle_mod):
    import torch
    from edge_loops_gb300 import api
    from oracle.ref import ref_gpu
    if not ref_gpu.available():
        pytest.skip("oracle/_ref/ref_kernels.cubin not built (needs the reference sources)")
    R = ref_gpu.RefKernels()
    rng = np.random.default_rng(61)
    cases = [random_csr(rng, rows=20000, cols=9000, max_len=60, empty_frac=0.2,
                        long_rows=[(3, 8000), (19999, 5000)]),
             random_csr(rng, rows=300, cols=300, max_len=12)]
    for off, idx, vals, x in cases:
        A = api.CSR.from_arrays(off, idx, vals, len(x), device="cuda")
        xd = torch.from_numpy(x).cuda()
        y64, yabs = oracle_mod.spmv_f64(off, idx, vals, x)
        bound = order_free_bound(off, yabs)
        P = [ref_gpu.pad(t) for t in (A.offsets, A.indices, A.values, xd)]
        y = ref_gpu.pad(torch.empty(A.rows, device="cuda"))
        for sched in ("merge_path_flat", "thread_mapped", "group_mapped", "original"):
            ref = R.launch(sched, A.rows, A.cols, A.nnz, *P, y).cpu().numpy().astype(np.float64)
            assert np.all(np.abs(ref - y64) <= bound), sched
            mine_sched = "thread_mapped" if sched == "original" else sched
            mine = api.spmv(A, xd, schedule=mine_sched).cpu().numpy().astype(np.float64)
            assert np.all(np.abs(mine - ref) <= 2 * bound), sched
        # the reference's work_oriented kernel races at block boundaries
        # (a row split between blocks may be stored over an atomic add);
        # the library's work_oriented is within the bound everywhere
        mine = api.spmv(A, xd, schedule="work_oriented").cpu().numpy().astype(np.float64)
        assert np.all(np.abs(mine - y64) <= bound)


@pytest.mark.gpu
def test_reference_spmm_agrees_with_the_library(cuda, oracle_mod):
    import torch
    from edge_loops_gb300 import api
    from oracle.ref import ref_gpu
    if not ref_gpu.available():
        pytest.skip("oracle/_ref/ref_kernels.cubin not built (needs the reference sources)")
    R = ref_gpu.RefKernels()
    rng = np.random.default_rng(67)
    off, idx, vals, _ = random_csr(rng, rows=3000, cols=2000, max_len=30, empty_frac=0.2,
                                   long_rows=[(11, 1900)])
    A = api.CSR.from_arrays(off, idx, vals, 2000, device="cuda")
    for n in (1, 7, 32):
        B = torch.from_numpy(rng.uniform(-1, 1, (2000, n)).astype(np.float32)).cuda()
        P = [ref_gpu.pad(t) for t in (A.offsets, A.indices, A.values)]
        Cr = torch.empty(A.rows, n, device="cuda")
        R.spmm(A.rows, A.cols, A.nnz, *P, B, Cr)
        ref = Cr.cpu().numpy().astype(np.float64)
        c64, cabs = oracle_mod.spmm_f64(off, idx, vals, B.cpu().numpy())
        lens = np.diff(off).astype(np.float64)[:, None]
        bound = (lens + 2) * 2.0 ** -24 / (1 - (lens + 2) * 2.0 ** -24) * cabs
        assert np.all(np.abs(ref - c64) <= bound), n
        for sched in ("thread_mapped", "group_mapped", "merge_path_flat"):
            mine = api.spmm(A, B, schedule=sched).cpu().numpy().astype(np.float64)
            assert np.all(np.abs(mine - c64) <= bound), (n, sched)
