"""GPU parity of SpMM C = A B against the oracle, through the C ABI.

thread_mapped and group_mapped sum every C element in nonzero order with
separate FP32 roundings, so they are bit-identical to the reference loop
(algorithms/spmm/thread_mapped.cuh:41-52, restated in oracle.c); merge_path
splits long rows across warps and is held to the order-free FP32 bound."""
import numpy as np
import pytest
import torch

from conftest import load_golden, random_csr

pytestmark = pytest.mark.gpu


def dev(A_np, cols, cuda):
    from edge_loops_gb300.api import CSR
    off, idx, vals = A_np
    return CSR.from_arrays(off, idx, vals, cols, device=cuda)


def spmm(A, B, sched, cuda, **opts):
    from edge_loops_gb300 import api
    Cm = torch.full((A.rows, B.shape[1]), float("nan"), device=cuda)
    api.spmm(A, B, Cm, schedule=sched, **opts)
    flags = api.workspace_errors()
    return Cm.cpu().numpy(), flags


def bound_check(oracle_mod, off, idx, vals, Bnp, Cg, bdt=None):
    Bo = ("bf16", Bnp) if bdt == "bf16" else Bnp
    C64, Ca = oracle_mod.spmm_f64(off, idx, vals, Bo)
    u = 2.0 ** -24
    n = (np.diff(off.astype(np.int64)) + 2)[:, None]
    bound = (n * u / (1 - n * u)) * Ca
    err = np.abs(Cg.astype(np.float64) - C64)
    assert np.all(err <= bound), (np.max(err - bound), np.argmax(err - bound))


def test_chesapeake_exact(cuda, oracle_mod):
    g = load_golden("chesapeake.npz")
    A = dev((g["offsets"], g["indices"], g["values"]), 39, cuda)
    rng = np.random.default_rng(0)
    B = rng.integers(1, 11, size=(39, 10)).astype(np.float32)  # the reference example's n = 10
    exp = oracle_mod.spmm_f32(g["offsets"], g["indices"], g["values"], B)
    for sched in ("thread_mapped", "group_mapped", "merge_path_flat"):
        Cg, flags = spmm(A, torch.as_tensor(B, device=cuda), sched, cuda)
        assert flags == 0
        np.testing.assert_array_equal(Cg, exp)


@pytest.mark.parametrize("n", [1, 10, 32, 128, 200])
def test_ordered_schedules_bit_exact(cuda, oracle_mod, n):
    rng = np.random.default_rng(n)
    off, idx, vals, _ = random_csr(rng, rows=700, cols=900, max_len=40, empty_frac=0.1)
    B = rng.uniform(-1, 1, size=(900, n)).astype(np.float32)
    A = dev((off, idx, vals), 900, cuda)
    exp = oracle_mod.spmm_f32(off, idx, vals, B)
    for sched in ("thread_mapped", "group_mapped"):
        Cg, flags = spmm(A, torch.as_tensor(B, device=cuda), sched, cuda)
        assert flags == 0
        np.testing.assert_array_equal(Cg, exp)


@pytest.mark.parametrize("n", [32, 128, 160])
@pytest.mark.parametrize("bdt", ["f32", "bf16"])
def test_power_law_merge_path(cuda, oracle_mod, n, bdt):
    from edge_loops_gb300 import synth
    off, idx, vals, x, cols = synth.power_law(rows=1 << 14, target_nnz=250_000, cap=30_000,
                                              seed=3)
    off, idx, vals = off.numpy(), idx.numpy(), vals.numpy()
    rng = np.random.default_rng(1)
    B = torch.as_tensor(rng.uniform(-1, 1, size=(cols, n)).astype(np.float32), device=cuda)
    if bdt == "bf16":
        B = B.to(torch.bfloat16)
    A = dev((off, idx, vals), cols, cuda)
    for sched in ("merge_path_flat", "group_mapped"):
        Cg, flags = spmm(A, B, sched, cuda)
        assert flags == 0
        Bn = B.view(torch.int16).cpu().numpy().view(np.uint16) if bdt == "bf16" \
            else B.cpu().numpy()
        bound_check(oracle_mod, off, idx, vals, Bn, Cg, bdt)


def test_merge_path_long_rows_deterministic(cuda, oracle_mod):
    rng = np.random.default_rng(17)
    off, idx, vals, _ = random_csr(rng, rows=300, cols=200_000, max_len=30,
                                   long_rows=[(0, 150_000), (150, 90_000), (299, 100_000)])
    B = rng.uniform(-1, 1, size=(200_000, 64)).astype(np.float32)
    A = dev((off, idx, vals), 200_000, cuda)
    Bt = torch.as_tensor(B, device=cuda)
    C1, f1 = spmm(A, Bt, "merge_path_flat", cuda)
    C2, f2 = spmm(A, Bt, "merge_path_flat", cuda)
    assert f1 == 0 and f2 == 0
    np.testing.assert_array_equal(C1, C2)
    bound_check(oracle_mod, off, idx, vals, B, C1)


def test_bf16_values_with_scales(cuda, oracle_mod):
    from edge_loops_gb300 import synth
    off, idx, vals, x, rows = [t.numpy() if hasattr(t, "numpy") else t
                               for t in synth.stencil27(n=12, seed=2)]
    A = dev((off, idx, vals), rows, cuda).quantized(torch.bfloat16, per_row_scale=True)
    rng = np.random.default_rng(2)
    B = rng.uniform(-1, 1, size=(rows, 32)).astype(np.float32)
    qv = A.values.float().cpu().numpy()
    sc = A.row_scale.cpu().numpy()
    for sched in ("thread_mapped", "group_mapped", "merge_path_flat"):
        Cg, flags = spmm(A, torch.as_tensor(B, device=cuda), sched, cuda)
        assert flags == 0
        C64, Ca = oracle_mod.spmm_f64(off, idx, qv, B, row_scale=sc)
        n = (np.diff(off.astype(np.int64)) + 3)[:, None]
        assert np.all(np.abs(Cg - C64) <= n * 2.0 ** -24 * Ca * 1.001)
