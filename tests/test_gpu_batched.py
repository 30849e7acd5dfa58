"""GPU parity of the batched SpMV plan (many matrices, one persistent launch
captured in a CUDA graph), matrix by matrix against the oracle."""
import numpy as np
import pytest
import torch

from conftest import order_free_bound

pytestmark = pytest.mark.gpu


def make(cuda, count=96, rows_hi=4096, seed=4):
    from edge_loops_gb300 import api, synth
    R, off, idx, vals, x, rs, ns = synth.batched(count=count, rows_hi=rows_hi, seed=seed,
                                                 device=cuda)
    items, y = api.batched_items(R, off, idx, vals, x, rs, ns)
    return items, y


def check(oracle_mod, items, scale_of=None, vals_of=None):
    worst = 0.0
    for m, (A, x, y) in enumerate(items):
        if A.rows == 0:
            continue
        off = A.offsets.cpu().numpy()
        idx = A.indices.cpu().numpy()
        v = (vals_of(m) if vals_of else A.values).float().cpu().numpy()
        sc = None if A.row_scale is None else A.row_scale.cpu().numpy()
        y64, yabs = oracle_mod.spmv_f64(off, idx, v, x.cpu().numpy(), row_scale=sc)
        yy = y.cpu().numpy().astype(np.float64)
        bound = order_free_bound(off, yabs)
        assert np.all(np.abs(yy - y64) <= bound), m
        worst = max(worst, oracle_mod.error_metrics(yy, y64, yabs)[0])
    return worst


@pytest.mark.parametrize("use_graph", [True, False])
@pytest.mark.parametrize("tpr", [0, 1, 4, 32, 64])
def test_batched_f32(cuda, oracle_mod, use_graph, tpr):
    from edge_loops_gb300 import api
    items, y = make(cuda)
    y.fill_(float("nan"))
    plan = api.BatchPlan(items, use_graph=use_graph, force_threads_per_row=tpr)
    info = plan.info()
    assert info["heavy_matrices"] == 0 and info["work_items"] > 0
    if tpr == 64:
        assert info["matrices_nz_walk"] == len(items)
    plan.execute()
    assert plan.errors() == 0
    check(oracle_mod, items)
    y1 = y.clone()
    y.zero_()
    plan.execute()  # replay
    torch.cuda.synchronize()
    assert torch.equal(y, y1)


def test_batched_bf16_within_1e2_of_fp64(cuda, oracle_mod):
    from edge_loops_gb300 import api
    items, y = make(cuda, count=64, seed=5)
    qitems = [(A.quantized(torch.bfloat16, per_row_scale=True), x, yy) for A, x, yy in items]
    plan = api.BatchPlan(qitems)
    plan.execute()
    assert plan.errors() == 0
    check(oracle_mod, qitems)  # exact stored values: order-free FP32 bound
    worst = 0.0
    for (A, x, yy) in items:  # against FP64 of the FP32 matrices
        off = A.offsets.cpu().numpy()
        y64, yabs = oracle_mod.spmv_f64(off, A.indices.cpu().numpy(), A.values.cpu().numpy(),
                                        x.cpu().numpy())
        worst = max(worst, oracle_mod.error_metrics(yy.cpu().numpy(), y64, yabs)[0])
    assert worst <= 1e-2, worst


def test_heavy_empty_and_tiny_matrices(cuda, oracle_mod):
    from edge_loops_gb300 import api
    from conftest import random_csr
    rng = np.random.default_rng(3)
    mats = [random_csr(rng, rows=40, cols=30_000, max_len=20, long_rows=[(5, 20_000)]),
            (np.zeros(1, dtype=np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32),
             np.zeros(0, np.float32)),  # rows = 0
            (np.zeros(9, dtype=np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32),
             np.ones(3, np.float32)),  # no nonzeros
            random_csr(rng, rows=1, cols=1, max_len=1),
            random_csr(rng, rows=300, cols=200, max_len=60, empty_frac=0.5)]
    items = []
    for off, idx, vals, x in mats:
        A = api.CSR.from_arrays(off, idx, vals, len(x), device=cuda)
        items.append((A, torch.as_tensor(x, device=cuda),
                      torch.full((A.rows,), float("nan"), device=cuda)))
    plan = api.BatchPlan(items)
    assert plan.info()["heavy_matrices"] == 1
    plan.execute()
    assert plan.errors() == 0
    check(oracle_mod, items)


@pytest.mark.parametrize("entry", [16 | (11 << 8), 64 | (7 << 8), 2 | (14 << 8)])
def test_table_drives_configuration(cuda, oracle_mod, entry):
    from edge_loops_gb300 import api, _lib
    items, y = make(cuda, count=32)
    table = np.full(_lib.EL_BATCH_TABLE_SIZE, entry, dtype=np.int32)
    plan = api.BatchPlan(items, table=table)
    info = plan.info()
    if entry & 0xff == 64:
        assert info["matrices_nz_walk"] == 32
    else:
        assert info["matrices_by_threads_per_row"][entry & 0xff] == 32
    plan.execute()
    assert plan.errors() == 0
    check(oracle_mod, items)


def test_nz_walk_unaligned_and_ragged(cuda, oracle_mod):
    """Matrices whose indices/values start at every phase modulo 8 elements
    (the walk's 128-bit loads need a common phase; mismatched phases fall
    back to scalar loads), rows from empty to thousands of nonzeros, and
    items of 2^6 rows + nonzeros (many items per matrix)."""
    from edge_loops_gb300 import api
    from conftest import random_csr
    rng = np.random.default_rng(11)
    items = []
    keep = []
    for m in range(24):
        off, idx, vals, x = random_csr(rng, rows=int(rng.integers(1, 700)), cols=900,
                                       max_len=int(rng.integers(1, 80)), empty_frac=0.2)
        nnz = len(idx)
        si, sv = m % 8, (m * 3) % 8 if m % 3 else m % 8
        ib = torch.zeros(nnz + 16, dtype=torch.int32, device=cuda)
        vb = torch.zeros(nnz + 16, dtype=torch.float32, device=cuda)
        ib[si: si + nnz] = torch.as_tensor(idx, device=cuda)
        vb[sv: sv + nnz] = torch.as_tensor(vals, device=cuda)
        keep += [ib, vb]
        A = api.CSR(torch.as_tensor(off, device=cuda), ib[si: si + nnz], vb[sv: sv + nnz],
                    len(off) - 1, 900)
        items.append((A, torch.as_tensor(x, device=cuda),
                      torch.full((A.rows,), float("nan"), device=cuda)))
    for chunk in (6, 12):
        plan = api.BatchPlan(items, force_threads_per_row=64, force_chunk_log2=chunk)
        plan.execute()
        assert plan.errors() == 0
        check(oracle_mod, items)


def test_malformed_matrix_rejected(cuda):
    from edge_loops_gb300 import api, _lib
    items, y = make(cuda, count=8)
    A, x, yy = items[3]
    bad = A.offsets.clone()
    bad[5] = bad[-1] + 7
    items[3] = (api.CSR(bad, A.indices, A.values, A.rows, A.cols), x, yy)
    with pytest.raises(_lib.ElError) as e:
        api.BatchPlan(items)
    assert e.value.status == _lib.EL_ERR_MALFORMED_CSR
