"""Parity at the benchmark sizes: the default merge-path SpMV on the 16M-
nonzero power-law matrix and on the 109M-nonzero 27-point stencil (FP32, and
BF16 values with per-row scales), and the merge-path SpMM on the 8M-nonzero
power-law matrix, against the FP64 oracle.  Every output row is checked (the
SpMM: 2048 sampled rows of C), with the bound that holds for any summation
order of FP32 products; the BF16 stencil also within 1e-2 of FP64 of the FP32
matrix, the mixed-precision error budget."""
import numpy as np
import pytest
import torch

from conftest import order_free_bound

pytestmark = pytest.mark.gpu


def _host(*ts):
    return [t.cpu().numpy() for t in ts]


def _check_rows(oracle_mod, off, idx, vals, x, y, scale=None):
    y64, yabs = oracle_mod.spmv_f64(off, idx, vals, x, row_scale=scale)
    err = np.abs(y.astype(np.float64) - y64)
    bad = np.nonzero(err > order_free_bound(off, yabs))[0]
    assert len(bad) == 0, f"{len(bad)} rows outside the bound, first {bad[:5]}"
    return oracle_mod.error_metrics(y, y64, yabs)


def test_power_law_16M_default_spmv(cuda, oracle_mod):
    from edge_loops_gb300 import api, synth
    off, idx, vals, x, cols = synth.power_law(rows=1 << 20, target_nnz=16_000_000,
                                              exponent=2.0, cap=100_000, seed=1, device=cuda)
    A = api.CSR(off, idx, vals, off.numel() - 1, cols)
    ws = api.Workspace()
    y1 = api.spmv(A, x, torch.full((A.rows,), float("nan"), device=cuda), workspace=ws)
    y2 = api.spmv(A, x, torch.zeros(A.rows, device=cuda), workspace=ws)
    torch.cuda.synchronize()
    assert ws.errors() == 0
    assert torch.equal(y1, y2)  # deterministic: the same bits from any prior y
    o, i, v, xh, yh = _host(off, idx, vals, x, y1)
    comp, _ = _check_rows(oracle_mod, o, i, v, xh, yh)
    assert comp < 1e-5


def test_stencil160_f32_and_bf16(cuda, oracle_mod):
    from edge_loops_gb300 import api, synth
    off, idx, vals, x, rows = synth.stencil27(n=160, seed=2, device=cuda)
    assert idx.numel() == 109_215_352
    A = api.CSR(off, idx, vals, rows, rows)
    ws = api.Workspace()
    y = api.spmv(A, x, workspace=ws)
    torch.cuda.synchronize()
    assert ws.errors() == 0
    o, i, v, xh, yh = _host(off, idx, vals, x, y)
    _check_rows(oracle_mod, o, i, v, xh, yh)
    del y, yh

    Q = A.quantized(torch.bfloat16, per_row_scale=True)
    yq = api.spmv(Q, x, workspace=ws)
    torch.cuda.synchronize()
    assert ws.errors() == 0
    qv, sc, yqh = _host(Q.values.float(), Q.row_scale, yq)
    _check_rows(oracle_mod, o, i, qv, xh, yqh, scale=sc)
    # against FP64 of the FP32 matrix: the BF16 storage error, per row
    # relative to sum |a x|
    y64, yabs = oracle_mod.spmv_f64(o, i, v, xh)
    comp, _ = oracle_mod.error_metrics(yqh, y64, yabs)
    assert comp <= 1e-2, comp


def test_spmm_power_law_8M_n32(cuda, oracle_mod):
    from edge_loops_gb300 import api, synth
    off, idx, vals, x, cols = synth.power_law(rows=1 << 20, target_nnz=8_000_000, exponent=2.0,
                                              cap=100_000, seed=3, device=cuda)
    A = api.CSR(off, idx, vals, off.numel() - 1, cols)
    g = torch.Generator(device=cuda)
    g.manual_seed(33)
    B = torch.rand(cols, 32, generator=g, device=cuda) * 2 - 1
    ws = api.Workspace()
    Cm = api.spmm(A, B, torch.full((A.rows, 32), float("nan"), device=cuda), workspace=ws)
    torch.cuda.synchronize()
    assert ws.errors() == 0
    rng = np.random.default_rng(0)
    rows_s = np.sort(rng.choice(A.rows, 2048, replace=False))
    o, i, v = _host(off, idx, vals)
    lens = o[rows_s + 1] - o[rows_s]
    so = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    sel = np.concatenate([np.arange(o[r], o[r + 1]) for r in rows_s])
    C64, Ca = oracle_mod.spmm_f64(so, i[sel], v[sel], B.cpu().numpy())
    got = Cm[torch.as_tensor(rows_s, device=cuda)].cpu().numpy().astype(np.float64)
    n = (np.diff(so.astype(np.int64)) + 2)[:, None]
    bound = (n * 2.0 ** -24 / (1 - n * 2.0 ** -24)) * Ca
    assert int(np.sum(np.abs(got - C64) > bound)) == 0
