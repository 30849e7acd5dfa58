"""Parity at the benchmark sizes: the default merge-path SpMV on the 16M-
nonzero power-law matrix and on the 109M-nonzero 27-point stencil (FP32, and
BF16 and FP16 values with per-row scales), the schedule el_spmv_select picks
for the stencil (bit for bit), the merge-path and group_mapped
SpMM on the 8M-nonzero power-law matrix (n = 32 and 128, FP32 and BF16 B),
and the batched plan over 4096 matrices (~310M nonzeros, FP32 and BF16),
against the FP64 oracle.  Every output row is checked (the SpMM: 2048
sampled rows of C), with the bound that holds for any summation order of
FP32 products; the 16-bit runs also within 1e-2 of FP64 of the FP32 matrix,
the mixed-precision error budget."""
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


def test_stencil160_f32_bf16_f16(cuda, oracle_mod):
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
    y64, yabs = oracle_mod.spmv_f64(o, i, v, xh)

    for dt in (torch.bfloat16, torch.float16):
        Q = A.quantized(dt, per_row_scale=True)
        yq = api.spmv(Q, x, workspace=ws)
        torch.cuda.synchronize()
        assert ws.errors() == 0
        qv, sc, yqh = _host(Q.values.float(), Q.row_scale, yq)
        _check_rows(oracle_mod, o, i, qv, xh, yqh, scale=sc)
        # against FP64 of the FP32 matrix: the 16-bit storage error, per row
        # relative to sum |a x|
        comp, _ = oracle_mod.error_metrics(yqh, y64, yabs)
        assert comp <= 1e-2, (dt, comp)
        del Q, yq, qv, sc, yqh


def test_stencil160_selected_staged_thread_mapped(cuda, oracle_mod):
    """The schedule el_spmv_select picks for the stencil (thread_mapped's
    staged kernel): y is the reference CPU loop's bit for bit (FP32, and
    BF16 values, whose loop runs on their exact FP32 widening), and the BF16
    and FP16 runs with row scales agree bit for bit with the unstaged
    kernel."""
    from edge_loops_gb300 import api, synth
    off, idx, vals, x, rows = synth.stencil27(n=160, seed=2, device=cuda)
    A = api.CSR(off, idx, vals, rows, rows)
    ws = api.Workspace()
    sched, opts = api.select_schedule(A, workspace=ws)
    assert (sched, opts) == ("thread_mapped", {"threads_per_row": 1, "variant": 1})
    y = api.spmv(A, x, schedule=sched, workspace=ws, **opts)
    torch.cuda.synchronize()
    assert ws.errors() == 0
    o, i, v, xh, yh = _host(off, idx, vals, x, y)
    np.testing.assert_array_equal(yh, oracle_mod.spmv_f32(o, i, v, xh))
    del y, yh
    Q = A.quantized(torch.bfloat16, per_row_scale=False)
    yq = api.spmv(Q, x, schedule=sched, workspace=ws, **opts)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(
        yq.cpu().numpy(), oracle_mod.spmv_f32(o, i, Q.values.float().cpu().numpy(), xh))
    del Q, yq
    for dt in (torch.bfloat16, torch.float16):
        Q = A.quantized(dt, per_row_scale=True)
        ys = api.spmv(Q, x, schedule=sched, workspace=ws, **opts)
        yu = api.spmv(Q, x, schedule="thread_mapped", workspace=ws)
        torch.cuda.synchronize()
        assert ws.errors() == 0
        assert torch.equal(ys, yu), dt
        del Q, ys, yu


@pytest.mark.parametrize("n,bdt", [(32, torch.float32), (128, torch.float32),
                                   (128, torch.bfloat16)])
def test_spmm_power_law_8M(cuda, oracle_mod, n, bdt):
    """The SpMM workload at full size (2^20 x 2^20, ~8M nonzeros, B 2^20 x n)
    with FP32 and BF16 B, merge_path and group_mapped, on 2048 sampled rows
    of C."""
    from edge_loops_gb300 import api, synth
    off, idx, vals, x, cols = synth.power_law(rows=1 << 20, target_nnz=8_000_000, exponent=2.0,
                                              cap=100_000, seed=3, device=cuda)
    A = api.CSR(off, idx, vals, off.numel() - 1, cols)
    g = torch.Generator(device=cuda)
    g.manual_seed(33)
    B = (torch.rand(cols, n, generator=g, device=cuda) * 2 - 1).to(bdt)
    Bh = B.view(torch.int16).cpu().numpy().view(np.uint16) if bdt == torch.bfloat16 \
        else B.cpu().numpy()
    rng = np.random.default_rng(0)
    rows_s = np.sort(rng.choice(A.rows, 2048, replace=False))
    o, i, v = _host(off, idx, vals)
    lens = o[rows_s + 1] - o[rows_s]
    so = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    sel = np.concatenate([np.arange(o[r], o[r + 1]) for r in rows_s])
    C64, Ca = oracle_mod.spmm_f64(so, i[sel], v[sel],
                                  ("bf16", Bh) if bdt == torch.bfloat16 else Bh)
    nb = (np.diff(so.astype(np.int64)) + 2)[:, None]
    bound = (nb * 2.0 ** -24 / (1 - nb * 2.0 ** -24)) * Ca
    ws = api.Workspace()
    for sched in ("merge_path_flat", "group_mapped"):
        Cm = api.spmm(A, B, torch.full((A.rows, n), float("nan"), device=cuda), schedule=sched,
                      workspace=ws)
        torch.cuda.synchronize()
        assert ws.errors() == 0
        got = Cm[torch.as_tensor(rows_s, device=cuda)].cpu().numpy().astype(np.float64)
        assert int(np.sum(np.abs(got - C64) > bound)) == 0, sched
        del Cm


def test_batched_4096_matrices_f32_and_bf16(cuda, oracle_mod):
    """The batched workload at full size: 4096 square CSRs (rows log-uniform
    in [64, 65536], log-normal row lengths with mean 8, seed 4, ~310M
    nonzeros), one plan each for FP32 and for BF16 values with per-row
    scales.  Every row of every matrix is checked: FP32 within the
    order-free bound of FP64, BF16 within that bound of FP64 of its stored
    values and within 1e-2 (componentwise, relative to sum |a x|) of FP64 of
    the FP32 matrices."""
    from edge_loops_gb300 import api, synth
    R, offc, idxc, valc, xc, rs, ns = synth.batched(count=4096, seed=4, device=cuda)
    assert int(R.sum()) > 30_000_000 and idxc.numel() > 250_000_000
    items, y = api.batched_items(R, offc, idxc, valc, xc, rs, ns)
    y.fill_(float("nan"))
    plan = api.BatchPlan(items)
    plan.execute()
    torch.cuda.synchronize()
    assert plan.errors() == 0
    goff, gidx = synth.batch_as_one_csr(R, offc, idxc, rs, ns)
    o, i, v, xh, yh = _host(goff, gidx, valc, xc, y)
    y64, yabs = oracle_mod.spmv_f64(o, i, v, xh)
    bad = np.nonzero(np.abs(yh.astype(np.float64) - y64) > order_free_bound(o, yabs))[0]
    assert len(bad) == 0, f"{len(bad)} rows outside the bound, first {bad[:5]}"
    plan.close()
    del plan, items, yh

    # BF16 values and per-row scales of the whole batch in one array each
    # (rows are independent, so quantizing the block-diagonal matrix row by
    # row is quantizing every matrix), sliced per matrix
    Q = api.CSR(goff, gidx, valc, goff.numel() - 1, goff.numel() - 1).quantized(
        torch.bfloat16, per_row_scale=True)
    yq = torch.full_like(y, float("nan"))
    qitems = []
    for m, (r, r0, n0) in enumerate(zip(R.tolist(), rs.tolist(), ns.tolist())):
        o_m = offc[r0 + m: r0 + m + r + 1]
        nn = int(o[r0 + r] - o[r0])
        qitems.append((api.CSR(o_m, idxc[n0: n0 + nn], Q.values[n0: n0 + nn], r, r,
                               row_scale=Q.row_scale[r0: r0 + r]),
                       xc[r0: r0 + r], yq[r0: r0 + r]))
    plan = api.BatchPlan(qitems)
    plan.execute()
    torch.cuda.synchronize()
    assert plan.errors() == 0
    qv, sc, yqh = _host(Q.values.float(), Q.row_scale, yq)
    yq64, yqabs = oracle_mod.spmv_f64(o, i, qv, xh, row_scale=sc)
    bad = np.nonzero(np.abs(yqh.astype(np.float64) - yq64) > order_free_bound(o, yqabs))[0]
    assert len(bad) == 0, f"BF16: {len(bad)} rows outside the bound, first {bad[:5]}"
    comp, _ = oracle_mod.error_metrics(yqh, y64, yabs)
    assert comp <= 1e-2, comp
    plan.close()
