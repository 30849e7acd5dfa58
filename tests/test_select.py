"""Schedule selection (csrc/select.cu): the cost model picks, from (rows,
nnz, longest row), a schedule whose measured time is close to the best one.

CPU: the model's choices on the committed GB300 sweep
(tests/data/select_sweep_gb300.csv, made by edge_loops_gb300/tune_select.py:
every schedule timed on 133 synthetic shapes) are within 2 % of the best
per shape on geometric mean, never worse than 1.35x, and better than always
running merge_path; argument errors.  GPU: row statistics (with the row
coherence) equal numpy's, and the selected schedule's SpMV is within the
FP32 bound.
"""
import csv
import ctypes as C
import os

import numpy as np
import pytest

from conftest import REPO, order_free_bound, random_csr

SWEEP = os.path.join(REPO, "tests", "data", "select_sweep_gb300.csv")
CANDIDATES = ("merge_path", "tm1", "tm4", "tm32")


def coherence(off, idx):
    """el_row_stats.coherence restated: on every (rows >> 16)-th row r, the
    first min(len r, len r+1, 32) column pairs of rows r and r+1 that step by
    0, 1 or 2."""
    rows = len(off) - 1
    stride = max(1, rows >> 16)
    off = off.astype(np.int64)
    idx = idx.astype(np.int64)
    pairs = steps = 0
    for r in range(0, rows - 1, stride):
        lo, hi, hi2 = off[r], off[r + 1], off[r + 2]
        m = min(hi - lo, hi2 - hi, 32)
        if m > 0:
            d = idx[hi:hi + m] - idx[lo:lo + m]
            steps += int(((d >= 0) & (d <= 2)).sum())
            pairs += m
    return steps / pairs if pairs else 0.0


def choose(L, rows, nnz, mx):
    s, t, est = C.c_int32(), C.c_int32(), C.c_double()
    assert L.lib().el_select_schedule(rows, rows, nnz, mx, C.byref(s), C.byref(t),
                                      C.byref(est)) == L.EL_OK
    return ("merge_path" if s.value == L.EL_SCHED_MERGE_PATH_FLAT else "tm%d" % t.value,
            est.value)


def choose_stats(L, rows, nnz, mx, coh):
    """el_select_schedule_stats: "tms" for thread_mapped's staged kernel."""
    from edge_loops_gb300 import api
    st = L.ElRowStats()
    st.max_row_nnz, st.coherence = mx, coh
    s, o, est = C.c_int32(), api.make_opts(), C.c_double()
    assert L.lib().el_select_schedule_stats(rows, rows, nnz, C.byref(st), C.byref(s),
                                            C.byref(o), C.byref(est)) == L.EL_OK
    if s.value == L.EL_SCHED_MERGE_PATH_FLAT:
        return "merge_path", est.value
    return ("tms" if o.variant == 1 else "tm%d" % o.threads_per_row), est.value


def test_model_quality_on_the_sweep(built_lib):
    """Measured time of the chosen kernel over the best one per shape (the
    staged kernel's time counts where it was measured: rows of at most 27
    nonzeros, coherent or not)."""
    from edge_loops_gb300 import _lib as L
    loss, loss_mp, loss_plain = [], [], []
    staged_picked = 0
    with open(SWEEP) as f:
        for r in csv.DictReader(f):
            t = {c: float(r[c]) for c in CANDIDATES + ("tms",) if r[c] != ""}
            best = min(t.values())
            c, est = choose_stats(L, int(r["rows"]), int(r["nnz"]), int(r["max"]),
                                  float(r["coherence"]))
            assert est > 0
            staged_picked += c == "tms"
            loss.append(t[c] / best)
            loss_mp.append(t["merge_path"] / best)
            # without the coherence the staged kernel is never picked
            c0, _ = choose(L, int(r["rows"]), int(r["nnz"]), int(r["max"]))
            assert c0 != "tms"
            loss_plain.append(t[c0] / best)
    loss, loss_mp = np.array(loss), np.array(loss_mp)
    gm = float(np.exp(np.log(loss).mean()))
    assert len(loss) >= 130
    assert gm <= 1.02, gm
    assert loss.max() <= 1.35, loss.max()
    assert gm < float(np.exp(np.log(loss_mp).mean())) - 0.2
    assert staged_picked >= 3  # the larger stencils
    assert gm <= float(np.exp(np.log(np.array(loss_plain)).mean()))


def test_staged_kernel_rules(built_lib):
    """el_select_schedule_stats weighs thread_mapped's staged kernel only on
    rows of at most 27 nonzeros with a row coherence of at least 0.5, and
    el_select_schedule (no coherence) never picks it."""
    from edge_loops_gb300 import _lib as L
    stencil = (1 << 21, 55_742_968)  # the 128^3 stencil's rows and nonzeros
    assert choose_stats(L, *stencil, 27, 0.84)[0] == "tms"
    assert choose_stats(L, *stencil, 27, 0.49)[0] != "tms"
    assert choose_stats(L, *stencil, 28, 0.99)[0] != "tms"
    assert choose(L, *stencil, 27)[0] != "tms"
    # merge_path chosen: opts left alone; thread_mapped chosen: its lanes per
    # row and variant written, the other fields left alone
    from edge_loops_gb300 import api
    st = L.ElRowStats()
    st.max_row_nnz, st.coherence = 100_000, 0.0  # the power-law matrix
    s, o = C.c_int32(), api.make_opts(items_per_thread=5, variant=1)
    assert L.lib().el_select_schedule_stats(1 << 20, 1 << 20, 16_000_000, C.byref(st), C.byref(s),
                                            C.byref(o), None) == L.EL_OK
    assert (s.value, o.items_per_thread, o.variant) == (L.EL_SCHED_MERGE_PATH_FLAT, 5, 1)
    st.max_row_nnz, st.coherence = 10, 0.0  # 1000 x 1000, 10 scattered nonzeros per row
    o = api.make_opts(items_per_thread=5, variant=1)
    assert L.lib().el_select_schedule_stats(1000, 1000, 10_000, C.byref(st), C.byref(s),
                                            C.byref(o), None) == L.EL_OK
    assert s.value == L.EL_SCHED_THREAD_MAPPED
    assert (o.variant, o.items_per_thread) == (0, 5) and o.threads_per_row in (1, 4, 32)
    assert L.lib().el_select_schedule_stats(10, 10, 5, None, C.byref(s), C.byref(o),
                                            None) == L.EL_ERR_NULL_POINTER


def test_selection_rules_and_errors(built_lib):
    from edge_loops_gb300 import _lib as L
    assert choose(L, 1 << 20, 16_000_000, 100_000)[0] == "merge_path"  # power-law
    assert choose(L, 1 << 22, 1 << 26, 4000)[0] == "merge_path"        # large, skewed
    assert choose(L, 1000, 10_000, 10)[0].startswith("tm")             # small regular
    assert choose(L, 1 << 20, 1 << 20, 1)[0] == "tm1"                  # one per row
    assert choose(L, 0, 0, 0)[0] in CANDIDATES
    s, t = C.c_int32(), C.c_int32()
    assert L.lib().el_select_schedule(10, 10, 5, 6, C.byref(s), C.byref(t),
                                      None) == L.EL_ERR_INVALID_ARGUMENT
    assert L.lib().el_select_schedule(-1, 10, 5, 1, C.byref(s), C.byref(t),
                                      None) == L.EL_ERR_INVALID_ARGUMENT
    assert L.lib().el_select_schedule(10, 10, 5, 1, None, C.byref(t),
                                      None) == L.EL_ERR_NULL_POINTER


@pytest.mark.gpu
def test_row_stats(cuda):
    from edge_loops_gb300 import api
    rng = np.random.default_rng(53)
    for off, idx, vals, x in [random_csr(rng, rows=20000, cols=3000, max_len=40, empty_frac=0.3,
                                         long_rows=[(7, 2900)]),
                              random_csr(rng, rows=3, cols=10, max_len=0)]:
        A = api.CSR.from_arrays(off, idx, vals, len(x), device="cuda")
        st = api.row_stats(A)
        lens = np.diff(off).astype(np.float64)
        assert st["max_row_nnz"] == int(lens.max())
        assert st["empty_rows"] == int((lens == 0).sum())
        assert st["mean_row_nnz"] == pytest.approx(lens.mean())
        cv = lens.std() / lens.mean() if lens.mean() > 0 else 0.0
        assert st["cv"] == pytest.approx(cv, rel=1e-6, abs=1e-9)
        assert st["coherence"] == pytest.approx(coherence(off, idx), rel=1e-12, abs=1e-12)
    # a stencil's consecutive rows repeat their pattern one column over
    from edge_loops_gb300 import synth
    o, i, v, x, n = synth.stencil27(n=20, seed=2)
    st = api.row_stats(api.CSR.from_arrays(o, i, v, n, device="cuda"))
    assert st["coherence"] == pytest.approx(coherence(o.numpy(), i.numpy()), rel=1e-12)
    assert st["coherence"] > 0.8 and st["max_row_nnz"] == 27


@pytest.mark.gpu
def test_select_then_spmv(cuda, oracle_mod):
    import torch
    from edge_loops_gb300 import api, synth
    dev = torch.device("cuda", 0)
    off, idx, vals, x, cols = synth.uniform_rows(rows=1000, cols=1000, per_row=10, seed=0)
    A = api.CSR.from_arrays(off, idx, vals, cols, device=dev)
    sched, o = api.select_schedule(A)
    assert sched == "thread_mapped" and o["threads_per_row"] in (1, 4, 32)
    assert o.get("variant", 0) == 0  # scattered columns: the unstaged walk
    y = api.spmv(A, x.to(dev), schedule=sched, **o).cpu().numpy()
    on, ix, vv, xx = off.numpy(), idx.numpy(), vals.numpy(), x.numpy()
    y64, yabs = oracle_mod.spmv_f64(on, ix, vv, xx)
    assert np.all(np.abs(y - y64) <= order_free_bound(on, yabs))
    off, idx, vals, x, cols = synth.power_law(rows=1 << 16, target_nnz=1 << 20, exponent=2.0,
                                              cap=60_000, seed=9)
    A = api.CSR.from_arrays(off, idx, vals, cols, device=dev)
    assert api.select_schedule(A) == ("merge_path_flat", {})
    # a stencil: short coherent rows, the staged kernel, bit-identical to the
    # reference CPU loop
    off, idx, vals, x, n = synth.stencil27(n=100, seed=2)
    A = api.CSR.from_arrays(off, idx, vals, n, device=dev)
    sched, o = api.select_schedule(A)
    assert (sched, o) == ("thread_mapped", {"threads_per_row": 1, "variant": 1})
    y = api.spmv(A, x.to(dev), schedule=sched, **o).cpu().numpy()
    np.testing.assert_array_equal(
        y, oracle_mod.spmv_f32(off.numpy(), idx.numpy(), vals.numpy(), x.numpy()))


@pytest.mark.gpu
def test_auto_schedule(cuda, oracle_mod):
    """EL_SCHED_AUTO: the model with the longest row taken as nnz -- a
    thread_mapped warp per row on a matrix of a few hundred nonzeros,
    merge_path (bit for bit) otherwise."""
    import torch
    from edge_loops_gb300 import api
    rng = np.random.default_rng(59)
    for rows, max_len in [(100, 3), (3000, 20)]:
        off, idx, vals, x = random_csr(rng, rows=rows, cols=rows, max_len=max_len,
                                       empty_frac=0.2)
        A = api.CSR.from_arrays(off, idx, vals, len(x), device="cuda")
        xd = torch.from_numpy(x).cuda()
        y = api.spmv(A, xd, schedule="auto").cpu().numpy()
        y64, yabs = oracle_mod.spmv_f64(off, idx, vals, x)
        assert np.all(np.abs(y - y64) <= order_free_bound(off, yabs))
        if A.nnz > 400:
            ym = api.spmv(A, xd, schedule="merge_path_flat").cpu().numpy()
            np.testing.assert_array_equal(y, ym)
