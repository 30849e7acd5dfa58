"""GPU parity of the SpMV path against the oracle, through the C ABI.

Bars: split points bit-identical to the restated reference search; the
TPR=1 thread_mapped schedule (both kernels) bit-identical to the reference
CPU loop; every
schedule within the order-free FP32 bound gamma_(n+2) * sum|a x| of the FP64
oracle (valid for any summation order) and within the reference's own
|gpu - cpu| <= 1e-2 check."""
import numpy as np
import pytest
import torch

from conftest import load_golden, order_free_bound, random_csr

pytestmark = pytest.mark.gpu

SCHEDS = [
    ("merge_path_flat", {}),
    ("merge_path_flat", {"compensated": True}),
    ("merge_path_flat", {"row_weight": 1}),
    ("merge_path_flat", {"row_weight": 5, "max_ctas": 3}),
    ("merge_path_flat", {"nz_per_lane": 16}),
    ("merge_path_flat", {"nz_per_lane": 16, "compensated": True}),
    ("merge_path_flat", {"nz_per_lane": 16, "max_ctas": 2}),
    ("merge_path_flat", {"variant": 2}),
    ("merge_path_flat", {"variant": 2, "compensated": True}),
    ("merge_path_flat", {"variant": 1}),
    ("merge_path_flat", {"variant": 1, "items_per_thread": 4}),
    ("merge_path_flat", {"variant": 1, "compensated": True}),
    ("work_oriented", {}),
    ("work_oriented", {"num_threads": 1024}),
    ("thread_mapped", {}),
    ("thread_mapped", {"compensated": True}),
    ("thread_mapped", {"threads_per_row": 8}),
    ("thread_mapped", {"threads_per_row": 32}),
    ("thread_mapped", {"variant": 1}),
    ("thread_mapped", {"variant": 1, "compensated": True}),
    ("thread_mapped", {"variant": 1, "max_ctas": 1}),
    ("group_mapped", {}),
    ("group_mapped", {"group_rows": 32}),
    ("group_mapped", {"threads_per_block": 256, "group_rows": 256}),
]
IDS = [f"{s}{'-' + '-'.join(f'{k}{v}' for k, v in o.items()) if o else ''}" for s, o in SCHEDS]


def dev_csr(off, idx, vals, cols, cuda):
    from edge_loops_gb300.api import CSR
    return CSR.from_arrays(off, idx, vals, cols, device=cuda)


def run(A, x, sched, opts, cuda, fill=np.nan):
    from edge_loops_gb300 import api
    xt = torch.as_tensor(x, device=cuda)
    y = torch.full((A.rows,), fill, dtype=torch.float32, device=cuda)
    api.spmv(A, xt, y, schedule=sched, **opts)
    flags = api.workspace_errors()
    torch.cuda.synchronize()
    return y.cpu().numpy(), flags


def check_against_oracle(oracle_mod, off, idx, vals, x, y, scale=None):
    y64, yabs = oracle_mod.spmv_f64(off, idx, vals, x, row_scale=scale)
    bound = order_free_bound(off, yabs)
    err = np.abs(y.astype(np.float64) - y64)
    bad = np.nonzero(err > bound)[0]
    assert len(bad) == 0, f"{len(bad)} rows off, first {bad[:5]} err {err[bad[:5]]} " \
                          f"bound {bound[bad[:5]]}"
    return oracle_mod.error_metrics(y, y64, yabs)


@pytest.mark.parametrize("sched,opts", SCHEDS, ids=IDS)
def test_chesapeake_exact(cuda, oracle_mod, sched, opts):
    g = load_golden("chesapeake.npz")
    A = dev_csr(g["offsets"], g["indices"], g["values"], int(g["cols"]), cuda)
    y, flags = run(A, g["x"], sched, opts, cuda)
    assert flags == 0
    np.testing.assert_array_equal(y, g["y_exact"].astype(np.float32))


@pytest.mark.parametrize("sched,opts", SCHEDS, ids=IDS)
def test_uniform_1000_matches_reference_cpu(cuda, oracle_mod, sched, opts):
    from edge_loops_gb300 import synth
    off, idx, vals, x, cols = [t.numpy() if hasattr(t, "numpy") else t
                               for t in synth.uniform_rows(seed=0)]
    A = dev_csr(off, idx, vals, cols, cuda)
    y, flags = run(A, x, sched, opts, cuda)
    assert flags == 0
    yref = oracle_mod.spmv_f32(off, idx, vals, x)
    # the reference's validation (examples/spmv/helpers.hxx:138)
    assert int(np.sum(np.abs(y - yref) > 1e-2)) == 0
    check_against_oracle(oracle_mod, off, idx, vals, x, y)


def _tm_cases():
    from edge_loops_gb300 import synth
    rng = np.random.default_rng(21)
    yield "random", random_csr(rng, rows=5000, cols=3000, max_len=60, empty_frac=0.1), 3000
    o, i, v, x, n = synth.stencil27(n=24, seed=2)
    yield "stencil24", (o.numpy(), i.numpy(), v.numpy(), x.numpy()), n
    o, i, v, x, cols = synth.power_law(rows=1 << 14, target_nnz=300_000, cap=20_000, seed=5)
    yield "power_law", (o.numpy(), i.numpy(), v.numpy(), x.numpy()), cols
    # rows of every length from 0 to 70 around the 8-nonzero load batches
    lens = np.concatenate([np.arange(71), rng.integers(0, 70, 100)])
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    idx = np.concatenate([np.sort(rng.choice(500, L, replace=False)) for L in lens]).astype(np.int32)
    yield "row_lengths", (off, idx, rng.uniform(-1, 1, len(idx)).astype(np.float32),
                          rng.uniform(-1, 1, 500).astype(np.float32)), 500


@pytest.mark.parametrize("case", ["random", "stencil24", "power_law", "row_lengths"])
@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("variant", [0, 1])
def test_thread_mapped_bit_exact_with_reference_loop(cuda, oracle_mod, case, dtype, variant):
    """One lane per row, rows read in place (variant 0) or staged through
    shared memory (1): y is the reference CPU loop's, bit for bit (16-bit
    values: the loop over their exact FP32 widening)."""
    (off, idx, vals, x), cols = next(c[1:] for c in _tm_cases() if c[0] == case)
    A = dev_csr(off, idx, vals, cols, cuda)
    if dtype != torch.float32:
        A = A.quantized(dtype, per_row_scale=False)
        vals = A.values.float().cpu().numpy()
    y, flags = run(A, x, "thread_mapped", {"variant": variant}, cuda)
    assert flags == 0
    np.testing.assert_array_equal(y, oracle_mod.spmv_f32(off, idx, vals, x))


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16, torch.float16])
def test_thread_mapped_staged_equals_unstaged(cuda, dtype):
    """The staged kernel (variant 1) against the unstaged one, bit for bit:
    per-row scales, compensated sums, chunks that do not fit the buffer next
    to ones that do, arrays whose ends fall inside a 16-byte copy unit, and
    arrays not 16-byte aligned (the unstaged kernel runs)."""
    from edge_loops_gb300 import api
    rng = np.random.default_rng(61)
    cases = [random_csr(rng, rows=rows, cols=700, max_len=ml, empty_frac=0.1, long_rows=lr)
             for rows, ml, lr in [(1, 27, []), (31, 27, []), (33, 27, []), (4097, 27, []),
                                  (2000, 9, [(5, 600), (1999, 40)]), (3001, 60, []),
                                  (500, 1, [])]]
    for off, idx, vals, x in cases:
        nnz = len(idx)
        xt = torch.as_tensor(x, device=cuda)
        for shift in (0, 1, 4):  # 4 elements: still 16-byte aligned for FP32
            ib = torch.zeros(nnz + 8, dtype=torch.int32, device=cuda)
            vb = torch.zeros(nnz + 8, dtype=dtype, device=cuda)
            ib[shift: shift + nnz] = torch.as_tensor(idx, device=cuda)
            vb[shift: shift + nnz] = torch.as_tensor(vals).to(dtype).to(cuda)
            scale = None if dtype == torch.float32 else \
                torch.as_tensor(rng.uniform(0.5, 2.0, len(off) - 1).astype(np.float32),
                                device=cuda)
            A = api.CSR(torch.as_tensor(off, device=cuda), ib[shift: shift + nnz],
                        vb[shift: shift + nnz], len(off) - 1, len(x), row_scale=scale)
            for comp in (False, True):
                ys = []
                for variant in (0, 1):
                    y = torch.full((A.rows,), float("nan"), device=cuda)
                    api.spmv(A, xt, y, schedule="thread_mapped", variant=variant,
                             compensated=comp)
                    ys.append(y)
                assert api.workspace_errors() == 0
                assert torch.equal(ys[0], ys[1]), (len(off) - 1, shift, comp)


def _power_law_case(cuda, rows=1 << 16, nnz=1_500_000, cap=40_000, seed=1):
    from edge_loops_gb300 import synth
    off, idx, vals, x, cols = synth.power_law(rows=rows, target_nnz=nnz, cap=cap, seed=seed)
    return off.numpy(), idx.numpy(), vals.numpy(), x.numpy(), cols


@pytest.mark.parametrize("sched,opts", SCHEDS, ids=IDS)
def test_power_law_all_schedules(cuda, oracle_mod, sched, opts):
    off, idx, vals, x, cols = _power_law_case(cuda)
    A = dev_csr(off, idx, vals, cols, cuda)
    y, flags = run(A, x, sched, opts, cuda)
    assert flags == 0
    check_against_oracle(oracle_mod, off, idx, vals, x, y)


@pytest.mark.parametrize("sched,opts", SCHEDS, ids=IDS)
def test_edge_cases(cuda, oracle_mod, sched, opts):
    rng = np.random.default_rng(7)
    cases = [
        random_csr(rng, rows=1, cols=50000, max_len=0, long_rows=[(0, 40000)]),  # one long row
        random_csr(rng, rows=3000, cols=100, max_len=5, empty_frac=0.9),  # mostly empty
        random_csr(rng, rows=777, cols=1000, max_len=0, long_rows=[(3, 900), (776, 1000)]),
        (np.zeros(101, dtype=np.int32), np.zeros(0, dtype=np.int32),
         np.zeros(0, dtype=np.float32), np.ones(5, dtype=np.float32)),  # no nonzeros
        random_csr(rng, rows=2, cols=3, max_len=3),
    ]
    for off, idx, vals, x in cases:
        A = dev_csr(off, idx, vals, len(x), cuda)
        y, flags = run(A, x, sched, opts, cuda)
        assert flags == 0
        check_against_oracle(oracle_mod, off, idx, vals, x, y)


@pytest.mark.parametrize("opts", [{}, {"compensated": True}, {"variant": 2}, {"max_ctas": 2},
                                  {"nz_per_lane": 16}])
@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
def test_merge_path_unaligned_arrays(cuda, oracle_mod, opts, dtype):
    """indices and values starting at every phase modulo 8 elements, equal
    (128-bit loads of both) or not (element-wise loads), and arrays that end
    inside a 16-byte chunk."""
    from edge_loops_gb300 import api
    rng = np.random.default_rng(21)
    off, idx, vals, x = random_csr(rng, rows=3000, cols=5000, max_len=40, empty_frac=0.1,
                                   long_rows=[(7, 3000)])
    nnz = len(idx)
    xt = torch.as_tensor(x, device=cuda)
    offt = torch.as_tensor(off, device=cuda)
    vq = torch.as_tensor(vals).to(dtype)
    v64 = vq.float().numpy()
    # equal phases (128-bit loads), and values an odd or an even number of
    # elements off the indices (element-wise loads)
    for si, sv in [(0, 0), (1, 1), (3, 3), (5, 5), (7, 7), (1, 0), (2, 5), (6, 3),
                   (0, 2), (3, 7), (5, 1), (4, 6), (7, 3)]:
        ib = torch.zeros(nnz + 8, dtype=torch.int32, device=cuda)
        vb = torch.zeros(nnz + 8, dtype=dtype, device=cuda)
        ib[si: si + nnz] = torch.as_tensor(idx, device=cuda)
        vb[sv: sv + nnz] = vq.to(cuda)
        A = api.CSR(offt, ib[si: si + nnz], vb[sv: sv + nnz], len(off) - 1, len(x))
        y = torch.full((A.rows,), float("nan"), device=cuda)
        api.spmv(A, xt, y, schedule="merge_path_flat", **opts)
        assert api.workspace_errors() == 0
        check_against_oracle(oracle_mod, off, idx, v64, x, y.cpu().numpy())


def test_long_rows_across_many_ctas(cuda, oracle_mod):
    """Rows much longer than a CTA's range: the cross-range carry chain."""
    rng = np.random.default_rng(13)
    off, idx, vals, x = random_csr(rng, rows=400, cols=300_000, max_len=50,
                                   long_rows=[(0, 250_000), (17, 120_000), (399, 200_000)])
    A = dev_csr(off, idx, vals, 300_000, cuda)
    for opts in ({}, {"max_ctas": 3}, {"max_ctas": 1}, {"compensated": True},
                 {"row_weight": 1}, {"row_weight": 7, "max_ctas": 2},
                 {"variant": 2}, {"variant": 2, "max_ctas": 1},
                 {"variant": 1, "items_per_thread": 4},
                 {"variant": 1, "items_per_thread": 4, "max_ctas": 7},
                 {"variant": 1, "max_ctas": 1}, {"variant": 1, "compensated": True}):
        y, flags = run(A, x, "merge_path_flat", opts, cuda)
        assert flags == 0
        check_against_oracle(oracle_mod, off, idx, vals, x, y)
    for nt in (128, 128 * 64, 128 * 1000):
        y, flags = run(A, x, "work_oriented", {"num_threads": nt}, cuda)
        assert flags == 0
        check_against_oracle(oracle_mod, off, idx, vals, x, y)


@pytest.mark.parametrize("sched,opts", SCHEDS, ids=IDS)
def test_deterministic(cuda, sched, opts):
    off, idx, vals, x, cols = _power_law_case(cuda, rows=1 << 14, nnz=300_000, cap=20_000)
    A = dev_csr(off, idx, vals, cols, cuda)
    y1, _ = run(A, x, sched, opts, cuda)
    y2, _ = run(A, x, sched, opts, cuda, fill=0.0)
    np.testing.assert_array_equal(y1, y2)


def test_merge_path_partition_bit_exact(cuda, oracle_mod):
    from edge_loops_gb300 import api
    for off, nnz in [(load_golden("chesapeake.npz")["offsets"], 340)] + \
            [(_power_law_case(cuda, rows=5000, nnz=80_000, cap=9000)[0], None)]:
        nnz = int(off[-1])
        rows = len(off) - 1
        d = torch.as_tensor(off, device=cuda)
        for tpb, ipt in ((128, 5), (64, 3), (256, 8)):
            got = api.merge_path_partition(d, rows, nnz, tpb, ipt).cpu().numpy().view(np.uint32)
            exp = oracle_mod.merge_path_tile_coords(off, nnz, tpb * ipt)
            np.testing.assert_array_equal(got, exp)
            got = api.merge_path_thread_coords(d, rows, nnz, tpb, ipt).cpu().numpy()
            exp = oracle_mod.merge_path_thread_coords(off, nnz, tpb, ipt)
            np.testing.assert_array_equal(got.view(np.uint32), exp)
        for nt in (128, 304 * 128, 1000):
            got = api.work_oriented_partition(d, rows, nnz, nt).cpu().numpy()
            np.testing.assert_array_equal(got, oracle_mod.work_oriented_coords(off, nnz, nt))


def test_malformed_csr_sets_flags_without_fault(cuda, oracle_mod):
    from edge_loops_gb300 import api
    rng = np.random.default_rng(2)
    off, idx, vals, x = random_csr(rng, rows=500, cols=100, max_len=20)
    bad_idx = idx.copy()
    bad_idx[::7] = 100 + 5  # outside [0, cols)
    bad_idx[3] = -4
    A = dev_csr(off, bad_idx, vals, 100, cuda)
    assert api.validate(A) & 0x1
    for sched, opts in SCHEDS:
        y, flags = run(A, x, sched, opts, cuda)
        assert flags & 0x1, sched
    bad_off = off.copy()
    bad_off[100] = bad_off[300]  # not monotone
    bad_off[200] = -50
    A = dev_csr(bad_off, idx, vals, 100, cuda)
    assert api.validate(A) & 0x2
    for sched, opts in SCHEDS:
        y, flags = run(A, x, sched, opts, cuda)
    short = off.copy()
    short[-1] = off[-1] - 3  # offsets[rows] != nnz
    A = dev_csr(short, idx, vals, 100, cuda)
    assert api.validate(A) & 0x4
    # the workspace is healthy afterwards
    A = dev_csr(off, idx, vals, 100, cuda)
    for sched, opts in SCHEDS:
        y, flags = run(A, x, sched, opts, cuda)
        assert flags == 0
        check_against_oracle(oracle_mod, off, idx, vals, x, y)


@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float16])
@pytest.mark.parametrize("per_row", [True, False])
def test_mixed_precision_stencil(cuda, oracle_mod, dtype, per_row):
    from edge_loops_gb300 import api, synth
    off, idx, vals, x, rows = [t.numpy() if hasattr(t, "numpy") else t
                               for t in synth.stencil27(n=24, seed=2)]
    A = dev_csr(off, idx, vals, rows, cuda)
    Aq = A.quantized(dtype, per_row_scale=per_row)
    qv = Aq.values.float().cpu().numpy()
    sc = Aq.row_scale.cpu().numpy() if per_row else None
    row_of = np.repeat(np.arange(rows), np.diff(off))
    top = 0 if dtype == torch.bfloat16 else 14  # row max lands in [2^top, 2^(top+1))
    if per_row:
        assert np.all(np.log2(sc) == np.round(np.log2(sc)))  # powers of two
        assert np.all(np.abs(qv) < 2.0 ** (top + 1))
        rmax = np.maximum.reduceat(np.abs(qv), off[:-1])
        assert np.all(rmax >= 2.0 ** top)
        s_of = sc[row_of]
    else:
        s_of = np.ones(len(qv))
    deq = qv * s_of
    u = 2.0 ** -8 if dtype == torch.bfloat16 else 2.0 ** -11  # unit roundoff
    tiny = 0.0 if dtype == torch.bfloat16 else 2.0 ** -25  # half a subnormal ulp of FP16
    err = np.abs(deq.astype(np.float64) - vals)
    assert np.all(err <= np.maximum(u * np.abs(vals), tiny * s_of)), np.max(err)
    for sched, opts in SCHEDS:
        y, flags = run(Aq, x, sched, opts, cuda)
        assert flags == 0
        # exact stored values: order-free bound against FP64 of the stored matrix
        check_against_oracle(oracle_mod, off, idx, qv, x, y, scale=sc)
        # against the FP32 matrix: the quantisation error is inside 1e-2
        y64, yabs = oracle_mod.spmv_f64(off, idx, vals, x)
        comp, _ = oracle_mod.error_metrics(y, y64, yabs)
        assert comp <= 1e-2, (sched, comp)


def test_lookback_wait_times_out_with_status(cuda):
    """A bounded device wait that nothing satisfies ends with a status
    (EL_FLAG_TIMEOUT), not a hang; the workspace stays usable."""
    from edge_loops_gb300 import api
    rng = np.random.default_rng(8)
    off, idx, vals, x = random_csr(rng, rows=10, cols=100_000, max_len=5,
                                   long_rows=[(4, 90_000)])
    A = dev_csr(off, idx, vals, 100_000, cuda)
    ws = api.Workspace()
    xt = torch.as_tensor(x, device=cuda)
    y = torch.empty(A.rows, device=cuda)
    o = api.make_opts(items_per_thread=4, wait_limit_us=2000)
    o.test_hooks = 1  # ranges do not publish their carries
    import ctypes as C
    from edge_loops_gb300 import _lib
    a = A.el()
    st = _lib.lib().el_spmv(ws.handle, C.byref(a), 0, C.byref(o), C.c_void_p(xt.data_ptr()),
                            C.c_void_p(y.data_ptr()),
                            C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    assert ws.errors() & 0x8
    api.spmv(A, xt, y, workspace=ws, items_per_thread=4)
    assert ws.errors() == 0


@pytest.mark.parametrize("block_nnz", [0, 5000, 7])
@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
def test_spmv_host_streams_blocks(cuda, oracle_mod, block_nnz, dtype):
    """el_spmv_host: CSR, x and y in (pinned) host memory, row blocks copied
    while the previous block is multiplied; blocks smaller than a row give
    one-row blocks."""
    from edge_loops_gb300 import api
    rng = np.random.default_rng(31)
    off, idx, vals, x = random_csr(rng, rows=4000, cols=6000, max_len=60, empty_frac=0.1,
                                   long_rows=[(11, 5000), (3999, 900)])
    A = api.CSR(torch.as_tensor(off).pin_memory(), torch.as_tensor(idx).pin_memory(),
                torch.as_tensor(vals).pin_memory(), len(off) - 1, len(x))
    scale = None
    if dtype != torch.float32:
        Ad = A.__class__(A.offsets.to(cuda), A.indices.to(cuda), A.values.to(cuda), A.rows, A.cols)
        Aq = Ad.quantized(dtype, per_row_scale=True)
        A = api.CSR(A.offsets, A.indices, Aq.values.cpu().pin_memory(), A.rows, A.cols,
                    row_scale=Aq.row_scale.cpu().pin_memory())
        scale = A.row_scale.numpy()
    xh = torch.as_tensor(x).pin_memory()
    y = torch.full((A.rows,), float("nan")).pin_memory()
    ws = api.Workspace()
    for _ in range(2):  # the second call reuses the staging memory
        api.spmv_host(A, xh, y, block_nnz=block_nnz, workspace=ws)
        torch.cuda.synchronize()
    assert ws.errors() == 0
    check_against_oracle(oracle_mod, off, idx, A.values.float().numpy(), x, y.numpy(),
                         scale=scale)


def test_spmv_host_pageable_and_malformed(cuda, oracle_mod):
    from edge_loops_gb300 import api, _lib
    rng = np.random.default_rng(32)
    off, idx, vals, x = random_csr(rng, rows=700, cols=800, max_len=30)
    A = api.CSR(torch.as_tensor(off), torch.as_tensor(idx), torch.as_tensor(vals),
                len(off) - 1, len(x))
    y = api.spmv_host(A, torch.as_tensor(x), torch.empty(A.rows), block_nnz=999)
    torch.cuda.synchronize()
    check_against_oracle(oracle_mod, off, idx, vals, x, y.numpy())
    bad = off.copy()
    bad[-1] += 3  # offsets[rows] != nnz
    B = api.CSR(torch.as_tensor(bad), torch.as_tensor(idx), torch.as_tensor(vals),
                len(off) - 1, len(x))
    with pytest.raises(_lib.ElError) as e:
        api.spmv_host(B, torch.as_tensor(x))
    assert e.value.status == _lib.EL_ERR_MALFORMED_CSR


@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float16])
def test_quantized_into_slices(cuda, dtype):
    """quantized(out=, out_scale=) writes the same values and scales as a
    fresh quantization, into slices of larger arrays."""
    from edge_loops_gb300 import api
    rng = np.random.default_rng(71)
    off, idx, vals, x = random_csr(rng, rows=700, cols=500, max_len=20, empty_frac=0.1)
    A = dev_csr(off, idx, vals, 500, cuda)
    ref = A.quantized(dtype, per_row_scale=True)
    big = torch.zeros(A.nnz + 13, dtype=dtype, device=cuda)
    bigs = torch.zeros(A.rows + 5, dtype=torch.float32, device=cuda)
    Q = A.quantized(dtype, per_row_scale=True, out=big[7: 7 + A.nnz],
                    out_scale=bigs[3: 3 + A.rows])
    assert torch.equal(Q.values.view(torch.int16), ref.values.view(torch.int16))
    assert torch.equal(Q.row_scale, ref.row_scale)
    assert torch.count_nonzero(big[:7].float()) == 0 and torch.count_nonzero(bigs[:3]) == 0
    # y agrees within the FP32 bound (not bit for bit: the tiles' boundaries
    # follow the arrays' alignment, which differs between the two layouts)
    y = api.spmv(Q, torch.from_numpy(x).to(cuda)).cpu().numpy().astype(np.float64)
    yr = api.spmv(ref, torch.from_numpy(x).to(cuda)).cpu().numpy().astype(np.float64)
    vq = ref.values.float().cpu().numpy()
    sq = ref.row_scale.cpu().numpy()
    lens = np.diff(off).astype(np.float64)
    y_abs = np.zeros(len(lens))
    rows_of = np.repeat(np.arange(len(lens)), np.diff(off))
    np.add.at(y_abs, rows_of, np.abs(vq.astype(np.float64) * x[idx]))
    bound = 2 * (lens + 2) * 2.0 ** -24 / (1 - (lens + 2) * 2.0 ** -24) * y_abs * sq
    assert np.all(np.abs(y - yr) <= bound)
    with pytest.raises(ValueError):
        A.quantized(dtype, out=big[: A.nnz - 1])
