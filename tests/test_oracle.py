"""The oracle restatement, pinned against the reference's own outputs
(golden fixtures made from the reference's loader, CSR conversion, x
generator and sample matrix) and against an independent brute-force merge
walk.  CPU only."""
import numpy as np
import pytest

from conftest import load_golden, merge_coords_weighted, merge_walk_weighted, random_csr


def test_chesapeake_matches_reference_fixture(oracle_mod):
    g = load_golden("chesapeake.npz")
    # README.md:84-88 of the reference: "Dimensions: 39 x 39 (340)"
    assert (int(g["rows"]), int(g["cols"]), int(g["nnz"])) == (39, 39, 340)
    y = oracle_mod.spmv_f32(g["offsets"], g["indices"], g["values"], g["x"])
    # values are 1.0 and x integers: every summation order is exact
    np.testing.assert_array_equal(y.astype(np.int64), g["y_exact"])
    y64, yabs = oracle_mod.spmv_f64(g["offsets"], g["indices"], g["values"], g["x"])
    np.testing.assert_array_equal(y64, g["y_exact"].astype(np.float64))
    # the reference's validation criterion: |gpu - cpu| > 1e-2 counts an error
    assert np.sum(np.abs(y - g["y_exact"]) > 1e-2) == 0


def test_sample_csr_matches_reference_fixture(oracle_mod):
    g = load_golden("sample.npz")
    np.testing.assert_array_equal(g["offsets"], [0, 0, 2, 3, 4])
    y = oracle_mod.spmv_f32(g["offsets"], g["indices"], g["values"], g["x"])
    np.testing.assert_array_equal(y, [0.0, 21.0, 9.0, 12.0])
    np.testing.assert_array_equal(g["y_exact"], [0, 21, 9, 12])


def _cases():
    rng = np.random.default_rng(11)
    yield "chesapeake", load_golden("chesapeake.npz")["offsets"]
    yield "sample", load_golden("sample.npz")["offsets"]
    for i in range(6):
        off, *_ = random_csr(rng, rows=int(rng.integers(1, 300)), cols=200, max_len=30,
                             empty_frac=0.3 * (i % 2))
        yield f"random{i}", off
    off, *_ = random_csr(rng, rows=50, cols=5000, max_len=3, long_rows=[(7, 4000)])
    yield "long_row", off
    yield "one_row", np.array([0, 57], dtype=np.int32)
    yield "no_nnz", np.zeros(17, dtype=np.int32)


@pytest.mark.parametrize("name,off", list(_cases()), ids=[c[0] for c in _cases()])
def test_search_matches_brute_force_walk(oracle_mod, name, off):
    nnz = int(off[-1])
    rows = len(off) - 1
    walk = oracle_mod.merge_path_walk(off, nnz, 1)  # coordinate at every diagonal
    for d in range(0, rows + nnz + 1):
        x, y = oracle_mod.mp_search(d, off[1:], rows, 0, nnz)
        assert (x, y) == tuple(walk[d]), (name, d)


@pytest.mark.parametrize("name,off", list(_cases()), ids=[c[0] for c in _cases()])
@pytest.mark.parametrize("tpb,ipt", [(128, 5), (64, 3), (32, 1)])
def test_tile_and_thread_coords(oracle_mod, name, off, tpb, ipt):
    nnz = int(off[-1])
    rows = len(off) - 1
    items = tpb * ipt
    walk = oracle_mod.merge_path_walk(off, nnz, 1)
    total = rows + nnz
    tiles = oracle_mod.merge_path_tile_coords(off, nnz, items)
    for t in range(len(tiles)):
        d = min(t * items, total)
        assert tuple(tiles[t]) == tuple(walk[d])
    th = oracle_mod.merge_path_thread_coords(off, nnz, tpb, ipt)
    for t in range(th.shape[0]):
        st = walk[min(t * items, total)]
        en = walk[min((t + 1) * items, total)]
        for tid in range(tpb):
            d = t * items + tid * ipt
            if d <= min((t + 1) * items, total):
                exp = walk[d] - st
            else:  # past the last item: the reference's search returns the tile end
                exp = en - st
            assert tuple(th[t, tid]) == tuple(exp), (t, tid)


@pytest.mark.parametrize("name,off", list(_cases()), ids=[c[0] for c in _cases()])
@pytest.mark.parametrize("nt", [1, 7, 256])
def test_work_oriented_coords(oracle_mod, name, off, nt):
    nnz = int(off[-1])
    rows = len(off) - 1
    total = rows + nnz
    walk = oracle_mod.merge_path_walk(off, nnz, 1)
    wpt = -(-total // nt)
    c = oracle_mod.work_oriented_coords(off, nnz, nt)
    for t in range(nt):
        up = min(wpt * t, total)
        lo = min(up + wpt, total)
        assert tuple(c[t, :2]) == tuple(walk[up]) and tuple(c[t, 2:]) == tuple(walk[lo])


@pytest.mark.parametrize("tpt", [32, 128])
def test_group_mapped_map_covers_every_nonzero_once(oracle_mod, tpt):
    rng = np.random.default_rng(5)
    off, idx, vals, x = random_csr(rng, rows=333, cols=100, max_len=20, empty_frac=0.2)
    rows_, nzs = oracle_mod.group_mapped_map(off, int(off[-1]), tpt)
    assert len(nzs) == off[-1]
    np.testing.assert_array_equal(np.sort(nzs), np.arange(off[-1]))
    row_of = np.repeat(np.arange(len(off) - 1), np.diff(off))
    np.testing.assert_array_equal(rows_, row_of[nzs])


def test_spmv_variants_agree(oracle_mod):
    rng = np.random.default_rng(3)
    off, idx, vals, x = random_csr(rng, rows=2000, cols=700, max_len=40, empty_frac=0.1)
    y = oracle_mod.spmv_f32(off, idx, vals, x)
    for th in (1, 3, 8):
        np.testing.assert_array_equal(oracle_mod.spmv_f32_mt(off, idx, vals, x, th), y)
    y64, yabs = oracle_mod.spmv_f64(off, idx, vals, x)
    row_of = np.repeat(np.arange(2000), np.diff(off))
    ref = np.zeros(2000)
    np.add.at(ref, row_of, vals.astype(np.float64) * x[idx].astype(np.float64))
    np.testing.assert_allclose(y64, ref, rtol=1e-12, atol=1e-12)
    comp, norm = oracle_mod.error_metrics(y, y64, yabs)
    assert comp < 40 * 2.0 ** -24 * 1.01


def test_spmv_f64_dequantises_exactly(oracle_mod):
    import torch
    rng = np.random.default_rng(9)
    off, idx, vals, x = random_csr(rng, rows=100, cols=100, max_len=10)
    v16 = vals.astype(np.float16)
    y16, _ = oracle_mod.spmv_f64(off, idx, v16, x)
    ref, _ = oracle_mod.spmv_f64(off, idx, v16.astype(np.float32), x)
    np.testing.assert_array_equal(y16, ref)
    vb = torch.from_numpy(vals).to(torch.bfloat16)
    yb, _ = oracle_mod.spmv_f64(off, idx, ("bf16", vb.view(torch.int16).numpy().view(np.uint16)),
                                x)
    refb, _ = oracle_mod.spmv_f64(off, idx, vb.float().numpy(), x)
    np.testing.assert_array_equal(yb, refb)
    scale = rng.choice([0.25, 1.0, 8.0], size=100).astype(np.float32)
    ys, _ = oracle_mod.spmv_f64(off, idx, v16, x, row_scale=scale)
    np.testing.assert_allclose(ys, y16 * scale, rtol=1e-15)


def test_spmm_loop(oracle_mod):
    rng = np.random.default_rng(4)
    off, idx, vals, x = random_csr(rng, rows=50, cols=60, max_len=8)
    B = rng.uniform(-1, 1, size=(60, 7)).astype(np.float32)
    Cm = oracle_mod.spmm_f32(off, idx, vals, B)
    for c in range(7):
        np.testing.assert_array_equal(Cm[:, c], oracle_mod.spmv_f32(off, idx, vals, B[:, c]))
    C64, Ca = oracle_mod.spmm_f64(off, idx, vals, B)
    for c in range(7):
        y64, ya = oracle_mod.spmv_f64(off, idx, vals, B[:, c])
        np.testing.assert_allclose(C64[:, c], y64, rtol=1e-15, atol=1e-300)


def test_split_points_property_random_shapes(oracle_mod):
    """Property check over many random row-length patterns (empty rows, one
    row, no nonzeros, long rows): the restated search, the tile split and the
    work_oriented split all land on the brute-force merge walk."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")

    @hyp.settings(max_examples=150, deadline=None, derandomize=True)
    @hyp.given(lens=st.lists(st.integers(0, 12), min_size=1, max_size=40),
               items=st.integers(1, 9), nt=st.integers(1, 23))
    def check(lens, items, nt):
        off = np.zeros(len(lens) + 1, dtype=np.int32)
        off[1:] = np.cumsum(lens)
        rows, nnz = len(lens), int(off[-1])
        total = rows + nnz
        walk = oracle_mod.merge_path_walk(off, nnz, 1)
        assert len(walk) == total + 1
        for d in range(total + 1):
            assert oracle_mod.mp_search(d, off[1:], rows, 0, nnz) == tuple(walk[d])
        tiles = oracle_mod.merge_path_tile_coords(off, nnz, items)
        for t in range(len(tiles)):
            assert tuple(tiles[t]) == tuple(walk[min(t * items, total)])
        c = oracle_mod.work_oriented_coords(off, nnz, nt)
        wpt = -(-total // nt)
        for t in range(nt):
            up = min(wpt * t, total)
            assert tuple(c[t, :2]) == tuple(walk[up])
            assert tuple(c[t, 2:]) == tuple(walk[min(up + wpt, total)])

    check()


@pytest.mark.parametrize("seed", range(8))
def test_weighted_merge_closed_form(oracle_mod, seed):
    """The closed form the GPU split-point test holds the kernel's weighted
    ranges to: equal to an item-by-item walk for row weights 1-3, and for
    weight 1 to the restated reference search (util/search.hxx:34-60)."""
    rng = np.random.default_rng(seed)
    rows = int(rng.integers(1, 60))
    off, _, _, _ = random_csr(rng, rows, 50, max_len=int(rng.integers(0, 12)),
                              empty_frac=float(rng.choice([0.0, 0.5])))
    nnz = int(off[-1])
    for w in (1, 2, 3):
        walk = merge_walk_weighted(off, w)
        d = np.arange(w * rows + nnz + 1, dtype=np.int64)
        x, n = merge_coords_weighted(off, d, w)
        np.testing.assert_array_equal(np.stack([x, n], 1), walk)
        if w == 1:
            for k in d:
                assert oracle_mod.mp_search(int(k), off[1:], rows, 0, nnz) == tuple(walk[k])
