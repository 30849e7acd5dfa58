"""Seeded synthetic CSR matrices for the five benchmark workloads.

The reference measures on SuiteSparse matrices, which are not available
here; these generators stand in for them with the shapes, sizes and value
distributions the workloads name.  They run with torch on the CPU (small
sizes, test fixtures) or on the GPU (full sizes); a given (seed, device)
always gives the same matrix.

Returned arrays: offsets int32 (rows+1), indices int32 (nnz, sorted within a
row), values float32, x float32.
"""
import math

import torch


def _gen(seed, device):
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    return g


def _uniform(n, lo, hi, g, device):
    return torch.rand(n, generator=g, device=device, dtype=torch.float32) * (hi - lo) + lo


def _offsets(lens):
    off = torch.zeros(lens.numel() + 1, dtype=torch.int64, device=lens.device)
    off[1:] = torch.cumsum(lens, 0)
    return off


def _sorted_distinct_columns(lens, off, cols, g, device):
    """Per row, lens[r] distinct columns in [0, cols), sorted: draw lens[r]
    values uniformly from [0, cols - lens[r]], sort them within the row and
    add 0, 1, 2, ... (a bijection from sorted multisets to sorted sets)."""
    rows = lens.numel()
    nnz = int(off[-1])
    row_of = torch.repeat_interleave(torch.arange(rows, device=device), lens)
    span = (cols - lens + 1).to(torch.float64)[row_of]
    raw = torch.floor(torch.rand(nnz, generator=g, device=device, dtype=torch.float64) * span)
    raw = torch.minimum(raw, span - 1).to(torch.int64)
    key = row_of * cols + raw
    key, _ = torch.sort(key)
    rank = torch.arange(nnz, device=device) - off[:-1][row_of]
    return (key - row_of * cols + rank).to(torch.int32)


def uniform_rows(rows=1000, cols=1000, per_row=10, seed=0, device="cpu"):
    """Every row has exactly `per_row` nonzeros in distinct uniformly drawn
    columns (sorted); values and x uniform in [-1, 1].

    Up to 2^24 cells the columns are the `per_row` smallest keys of a dense
    rows x cols uniform draw (the draw the committed fixtures were made
    with); larger shapes draw them per row without the dense matrix."""
    if per_row > cols:
        raise ValueError(f"per_row={per_row} exceeds cols={cols}")
    g = _gen(seed, device)
    off = torch.arange(0, rows * per_row + 1, per_row, device=device, dtype=torch.int64)
    if rows * cols <= (1 << 24):
        keys = torch.rand(rows, cols, generator=g, device=device)
        idx = torch.topk(keys, per_row, dim=1, largest=False).indices
        idx, _ = torch.sort(idx, dim=1)
    else:
        lens = torch.full((rows,), per_row, device=device, dtype=torch.int64)
        idx = _sorted_distinct_columns(lens, off, cols, g, device)
    vals = _uniform(rows * per_row, -1.0, 1.0, g, device)
    x = _uniform(cols, -1.0, 1.0, g, device)
    return off.to(torch.int32), idx.reshape(-1).to(torch.int32), vals, x, cols


def power_law(rows=1 << 20, cols=None, target_nnz=16_000_000, exponent=2.0, cap=100_000,
              seed=1, device="cpu"):
    """Row lengths from a Zipf(exponent) law on [1, cap] (inverse CDF),
    rescaled to about target_nnz in total (scale, round, clamp to
    [1, cap]); columns uniform, distinct and sorted per row; values and x
    uniform in [-1, 1]."""
    cols = rows if cols is None else cols
    cap = min(cap, cols)
    g = _gen(seed, device)
    k = torch.arange(1, cap + 1, device=device, dtype=torch.float64)
    pmf = k.pow(-exponent)
    cdf = torch.cumsum(pmf, 0)
    cdf = cdf / cdf[-1]
    u = torch.rand(rows, generator=g, device=device, dtype=torch.float64)
    lens = torch.searchsorted(cdf, u).clamp_(max=cap - 1).to(torch.float64) + 1.0
    lens = torch.clamp(torch.round(lens * (target_nnz / float(lens.sum()))), 1, cap).to(torch.int64)
    off = _offsets(lens)
    idx = _sorted_distinct_columns(lens, off, cols, g, device)
    vals = _uniform(idx.numel(), -1.0, 1.0, g, device)
    x = _uniform(cols, -1.0, 1.0, g, device)
    return off.to(torch.int32), idx, vals, x, cols


def stencil27(n=160, seed=2, device="cpu"):
    """27-point stencil on an n^3 grid (row = (i*n + j)*n + k): diagonal
    26.5, off-diagonals uniform in [-1, 0]; columns in natural (sorted)
    order; x uniform in [-1, 1].  nnz = (3n-2)^3."""
    g = _gen(seed, device)
    rows = n ** 3
    t = torch.arange(n, device=device)
    c1 = 3 - (t == 0).to(torch.int64) - (t == n - 1).to(torch.int64)  # per-dimension count
    lo1 = torch.where(t == 0, 0, -1)  # lowest valid offset per dimension
    ii = torch.arange(rows, device=device)
    i, j, k = ii // (n * n), (ii // n) % n, ii % n
    ci, cj, ck = c1[i], c1[j], c1[k]
    lens = ci * cj * ck
    off = _offsets(lens)
    nnz = int(off[-1])
    idx = torch.empty(nnz, dtype=torch.int32, device=device)
    vals = torch.empty(nnz, dtype=torch.float32, device=device)
    for di in (-1, 0, 1):
        for dj in (-1, 0, 1):
            for dk in (-1, 0, 1):
                ok = ((i + di >= 0) & (i + di < n) & (j + dj >= 0) & (j + dj < n)
                      & (k + dk >= 0) & (k + dk < n))
                r = ii[ok]
                ri = di - lo1[i[ok]]
                rj = dj - lo1[j[ok]]
                rk = dk - lo1[k[ok]]
                pos = off[r] + ri * cj[ok] * ck[ok] + rj * ck[ok] + rk
                idx[pos] = (r + di * n * n + dj * n + dk).to(torch.int32)
                if di == 0 and dj == 0 and dk == 0:
                    vals[pos] = 26.5
    offdiag = idx != torch.repeat_interleave(ii, lens).to(torch.int32)
    m = int(offdiag.sum())
    vals[offdiag] = _uniform(m, -1.0, 0.0, g, device)
    x = _uniform(rows, -1.0, 1.0, g, device)
    return off.to(torch.int32), idx, vals, x, rows


def batched(count=4096, rows_lo=64, rows_hi=65536, mean_per_row=8.0, sigma=1.0, seed=4,
            device="cpu"):
    """`count` square CSRs: rows log-uniform in [rows_lo, rows_hi]; nonzeros
    per row log-normal with arithmetic mean `mean_per_row` (mu = ln(mean) -
    sigma^2/2), rounded, at least 1, at most rows; columns uniform, distinct
    and sorted per row; values and each x uniform in [-1, 1].

    Returns (rows, offsets_cat, indices_cat, values_cat, x_cat, row_start,
    nz_start): matrix m's offsets (starting at 0) are
    offsets_cat[row_start[m] + m : row_start[m] + m + rows[m] + 1], its
    nonzeros indices_cat / values_cat[nz_start[m] : nz_start[m] + nnz_m], its
    x (and y) x_cat[row_start[m] : row_start[m] + rows[m]]."""
    g = _gen(seed, device)
    lr = torch.rand(count, generator=g, device=device, dtype=torch.float64)
    rows = torch.floor(torch.exp(math.log(rows_lo) + lr * (math.log(rows_hi) - math.log(rows_lo))))
    rows = rows.clamp(rows_lo, rows_hi).to(torch.int64)
    R = int(rows.sum())
    mu = math.log(mean_per_row) - sigma * sigma / 2
    z = torch.randn(R, generator=g, device=device, dtype=torch.float64)
    lens = torch.round(torch.exp(mu + sigma * z)).clamp_(min=1)
    mat_of_row = torch.repeat_interleave(torch.arange(count, device=device), rows)
    lens = torch.minimum(lens, rows[mat_of_row].to(torch.float64)).to(torch.int64)
    goff = _offsets(lens)  # global offsets over all rows
    # per-matrix distinct sorted columns: same construction with each row's
    # own column count
    nnz = int(goff[-1])
    row_of = torch.repeat_interleave(torch.arange(R, device=device), lens)
    ncol = rows[mat_of_row][row_of]
    span = (ncol - lens[row_of] + 1).to(torch.float64)
    raw = torch.floor(torch.rand(nnz, generator=g, device=device, dtype=torch.float64) * span)
    raw = torch.minimum(raw, span - 1).to(torch.int64)
    key = row_of * (rows_hi + 1) + raw
    key, _ = torch.sort(key)
    rank = torch.arange(nnz, device=device) - goff[:-1][row_of]
    idx = (key - row_of * (rows_hi + 1) + rank).to(torch.int32)
    vals = _uniform(nnz, -1.0, 1.0, g, device)
    x = _uniform(R, -1.0, 1.0, g, device)
    # per-matrix offsets (each starting at 0), concatenated: matrix m owns
    # rows[m] + 1 entries starting at cat_start[m] = row_start[m] + m
    row_start = _offsets(rows)[:-1]  # first global row of every matrix
    nz_start = goff[row_start]  # first global nonzero of every matrix
    cat_start = row_start + torch.arange(count, device=device)
    p = torch.arange(R + count, device=device)
    m = torch.searchsorted(cat_start, p, right=True) - 1
    off_cat = (goff[p - m] - nz_start[m]).to(torch.int32)
    return rows, off_cat, idx, vals, x, row_start, nz_start


def batch_as_one_csr(rows, off_cat, idx_cat, row_start, nz_start):
    """A batch from batched() as one block-diagonal CSR over all its rows:
    global offsets (matrix m's local offsets plus its first nonzero) and
    global column indices (matrix m's columns plus its first row; the
    matrices are square, so the batch's x and y are one vector each).
    Returns (offsets int32[R + 1], indices int32[nnz]) on the batch's
    device."""
    count = rows.numel()
    dev = off_cat.device
    R = int(rows.sum())
    nnz = idx_cat.numel()
    mat_of_row = torch.repeat_interleave(torch.arange(count, device=dev), rows)
    p = torch.arange(R, device=dev)
    goff = torch.empty(R + 1, dtype=torch.int64, device=dev)
    goff[:-1] = off_cat[p + mat_of_row].long() + nz_start[mat_of_row]
    goff[-1] = nnz
    nnz_m = torch.diff(torch.cat([nz_start, torch.tensor([nnz], device=dev)]))
    mat_of_nz = torch.repeat_interleave(torch.arange(count, device=dev), nnz_m)
    gidx = idx_cat.long() + row_start[mat_of_nz]
    return goff.to(torch.int32), gidx.to(torch.int32)


def algorithmic_bytes(rows, cols, nnz, value_bytes=4, row_scale=False):
    """Compulsory bytes of one SpMV: values + indices, offsets, x once, y
    written once (+ per-row scales)."""
    b = nnz * (value_bytes + 4) + 4 * (rows + 1) + 4 * cols + 4 * rows
    if row_scale:
        b += 4 * rows
    return b
