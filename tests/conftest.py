import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built_lib():
    """Builds (if out of date) and returns the path of libedgeloops.so."""
    from edge_loops_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from edge_loops_gb300 import build
    build.build()
    return torch.device("cuda:0")


def load_golden(name):
    d = np.load(os.path.join(GOLDEN, name))
    return {k: d[k] for k in d.files}


def random_csr(rng, rows, cols, max_len, empty_frac=0.0, long_rows=()):
    """Small random CSR with sorted distinct columns per row (numpy)."""
    lens = rng.integers(0, max_len + 1, size=rows)
    if empty_frac:
        lens[rng.random(rows) < empty_frac] = 0
    for r, L in long_rows:
        lens[r] = L
    lens = np.minimum(lens, cols)
    off = np.zeros(rows + 1, dtype=np.int64)
    off[1:] = np.cumsum(lens)
    idx = np.empty(off[-1], dtype=np.int32)
    for r in range(rows):
        if lens[r]:
            idx[off[r]:off[r + 1]] = np.sort(rng.choice(cols, size=lens[r], replace=False))
    vals = rng.uniform(-1, 1, size=off[-1]).astype(np.float32)
    x = rng.uniform(-1, 1, size=cols).astype(np.float32)
    return off.astype(np.int32), idx, vals, x


def order_free_bound(offsets, yabs, extra=2):
    """Rigorous bound of |fp32 sum - exact| for ANY summation order of a
    row's n products (each rounded once): gamma_(n+extra) * sum |a x|."""
    u = 2.0 ** -24
    n = np.diff(offsets.astype(np.int64)) + extra
    return (n * u / (1 - n * u)) * yabs


def merge_coords_weighted(off, d, w):
    """Coordinates at diagonals d of the merge with every row end counted as w
    items (closed form)."""
    off = off.astype(np.int64)
    rows = len(off) - 1
    ends = off[1:] + w * np.arange(1, rows + 1, dtype=np.int64)
    x = np.searchsorted(ends, d, side="right")
    n = d - w * x
    lim = np.where(x < rows, off[np.minimum(x + 1, rows)], np.iinfo(np.int64).max)
    return x, np.minimum(n, lim)


def merge_walk_weighted(off, w):
    """Item-by-item walk of the weighted merge: the (row, nonzero) state after
    each number of items 0..w rows + nnz (a row end is w items; the row
    closes on its last one)."""
    rows = len(off) - 1
    r = n = 0
    out = [(0, 0)]
    pend = 0  # items of the current row end consumed so far
    while r < rows or n < off[-1]:
        if r < rows and n == off[r + 1]:
            pend += 1
            if pend == w:
                r, pend = r + 1, 0
        else:
            n += 1
        out.append((r, n))
    return np.array(out, dtype=np.int64)
