"""Bounds of thread_mapped's staged kernel (csrc/spmv_schedules.cuh,
thread_mapped_staged_kernel), checked on the CPU: the chunk-staging
arithmetic restated and run over random and edge-case offsets.  For every
chunk of 32 rows it decides, as the kernel does, whether the chunk is staged;
if so it asserts that the two bulk copies start 16-byte aligned, have sizes
that are multiples of 16, read only [0, nnz) and land inside the warp's
buffers, that the lane-0 tail loads read only [0, nnz) and write inside the
buffers, and that every lane's walk reads only shared-memory positions that
a copy or a tail load wrote."""
import numpy as np
import pytest

CAP = 880  # TmStage::kCap


def stage_plan(off, rows, nnz, cols, q, vbytes):
    """The kernel's stage() for chunk q: None (not staged) or the copies."""
    r0 = q * 32
    last = min(rows - r0, 32) - 1
    lo = off[r0: r0 + last + 1].astype(np.int64)
    hi = off[r0 + 1: r0 + last + 2].astype(np.int64)
    b0, e0 = int(lo[0]), int(hi[-1])
    ok = bool(np.all((lo >= b0) & (lo <= hi) & (hi <= e0)))
    vpu = 16 // vbytes
    i0 = b0 & ~3
    v0 = b0 & ~(vpu - 1)
    ni = (e0 - i0 + 3) >> 2
    nv = (e0 - v0 + vpu - 1) // vpu
    idx_bytes = CAP * 4
    val_bytes = (CAP * vbytes + 15) // 16 * 16
    fits = cols > 0 and b0 >= 0 and e0 <= nnz and b0 <= e0 and ni * 16 <= idx_bytes \
        and nv * 16 <= val_bytes
    if not (ok and fits):
        return None
    fi = min(ni, (nnz - i0) >> 2)
    fv = min(nv, (nnz - v0) // vpu)
    return dict(b0=b0, e0=e0, i0=i0, v0=v0, ni=ni, nv=nv, fi=fi, fv=fv, vpu=vpu,
                idx_bytes=idx_bytes, val_bytes=val_bytes, lo=lo, hi=hi)


def check_chunk(p, nnz, vbytes):
    i0, v0, fi, fv, vpu = p["i0"], p["v0"], p["fi"], p["fv"], p["vpu"]
    # bulk copies: 16-byte aligned source (element offset a multiple of the
    # unit), sizes multiples of 16, inside [0, nnz) and inside the buffers
    assert i0 % 4 == 0 and v0 % vpu == 0
    assert 0 <= i0 and i0 + 4 * fi <= nnz and 0 <= v0 and v0 + vpu * fv <= nnz
    assert 16 * fi <= p["idx_bytes"] and 16 * fv <= p["val_bytes"]
    # tail loads by lane 0: elements [i0 + 4 fi, e0) and [v0 + vpu fv, e0)
    written_i = np.zeros(p["idx_bytes"] // 4, bool)
    written_i[:4 * fi] = True
    for el in range(i0 + 4 * fi, p["e0"]):
        assert 0 <= el < nnz and 0 <= el - i0 < len(written_i)
        written_i[el - i0] = True
    written_v = np.zeros(p["val_bytes"] // vbytes, bool)
    written_v[:vpu * fv] = True
    for el in range(v0 + vpu * fv, p["e0"]):
        assert 0 <= el < nnz and 0 <= el - v0 < len(written_v)
        written_v[el - v0] = True
    # each lane reads positions lo - i0 + j and lo - v0 + j for j < hi - lo
    for lo, hi in zip(p["lo"], p["hi"]):
        if hi > lo:
            assert written_i[lo - i0: hi - i0].all()
            assert written_v[lo - v0: hi - v0].all()


def run_matrix(off, cols, vbytes):
    rows = len(off) - 1
    nnz = int(off[-1]) if rows else 0
    staged = 0
    for q in range((rows + 31) // 32):
        p = stage_plan(off, rows, nnz, cols, q, vbytes)
        if p is not None:
            staged += 1
            check_chunk(p, nnz, vbytes)
    return staged


@pytest.mark.parametrize("vbytes", [4, 2])
def test_staging_stays_in_bounds(vbytes):
    rng = np.random.default_rng(71)
    cases = []
    for rows in (1, 5, 31, 32, 33, 64, 100, 1000):
        for max_len in (0, 1, 3, 8, 27, 28, 40):
            lens = rng.integers(0, max_len + 1, rows)
            cases.append(np.concatenate([[0], np.cumsum(lens)]).astype(np.int64))
    # every row 27 long (the stencil's worst case), a few long rows, all empty
    cases.append(np.arange(0, 27 * 96 + 1, 27, dtype=np.int64))
    lens = rng.integers(0, 10, 200)
    lens[[3, 77]] = [900, 2000]
    cases.append(np.concatenate([[0], np.cumsum(lens)]).astype(np.int64))
    cases.append(np.zeros(65, np.int64))
    total = 0
    for off in cases:
        total += run_matrix(off, cols=50, vbytes=vbytes)
    assert total > 100  # most chunks of short rows are staged
    # malformed offsets: decreasing, past nnz, negative -- never staged past
    # the array, and what is staged stays in bounds
    for _ in range(200):
        rows = int(rng.integers(1, 100))
        off = np.sort(rng.integers(0, 300, rows + 1)).astype(np.int64)
        off[0] = 0
        k = int(rng.integers(0, rows + 1))
        off[k] = int(rng.integers(-5, 400))
        nnz = int(max(off[-1], 0))
        off[-1] = nnz
        for q in range((rows + 31) // 32):
            p = stage_plan(off, rows, nnz, 50, q, vbytes)
            if p is not None:
                check_chunk(p, nnz, vbytes)


def test_the_stencil_rows_always_fit():
    """kStagedMaxRow: 32 rows of 27 nonzeros fit from any start, for both
    value widths (the static_asserts beside the kernel, restated)."""
    for vbytes in (4, 2):
        for start in range(16):
            # rows 0-31: `start` nonzeros in row 0; rows 32-63: 27 each
            lens = np.array([start] + [0] * 31 + [27] * 32)
            off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
            p = stage_plan(off, 64, int(off[-1]), 10, 1, vbytes)
            assert p is not None and p["b0"] == start
            check_chunk(p, int(off[-1]), vbytes)
