"""ctypes wrapper of oracle.c (TEST INFRASTRUCTURE ONLY; see __init__.py)."""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "oracle.c")
LIB = os.path.join(HERE, "liboracle.so")

__all__ = [
    "build", "spmv_f32", "spmv_f32_mt", "spmv_f64", "spmm_f32", "spmm_f64", "mp_search",
    "merge_path_tile_coords", "merge_path_thread_coords", "merge_path_walk",
    "work_oriented_coords", "group_mapped_map", "error_metrics", "matrix_market_coo",
    "csr_from_coo", "coo_sort", "edge_partition_coordinate", "edge_partition_position",
]


def build(force=False):
    """Compiles oracle.c -> liboracle.so with gcc (no FMA contraction)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = "%s.tmp%d" % (LIB, os.getpid())
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                               "-pthread", SRC, "-o", tmp, "-lm"])
        os.replace(tmp, LIB)
    return LIB


_lib = None


def _L():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        _lib.oracle_merge_path_tile_coords.restype = C.c_int64
        _lib.oracle_merge_path_thread_coords.restype = C.c_int64
        _lib.oracle_merge_path_walk.restype = C.c_int64
        _lib.oracle_group_mapped_map.restype = C.c_int64
        _lib.oracle_spmv_f32_mt.restype = C.c_int
    return _lib


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


_DT_CODE = {np.dtype(np.float32): 0, "bfloat16": 1, np.dtype(np.float16): 2}


def _values(values):
    """(array, dtype code) for float32 / float16 numpy arrays or bfloat16 given
    as a uint16 array tagged ('bf16', arr)."""
    if isinstance(values, tuple) and values[0] == "bf16":
        return _c(values[1], np.uint16), 1
    v = np.ascontiguousarray(values)
    if v.dtype == np.float16:
        return v, 2
    return _c(v, np.float32), 0


def spmv_f32(offsets, indices, values, x):
    """The reference CPU loop (examples/spmv/helpers.hxx:106-112), FP32."""
    off, idx = _c(offsets, np.int32), _c(indices, np.int32)
    val, xx = _c(values, np.float32), _c(x, np.float32)
    y = np.empty(len(off) - 1, dtype=np.float32)
    _L().oracle_spmv_f32(C.c_int64(len(y)), _p(off), _p(idx), _p(val), _p(xx), _p(y))
    return y


def spmv_f32_mt(offsets, indices, values, x, threads):
    """Same loop, rows split over `threads` host threads (identical y)."""
    off, idx = _c(offsets, np.int32), _c(indices, np.int32)
    val, xx = _c(values, np.float32), _c(x, np.float32)
    y = np.empty(len(off) - 1, dtype=np.float32)
    _L().oracle_spmv_f32_mt(C.c_int64(len(y)), _p(off), _p(idx), _p(val), _p(xx), _p(y),
                            C.c_int(threads))
    return y


def spmv_f64(offsets, indices, values, x, row_scale=None):
    """FP64 y over the exactly dequantised values, and sum_j |a_ij x_j|."""
    off, idx = _c(offsets, np.int32), _c(indices, np.int32)
    val, code = _values(values)
    xx = _c(x, np.float32)
    sc = _c(row_scale, np.float32) if row_scale is not None else None
    n = len(off) - 1
    y = np.empty(n, dtype=np.float64)
    ya = np.empty(n, dtype=np.float64)
    _L().oracle_spmv_f64_q(C.c_int64(n), _p(off), _p(idx), _p(val), C.c_int(code), _p(sc),
                           _p(xx), _p(y), _p(ya))
    return y, ya


def spmm_f32(offsets, indices, values, B):
    """The reference SpMM loop order (algorithms/spmm/thread_mapped.cuh:41-52)."""
    off, idx, val = _c(offsets, np.int32), _c(indices, np.int32), _c(values, np.float32)
    Bm = _c(B, np.float32)
    n = Bm.shape[1]
    Cm = np.empty((len(off) - 1, n), dtype=np.float32)
    _L().oracle_spmm_f32(C.c_int64(len(off) - 1), _p(off), _p(idx), _p(val), _p(Bm),
                         C.c_int64(n), C.c_int64(n), _p(Cm), C.c_int64(n))
    return Cm


def spmm_f64(offsets, indices, values, B, row_scale=None):
    """FP64 SpMM over dequantised values and B (float32/float16 array or
    ('bf16', uint16 array)); returns (C, sum |a b|)."""
    off, idx = _c(offsets, np.int32), _c(indices, np.int32)
    val, code = _values(values)
    Bv, bcode = _values(B)
    n = Bv.shape[1]
    rows = len(off) - 1
    sc = _c(row_scale, np.float32) if row_scale is not None else None
    Cm = np.empty((rows, n), dtype=np.float64)
    Ca = np.empty((rows, n), dtype=np.float64)
    _L().oracle_spmm_f64_q(C.c_int64(rows), _p(off), _p(idx), _p(val), C.c_int(code), _p(sc),
                           _p(Bv), C.c_int(bcode), C.c_int64(n), C.c_int64(n), _p(Cm), _p(Ca))
    return Cm, Ca


def mp_search(diag, a, a_len, b0, b_len):
    """util/search.hxx:34-60 restated: returns (x, y)."""
    aa = _c(a, np.int32)
    x, y = C.c_uint32(), C.c_uint32()
    _L().oracle_mp_search(C.c_int64(diag), _p(aa), C.c_int64(a_len), C.c_int64(b0),
                          C.c_int64(b_len), C.byref(x), C.byref(y))
    return x.value, y.value


def merge_path_tile_coords(offsets, nnz, items):
    off = _c(offsets, np.int32)
    rows = len(off) - 1
    tiles = (rows + nnz + items - 1) // items
    out = np.empty((tiles + 1) * 2, dtype=np.uint32)
    _L().oracle_merge_path_tile_coords(C.c_int64(rows), C.c_int64(nnz), _p(off),
                                       C.c_int64(items), _p(out))
    return out.reshape(tiles + 1, 2)


def merge_path_thread_coords(offsets, nnz, tpb, ipt):
    off = _c(offsets, np.int32)
    rows = len(off) - 1
    items = tpb * ipt
    tiles = (rows + nnz + items - 1) // items
    out = np.empty(max(tiles, 1) * tpb * 2, dtype=np.uint32)
    scratch = np.empty(items + ipt + 1, dtype=np.int32)
    _L().oracle_merge_path_thread_coords(C.c_int64(rows), C.c_int64(nnz), _p(off),
                                         C.c_int64(tpb), C.c_int64(ipt), _p(out), _p(scratch))
    return out[: tiles * tpb * 2].reshape(tiles, tpb, 2)


def merge_path_walk(offsets, nnz, step):
    off = _c(offsets, np.int32)
    rows = len(off) - 1
    out = np.empty(((rows + nnz) // step + 2) * 2, dtype=np.uint32)
    k = _L().oracle_merge_path_walk(C.c_int64(rows), C.c_int64(nnz), _p(off), C.c_int64(step),
                                    _p(out))
    return out[: 2 * k].reshape(k, 2)


def work_oriented_coords(offsets, nnz, num_threads):
    off = _c(offsets, np.int32)
    out = np.empty(num_threads * 4, dtype=np.int64)
    _L().oracle_work_oriented_coords(C.c_int64(len(off) - 1), C.c_int64(nnz), _p(off),
                                     C.c_int64(num_threads), _p(out))
    return out.reshape(num_threads, 4)


def group_mapped_map(offsets, nnz, tpt):
    off = _c(offsets, np.int32)
    rows_ = np.empty(max(nnz, 1), dtype=np.int32)
    nzs = np.empty(max(nnz, 1), dtype=np.int32)
    scan = np.empty(tpt, dtype=np.int32)
    w = _L().oracle_group_mapped_map(C.c_int64(len(off) - 1), _p(off), C.c_int64(tpt),
                                     _p(rows_), _p(nzs), _p(scan))
    return rows_[:w], nzs[:w]


def error_metrics(y, y64, yabs):
    """(max_i |y_i - y64_i| / sum_j |a_ij x_j|, ||y - y64||_inf / ||y64||_inf)
    against the FP64 oracle; rows whose sum |a x| is 0 must be exact."""
    y = np.asarray(y, dtype=np.float64)
    d = np.abs(y - y64)
    den = np.where(yabs > 0, yabs, 1.0)
    comp = float(np.max(d / den)) if len(d) else 0.0
    ninf = float(np.max(np.abs(y64))) if len(d) else 0.0
    norm = float(np.max(d) / ninf) if ninf > 0 else float(np.max(d) if len(d) else 0.0)
    return comp, norm


def matrix_market_coo(path):
    """The reference's MatrixMarket loader restated
    (include/loops/container/market.hxx:99-227): coordinate files, real /
    integer / pattern (value 1.0), 1-based -> 0-based, values read as double
    and stored as float32; for "symmetric" every off-diagonal entry is
    followed by its mirror (market.hxx:195-221).  Returns (rows, cols,
    row_indices, col_indices, values)."""
    with open(path) as f:
        banner = f.readline().split()
        field, symmetry = banner[3].lower(), banner[4].lower()
        lines = [ln for ln in f if ln.strip() and not ln.lstrip().startswith("%")]
    rows, cols, n = (int(t) for t in lines[0].split()[:3])
    ri, ci, vv = [], [], []
    for ln in lines[1:1 + n]:
        t = ln.split()
        i, j = int(t[0]) - 1, int(t[1]) - 1
        v = 1.0 if field == "pattern" else float(t[2])
        ri.append(i)
        ci.append(j)
        vv.append(v)
        if symmetry == "symmetric" and i != j:
            ri.append(j)
            ci.append(i)
            vv.append(v)
    return (rows, cols, np.array(ri, dtype=np.int32), np.array(ci, dtype=np.int32),
            np.array(vv, dtype=np.float64).astype(np.float32))


def csr_from_coo(rows, row_indices, col_indices, values):
    """The reference's CSR construction restated (container/csr.hxx:86-94):
    sort the entries by (row, column) (coo.hxx:104-113; a stable sort here,
    so equal entries keep their order), indices and values in that order,
    offsets[r] = lower_bound(sorted rows, r) (detail/convert.hxx:75-77)."""
    ri = np.asarray(row_indices, dtype=np.int64)
    ci = np.asarray(col_indices, dtype=np.int64)
    order = np.lexsort((ci, ri))  # stable
    offsets = np.searchsorted(ri[order], np.arange(rows + 1), side="left").astype(np.int32)
    return offsets, ci[order].astype(np.int32), np.asarray(values, dtype=np.float32)[order]


def coo_sort(row_indices, col_indices, values, by_column=False):
    """coo_t::sort_by_row / sort_by_column restated (container/coo.hxx:
    104-122): entries ordered by (row, column) or (column, row); stable, so
    equal entries keep their order."""
    ri = np.asarray(row_indices, dtype=np.int64)
    ci = np.asarray(col_indices, dtype=np.int64)
    order = np.lexsort((ri, ci)) if by_column else np.lexsort((ci, ri))
    return (ri[order].astype(np.int32), ci[order].astype(np.int32),
            np.asarray(values, dtype=np.float32)[order])


def _edge_layout(atom_quarks, atom_xy, tile_atoms):
    """The host-side WorkAtom / WorkTile structure flattened: quarks tile by
    tile, atom by atom; atom_begin (atoms in tile order); atom_x, atom_y;
    tile_begin."""
    quarks, atom_begin, ax, ay, tile_begin = [], [0], [], [], [0]
    for atoms in tile_atoms:
        for a in atoms:
            quarks.extend(atom_quarks[a])
            atom_begin.append(len(quarks))
            ax.append(atom_xy[a][0])
            ay.append(atom_xy[a][1])
        tile_begin.append(len(ax))
    i32 = lambda v: np.array(v, dtype=np.int32)  # noqa: E731
    return {"quarks": i32(quarks), "atom_begin": i32(atom_begin), "atom_x": i32(ax),
            "atom_y": i32(ay), "tile_begin": i32(tile_begin)}


def edge_partition_coordinate(rows, cols, row_indices, col_indices, M0, K0, M1, K1):
    """The reference's coordinate-space partition restated
    (util/partitioner.hxx:81-176) over a COO already sorted by row: atom of
    quark q = (row / M0) * atoms_y + col / K0, the quarks of each atom in q
    order (:103-117); atom a at (a / atoms_y, a % atoms_y) (:120-124); tile of
    atom = (x / M1) * tiles_y + y / K1 (:152-157), the atoms of each tile in
    atom order (:159-173).  Plain loops: small inputs only.  Raises
    ValueError on the reference's argument errors (:85-93, :133-143)."""
    if M0 <= 0 or K0 <= 0 or M0 > rows or K0 > cols:
        raise ValueError("bad atom size")
    nax, nay = (rows + M0 - 1) // M0, (cols + K0 - 1) // K0
    if M1 <= 0 or K1 <= 0 or M1 > nax or K1 > nay:
        raise ValueError("bad tile size")
    ntx, nty = (nax + M1 - 1) // M1, (nay + K1 - 1) // K1
    atom_quarks = [[] for _ in range(nax * nay)]
    for q, (r, c) in enumerate(zip(np.asarray(row_indices).tolist(),
                                   np.asarray(col_indices).tolist())):
        atom_quarks[(r // M0) * nay + c // K0].append(q)
    atom_xy = [(a // nay, a % nay) for a in range(nax * nay)]
    tile_atoms = [[] for _ in range(ntx * nty)]
    for a, (x, y) in enumerate(atom_xy):
        tile_atoms[(x // M1) * nty + y // K1].append(a)
    out = _edge_layout(atom_quarks, atom_xy, tile_atoms)
    out["atoms_x"], out["atoms_y"] = nax, nay
    return out


def edge_partition_position(nnz, nnz_per_atom, atoms_per_tile):
    """The reference's position-space partition restated
    (util/partitioner.hxx:178-226): atom i = quarks [i P, min(i P + P,
    nnz)) with coordinates (0, 0); tile t = atoms [t T, min(t T + T,
    atoms))."""
    if nnz_per_atom <= 0 or nnz_per_atom > nnz or atoms_per_tile <= 0:
        raise ValueError("bad atom or tile size")
    atoms = (nnz + nnz_per_atom - 1) // nnz_per_atom
    tiles = (atoms + atoms_per_tile - 1) // atoms_per_tile
    atom_quarks = [list(range(i * nnz_per_atom, min(i * nnz_per_atom + nnz_per_atom, nnz)))
                   for i in range(atoms)]
    tile_atoms = [list(range(t * atoms_per_tile, min(t * atoms_per_tile + atoms_per_tile,
                                                     atoms))) for t in range(tiles)]
    out = _edge_layout(atom_quarks, [(0, 0)] * atoms, tile_atoms)
    out["atoms_x"], out["atoms_y"] = 0, 0
    return out
