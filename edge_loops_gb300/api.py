"""Python face of the C ABI: CSR matrices held in torch device tensors, and
the reference's entry points (spmv / spmm per schedule) as functions.

Everything computed here runs in libedgeloops.so; torch only provides device
memory and the current CUDA stream.  The schedule names are the reference's
(loops::schedule::algorithms_t, include/loops/schedule.hxx:23-29, and the
entry points of include/loops/algorithms/spmv/*.cuh): "merge_path_flat"
(alias "merge_path"), "work_oriented", "thread_mapped" (alias "original"),
"group_mapped", plus "auto".
"""
import ctypes as C
import os

import torch

from . import _lib as L

SCHEDULES = {
    "merge_path_flat": L.EL_SCHED_MERGE_PATH_FLAT,
    "merge_path": L.EL_SCHED_MERGE_PATH_FLAT,
    "work_oriented": L.EL_SCHED_WORK_ORIENTED,
    "thread_mapped": L.EL_SCHED_THREAD_MAPPED,
    "original": L.EL_SCHED_THREAD_MAPPED,
    "group_mapped": L.EL_SCHED_GROUP_MAPPED,
    "bucketing": L.EL_SCHED_BUCKETING,
    "auto": L.EL_SCHED_AUTO,
}

_DT = {torch.float32: L.EL_F32, torch.bfloat16: L.EL_BF16, torch.float16: L.EL_F16}
_DT_BY_CODE = {v: k for k, v in _DT.items()}


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream(stream):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _check_vector(name, t, device, n, dtype=torch.float32):
    """t must be a contiguous `dtype` tensor of at least n entries on `device`
    (the library reads n entries from its first element)."""
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}")
    if t.device != device:
        raise ValueError(f"{name} is on {t.device}, the matrix on {device}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if t.numel() < n:
        raise ValueError(f"{name} holds {t.numel()} entries, needs {n}")


def _check_on_gpu(A):
    if A.device.type != "cuda":
        raise ValueError("the matrix is in host memory: use spmv_host, or move it to the GPU")


def _sched(schedule):
    if isinstance(schedule, int):
        return schedule
    try:
        return SCHEDULES[schedule]
    except KeyError:
        raise ValueError(f"unknown schedule {schedule!r}; one of {sorted(SCHEDULES)}")


class CSR:
    """A CSR matrix in device memory (the reference's csr_t,
    include/loops/container/csr.hxx:32-95): int32 offsets (rows+1), int32
    column indices and values (float32, bfloat16 or float16), with an
    optional float32 per-row scale (A[i, j] = row_scale[i] * values[ij])."""

    def __init__(self, offsets, indices, values, rows, cols, row_scale=None):
        self.offsets = offsets
        self.indices = indices
        self.values = values
        self.rows = int(rows)
        self.cols = int(cols)
        self.row_scale = row_scale
        # the library reads these as plain arrays from their first element
        if values.dtype not in _DT:
            raise TypeError(f"values dtype {values.dtype} not supported")
        if offsets.dtype != torch.int32 or indices.dtype != torch.int32:
            raise TypeError("offsets and indices must be int32")
        if row_scale is not None and row_scale.dtype != torch.float32:
            raise TypeError("row_scale must be float32")
        arrays = [offsets, indices, values] + ([row_scale] if row_scale is not None else [])
        if any(t.device != offsets.device for t in arrays):
            raise ValueError("offsets, indices, values and row_scale must be on one device")
        if not all(t.is_contiguous() for t in arrays):
            raise ValueError("offsets, indices, values and row_scale must be contiguous")
        if self.rows < 0 or self.cols < 0 or offsets.numel() < self.rows + 1:
            raise ValueError("offsets must hold rows + 1 entries")
        if values.numel() < indices.numel():
            raise ValueError("values must hold an entry per index")
        if row_scale is not None and row_scale.numel() < self.rows:
            raise ValueError("row_scale must hold an entry per row")

    @property
    def nnz(self):
        return int(self.indices.numel())

    @property
    def nnzs(self):  # the reference's field name
        return self.nnz

    @property
    def device(self):
        return self.offsets.device

    def el(self):
        s = L.ElCsr()
        s.rows, s.cols, s.nnz = self.rows, self.cols, self.nnz
        s.offsets = self.offsets.data_ptr()
        s.indices = self.indices.data_ptr() if self.nnz else None
        s.values = self.values.data_ptr() if self.nnz else None
        s.value_dtype = _DT[self.values.dtype]
        s.row_scale = self.row_scale.data_ptr() if self.row_scale is not None else None
        return s

    @classmethod
    def from_arrays(cls, offsets, indices, values, cols, device="cuda", rows=None):
        """From numpy/torch host arrays (copied to `device`)."""
        off = torch.as_tensor(offsets, dtype=torch.int32).to(device)
        idx = torch.as_tensor(indices, dtype=torch.int32).to(device)
        val = torch.as_tensor(values).to(device)
        r = int(off.numel() - 1) if rows is None else int(rows)
        return cls(off, idx, val, r, cols)

    def quantized(self, dtype, per_row_scale=True, stream=None, out=None, out_scale=None):
        """BF16/FP16 copy of an FP32 matrix (el_quantize_values); with
        per_row_scale each row is divided by a power of two that puts its
        largest magnitude in [1, 2) (BF16) or [2^14, 2^15) (FP16).

        out / out_scale: where to write the values (nnz) and scales (rows),
        e.g. slices of one array holding many matrices at the same element
        offsets as their indices -- the kernels load whole tiles with
        128-bit loads only where indices and values share their position
        modulo 8 elements."""
        if self.values.dtype != torch.float32:
            raise TypeError("quantize an FP32 matrix")
        if out is None:
            out = torch.empty(self.nnz, dtype=dtype, device=self.device)
        if out.dtype != dtype or out.numel() != self.nnz or not out.is_contiguous():
            raise ValueError("out must be a contiguous tensor of nnz elements of dtype")
        scale = None
        if per_row_scale:
            scale = out_scale if out_scale is not None else \
                torch.empty(self.rows, dtype=torch.float32, device=self.device)
            if scale.dtype != torch.float32 or scale.numel() != self.rows:
                raise ValueError("out_scale must hold rows float32 values")
        L.check(L.lib().el_quantize_values(
            _ptr(self.offsets), self.rows, self.nnz, _ptr(self.values), _DT[dtype],
            _ptr(out), _ptr(scale), _stream(stream)), "el_quantize_values")
        return CSR(self.offsets, self.indices, out, self.rows, self.cols, row_scale=scale)


class Workspace:
    """An el_workspace (device state of the persistent schedules)."""

    def __init__(self, device=None):
        dev = torch.cuda.current_device() if device is None else int(device)
        h = C.c_void_p()
        L.check(L.lib().el_workspace_create(dev, C.byref(h)), "el_workspace_create")
        self.handle = h

    def errors(self, clear=True, stream=None):
        return workspace_errors(self, clear=clear, stream=stream)

    def close(self):
        if self.handle:
            L.lib().el_workspace_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _ws(ws):
    return None if ws is None else ws.handle


def workspace_errors(ws=None, clear=True, stream=None):
    """Device error flags (EL_FLAG_*) of a workspace, or of the library's
    workspace for the current device and stream when ws is None."""
    f = C.c_uint32(0)
    L.check(L.lib().el_workspace_errors(_ws(ws), _stream(stream), C.byref(f), int(clear)),
            "el_workspace_errors")
    return int(f.value)


def make_opts(threads_per_block=0, items_per_thread=0, threads_per_row=0, group_rows=0,
              num_threads=0, compensated=False, max_ctas=0, wait_limit_us=0, variant=0,
              row_weight=0, nz_per_lane=0):
    o = L.ElSpmvOpts()
    L.lib().el_spmv_opts_default(C.byref(o))
    o.threads_per_block = threads_per_block
    o.items_per_thread = items_per_thread
    o.threads_per_row = threads_per_row
    o.group_rows = group_rows
    o.num_threads = num_threads
    o.compensated = int(bool(compensated))
    o.max_ctas = max_ctas
    o.wait_limit_us = wait_limit_us
    o.variant = variant
    o.row_weight = row_weight
    o.nz_per_lane = nz_per_lane
    return o


def spmv(A, x, y=None, schedule="merge_path_flat", stream=None, workspace=None, **opts):
    """y = A x (y overwritten), the reference's
    loops::algorithms::spmv::<schedule>(csr, x, y, stream)."""
    _check_on_gpu(A)
    _check_vector("x", x, A.device, A.cols)
    if y is None:
        y = torch.empty(A.rows, dtype=torch.float32, device=A.device)
    _check_vector("y", y, A.device, A.rows)
    a = A.el()
    o = make_opts(**opts)
    L.check(L.lib().el_spmv(_ws(workspace), C.byref(a), _sched(schedule), C.byref(o),
                            _ptr(x), _ptr(y), _stream(stream)), "el_spmv")
    return y


def row_stats(A, stream=None, workspace=None):
    """el_csr_row_stats: longest row, empty rows, mean row length and its
    coefficient of variation, and the row-to-row coherence of the columns
    (synchronises the stream)."""
    st = L.ElRowStats()
    a = A.el()
    L.check(L.lib().el_csr_row_stats(_ws(workspace), C.byref(a), C.byref(st), _stream(stream)),
            "el_csr_row_stats")
    return {"max_row_nnz": int(st.max_row_nnz), "empty_rows": int(st.empty_rows),
            "mean_row_nnz": float(st.mean_row_nnz), "cv": float(st.cv),
            "coherence": float(st.coherence)}


def select_schedule(A, stream=None, workspace=None):
    """el_spmv_select: (schedule name, options) for spmv(A, x, schedule=...,
    **options), chosen once from A's row statistics by the cost model."""
    sched = C.c_int32(0)
    o = make_opts()
    a = A.el()
    L.check(L.lib().el_spmv_select(_ws(workspace), C.byref(a), C.byref(sched), C.byref(o),
                                   _stream(stream)), "el_spmv_select")
    if sched.value == L.EL_SCHED_THREAD_MAPPED:
        opts = {"threads_per_row": int(o.threads_per_row)}
        if o.variant:
            opts["variant"] = int(o.variant)  # rows staged through shared memory
        return "thread_mapped", opts
    return "merge_path_flat", {}


def spmv_host(A, x, y=None, schedule="merge_path_flat", block_nnz=0, stream=None,
              workspace=None, **opts):
    """el_spmv_host: y = A x with A (CSR of CPU tensors), x and y in host
    memory, streamed to the current GPU in row blocks that overlap the copies
    with the SpMV.  Pin the tensors (`.pin_memory()`) for full link speed.
    Asynchronous: synchronise the stream before reading y or reusing A, x."""
    if A.offsets.is_cuda:
        raise ValueError("spmv_host takes a matrix in host (CPU) memory")
    _check_vector("x", x, A.device, A.cols)
    if y is None:
        y = torch.empty(A.rows, dtype=torch.float32).pin_memory()
    _check_vector("y", y, A.device, A.rows)
    a = A.el()
    o = make_opts(**opts)
    L.check(L.lib().el_spmv_host(_ws(workspace), C.byref(a), _sched(schedule), C.byref(o),
                                 _ptr(x), _ptr(y), int(block_nnz), _stream(stream)),
            "el_spmv_host")
    return y


def read_matrix_market(path):
    """el_read_matrix_market: (rows, cols, row_indices, col_indices, values)
    of a MatrixMarket coordinate file as numpy arrays (0-based; symmetric
    files with their mirrored entries), the reference's
    matrix_market_t::load."""
    import numpy as np
    coo = L.ElCoo()
    L.check(L.lib().el_read_matrix_market(os.fsencode(path), C.byref(coo)),
            "el_read_matrix_market")
    try:
        n = int(coo.nnz)
        def arr(ptr, ctype, dtype):
            if n == 0:
                return np.zeros(0, dtype=dtype)
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ctype)), shape=(n,)).copy()
        ri = arr(coo.row_indices, C.c_int32, np.int32)
        ci = arr(coo.col_indices, C.c_int32, np.int32)
        vv = arr(coo.values, C.c_float, np.float32)
        return int(coo.rows), int(coo.cols), ri, ci, vv
    finally:
        L.lib().el_coo_free(C.byref(coo))


def csr_from_coo(rows, cols, row_indices, col_indices, values, device=None, stream=None,
                 workspace=None):
    """el_csr_from_coo: a CSR (device) from COO entries (tensors or arrays,
    copied to the device), sorted by (row, column) with duplicates kept in
    input order, the reference's csr_t(coo_t)."""
    dev = torch.device(device) if device is not None else torch.device(
        "cuda", torch.cuda.current_device())
    ri = torch.as_tensor(row_indices, dtype=torch.int32).to(dev).contiguous()
    ci = torch.as_tensor(col_indices, dtype=torch.int32).to(dev).contiguous()
    vv = torch.as_tensor(values, dtype=torch.float32).to(dev).contiguous()
    nnz = int(ri.numel())
    off = torch.empty(int(rows) + 1, dtype=torch.int32, device=dev)
    idx = torch.empty(nnz, dtype=torch.int32, device=dev)
    val = torch.empty(nnz, dtype=torch.float32, device=dev)
    coo = L.ElCoo()
    coo.rows, coo.cols, coo.nnz = int(rows), int(cols), nnz
    coo.row_indices = ri.data_ptr() if nnz else None
    coo.col_indices = ci.data_ptr() if nnz else None
    coo.values = vv.data_ptr() if nnz else None
    L.check(L.lib().el_csr_from_coo(_ws(workspace), C.byref(coo), _ptr(off),
                                    _ptr(idx) if nnz else None, _ptr(val) if nnz else None,
                                    _stream(stream)), "el_csr_from_coo")
    return CSR(off, idx, val, int(rows), int(cols))


def spmm(A, B, Cm=None, schedule="merge_path_flat", stream=None, workspace=None, **opts):
    """C = A B with B row-major (cols x n) float32/bfloat16/float16 and C
    float32 (rows x n), the reference's loops::algorithms::spmm."""
    _check_on_gpu(A)
    if B.dim() != 2 or B.shape[0] != A.cols or B.stride(1) != 1 or B.stride(0) < B.shape[1]:
        raise ValueError("B must be a row-major (cols x n) matrix")
    if B.dtype not in _DT or B.device != A.device:
        raise ValueError("B must be float32/bfloat16/float16 on the matrix's device")
    n = B.shape[1]
    if Cm is None:
        Cm = torch.empty(A.rows, n, dtype=torch.float32, device=A.device)
    if Cm.dtype != torch.float32 or Cm.stride(1) != 1 or Cm.shape != (A.rows, n) or \
            Cm.stride(0) < n or Cm.device != A.device:
        raise ValueError("C must be float32 row-major (rows x n) on the matrix's device")
    a = A.el()
    o = make_opts(**opts)
    L.check(L.lib().el_spmm(_ws(workspace), C.byref(a), _sched(schedule), C.byref(o),
                            _ptr(B), _DT[B.dtype], n, B.stride(0), _ptr(Cm), Cm.stride(0),
                            _stream(stream)), "el_spmm")
    return Cm


def validate(A, stream=None):
    """Returns the EL_FLAG_* defects of A (0 for a well-formed CSR)."""
    a = A.el()
    f = C.c_uint32(0)
    st = L.lib().el_csr_validate(C.byref(a), _stream(stream), C.byref(f))
    if st not in (L.EL_OK, L.EL_ERR_MALFORMED_CSR):
        L.check(st, "el_csr_validate")
    return int(f.value)


def merge_path_partition(offsets, rows, nnz, tpb=128, ipt=5, stream=None):
    """Tile start coordinates (row, nonzero) at diagonals k*tpb*ipt plus the
    end of the last tile: uint32 tensor of shape (tiles+1, 2)."""
    tiles = int(L.lib().el_merge_path_num_tiles(rows, nnz, tpb, ipt))
    out = torch.empty((tiles + 1) * 2, dtype=torch.int32, device=offsets.device)
    L.check(L.lib().el_merge_path_partition(_ptr(offsets), rows, nnz, tpb, ipt, _ptr(out),
                                            _stream(stream)), "el_merge_path_partition")
    return out.view(tiles + 1, 2)


def merge_path_thread_coords(offsets, rows, nnz, tpb=128, ipt=5, stream=None):
    """Per (tile, thread) local start coordinate: shape (tiles, tpb, 2)."""
    tiles = int(L.lib().el_merge_path_num_tiles(rows, nnz, tpb, ipt))
    out = torch.empty(max(tiles, 1) * tpb * 2, dtype=torch.int32, device=offsets.device)
    L.check(L.lib().el_merge_path_thread_coords(_ptr(offsets), rows, nnz, tpb, ipt,
                                                _ptr(out), _stream(stream)),
            "el_merge_path_thread_coords")
    return out[: tiles * tpb * 2].view(tiles, tpb, 2)


def work_oriented_partition(offsets, rows, nnz, num_threads, stream=None):
    """Per thread (start row, start nz, end row, end nz): shape (num_threads, 4)."""
    out = torch.empty(num_threads * 4, dtype=torch.int64, device=offsets.device)
    L.check(L.lib().el_work_oriented_partition(_ptr(offsets), rows, nnz, num_threads,
                                               _ptr(out), _stream(stream)),
            "el_work_oriented_partition")
    return out.view(num_threads, 4)


# ---------------------------------------------------------------- batched SpMV
def tuning_table(entries):
    """int32[EL_BATCH_TABLE_SIZE] from {"rb,lb,cb": [threads_per_row, chunk_log2]}."""
    import numpy as np
    t = np.zeros(L.EL_BATCH_TABLE_SIZE, dtype=np.int32)
    for key, (tpr, chunk_log2) in entries.items():
        rb, lb, cb = (int(v) for v in key.split(","))
        idx = (rb * L.EL_BATCH_LEN_BUCKETS + lb) * L.EL_BATCH_CV_BUCKETS + cb
        t[idx] = int(tpr) | (int(chunk_log2) << 8)
    return t


def load_tuning_table(path=None):
    """The batched tuning table (int32[EL_BATCH_TABLE_SIZE]) from the JSON the
    tuner wrote (edge_loops_gb300/batch_tuning.json by default), or None."""
    import json
    import os
    path = path or os.path.join(os.path.dirname(os.path.abspath(__file__)), "batch_tuning.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    return tuning_table(d["entries"])


def batch_item_array(items, count=None):
    """The el_batch_item array of a list of (CSR, x, y), for the first `count`
    of them (all by default); the tensors must outlive every plan made from
    it."""
    n = len(items) if count is None else count
    arr = (L.ElBatchItem * max(n, 1))()
    for i in range(n):
        A, x, y = items[i]
        arr[i].A = A.el()
        arr[i].x = x.data_ptr() if x is not None and x.numel() else None
        arr[i].y = y.data_ptr() if y is not None and y.numel() else None
    return arr


class BatchPlan:
    """el_batch_plan: y_i = A_i x_i for many independent matrices in one
    persistent launch captured in a CUDA graph.  `items` is a list of
    (CSR, x, y); the tensors must stay alive (the plan keeps references)."""

    def __init__(self, items, table="default", use_graph=True, force_threads_per_row=0,
                 force_chunk_log2=0, max_ctas=0, stream=None):
        import numpy as np
        self._keep = list(items)
        arr = batch_item_array(items)
        o = L.ElBatchOpts()
        L.lib().el_batch_opts_default(C.byref(o))
        if isinstance(table, str) and table == "default":
            table = load_tuning_table()
        self._table = None if table is None else np.ascontiguousarray(table, dtype=np.int32)
        o.table = self._table.ctypes.data if self._table is not None else None
        o.use_graph = int(bool(use_graph))
        o.force_threads_per_row = force_threads_per_row
        o.force_chunk_log2 = force_chunk_log2
        o.max_ctas = max_ctas
        h = C.c_void_p()
        L.check(L.lib().el_batch_plan_create(arr, len(self._keep), C.byref(o), _stream(stream),
                                             C.byref(h)), "el_batch_plan_create")
        self.handle = h

    @classmethod
    def from_array(cls, arr, count, keep, force_threads_per_row=0, force_chunk_log2=0,
                   use_graph=True, stream=None, table=None):
        """A plan over the first `count` entries of a prebuilt
        batch_item_array (`keep` holds the tensors; `table` an int32 tuning
        table or None for the built-in rule)."""
        import numpy as np
        self = cls.__new__(cls)
        self._keep = keep
        self._table = None if table is None else np.ascontiguousarray(table, dtype=np.int32)
        o = L.ElBatchOpts()
        L.lib().el_batch_opts_default(C.byref(o))
        o.table = self._table.ctypes.data if self._table is not None else None
        o.use_graph = int(bool(use_graph))
        o.force_threads_per_row = force_threads_per_row
        o.force_chunk_log2 = force_chunk_log2
        h = C.c_void_p()
        L.check(L.lib().el_batch_plan_create(arr, count, C.byref(o), _stream(stream),
                                             C.byref(h)), "el_batch_plan_create")
        self.handle = h
        return self

    def execute(self, stream=None):
        L.check(L.lib().el_batch_plan_execute(self.handle, _stream(stream)),
                "el_batch_plan_execute")

    def info(self):
        w = C.c_int64()
        t = (C.c_int32 * 7)()
        hv = C.c_int32()
        L.check(L.lib().el_batch_plan_info(self.handle, C.byref(w), t, C.byref(hv)),
                "el_batch_plan_info")
        return {"work_items": int(w.value),
                "matrices_by_threads_per_row": {1 << i: int(t[i]) for i in range(6)},
                "matrices_nz_walk": int(t[6]),
                "heavy_matrices": int(hv.value)}

    def errors(self, clear=True, stream=None):
        f = C.c_uint32(0)
        L.check(L.lib().el_batch_plan_errors(self.handle, _stream(stream), C.byref(f),
                                             int(clear)), "el_batch_plan_errors")
        return int(f.value)

    def close(self):
        if getattr(self, "handle", None):
            L.lib().el_batch_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batched_items(rows, off_cat, idx, vals, x_cat, row_start, nz_start, y_cat=None,
                  row_scale_cat=None):
    """CSR views of the concatenated arrays synth.batched returns: a list of
    (CSR, x, y) with y slices of y_cat (allocated if None)."""
    dev = off_cat.device
    if y_cat is None:
        y_cat = torch.empty(x_cat.numel(), dtype=torch.float32, device=dev)
    rows_l = rows.tolist()
    rs_l = row_start.tolist()
    ns_l = nz_start.tolist()
    out = []
    for m, r in enumerate(rows_l):
        o = off_cat[rs_l[m] + m: rs_l[m] + m + r + 1]
        nnz = int(o[-1]) if r else 0
        A = CSR(o, idx[ns_l[m]: ns_l[m] + nnz], vals[ns_l[m]: ns_l[m] + nnz], r, r,
                row_scale=None if row_scale_cat is None else
                row_scale_cat[rs_l[m]: rs_l[m] + r])
        out.append((A, x_cat[rs_l[m]: rs_l[m] + r], y_cat[rs_l[m]: rs_l[m] + r]))
    return out, y_cat
