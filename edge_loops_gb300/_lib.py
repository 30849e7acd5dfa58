"""ctypes bindings of libedgeloops.so (the C ABI in include/edge_loops.h).

The library is loaded from this package's folder.  There is no fallback: if
the shared object is missing, loading raises, so nothing can silently run
another implementation.
"""
import ctypes as C
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libedgeloops.so")

# ---- enums / flags (mirror include/edge_loops.h) ---------------------------
EL_OK = 0
EL_ERR_INVALID_ARGUMENT = 1
EL_ERR_NULL_POINTER = 2
EL_ERR_OVERFLOW = 3
EL_ERR_UNSUPPORTED = 4
EL_ERR_MALFORMED_CSR = 5
EL_ERR_CUDA = 6
EL_ERR_OUT_OF_MEMORY = 7
EL_ERR_DEVICE = 8
EL_ERR_IO = 9
EL_ERR_PARSE = 10

EL_F32, EL_BF16, EL_F16 = 0, 1, 2

EL_SCHED_MERGE_PATH_FLAT = 0
EL_SCHED_WORK_ORIENTED = 1
EL_SCHED_THREAD_MAPPED = 2
EL_SCHED_GROUP_MAPPED = 3
EL_SCHED_BUCKETING = 4
EL_SCHED_AUTO = 5

EL_FLAG_INDEX_RANGE = 0x1
EL_FLAG_OFFSETS = 0x2
EL_FLAG_NNZ_MISMATCH = 0x4
EL_FLAG_TIMEOUT = 0x8


class ElCsr(C.Structure):
    _fields_ = [
        ("rows", C.c_int64),
        ("cols", C.c_int64),
        ("nnz", C.c_int64),
        ("offsets", C.c_void_p),
        ("indices", C.c_void_p),
        ("values", C.c_void_p),
        ("value_dtype", C.c_int32),
        ("reserved0", C.c_int32),
        ("row_scale", C.c_void_p),
    ]


class ElCoo(C.Structure):
    _fields_ = [
        ("rows", C.c_int64),
        ("cols", C.c_int64),
        ("nnz", C.c_int64),
        ("row_indices", C.c_void_p),
        ("col_indices", C.c_void_p),
        ("values", C.c_void_p),
    ]


class ElSpmvOpts(C.Structure):
    _fields_ = [
        ("threads_per_block", C.c_int32),
        ("items_per_thread", C.c_int32),
        ("threads_per_row", C.c_int32),
        ("group_rows", C.c_int32),
        ("num_threads", C.c_int64),
        ("compensated", C.c_int32),
        ("max_ctas", C.c_int32),
        ("wait_limit_us", C.c_int32),
        ("test_hooks", C.c_int32),
        ("variant", C.c_int32),
        ("row_weight", C.c_int32),
        ("nz_per_lane", C.c_int32),
        ("reserved", C.c_int32 * 3),
    ]


class ElEdgePartition(C.Structure):
    _fields_ = [
        ("nnz", C.c_int64),
        ("num_atoms", C.c_int64),
        ("num_tiles", C.c_int64),
        ("atoms_x", C.c_int64),
        ("atoms_y", C.c_int64),
        ("quarks", C.c_void_p),
        ("atom_begin", C.c_void_p),
        ("atom_x", C.c_void_p),
        ("atom_y", C.c_void_p),
        ("tile_begin", C.c_void_p),
    ]


class ElRowStats(C.Structure):
    _fields_ = [
        ("max_row_nnz", C.c_int64),
        ("empty_rows", C.c_int64),
        ("mean_row_nnz", C.c_double),
        ("cv", C.c_double),
        ("coherence", C.c_double),
    ]


class ElBatchItem(C.Structure):
    _fields_ = [("A", ElCsr), ("x", C.c_void_p), ("y", C.c_void_p)]


EL_BATCH_ROW_BUCKETS = 21
EL_BATCH_LEN_BUCKETS = 11
EL_BATCH_CV_BUCKETS = 4
EL_BATCH_TABLE_SIZE = EL_BATCH_ROW_BUCKETS * EL_BATCH_LEN_BUCKETS * EL_BATCH_CV_BUCKETS
EL_BATCH_MAX_ROW_NNZ = 16384
EL_BATCH_NZ_WALK = 64


class ElBatchOpts(C.Structure):
    _fields_ = [
        ("table", C.c_void_p),
        ("use_graph", C.c_int32),
        ("force_threads_per_row", C.c_int32),
        ("force_chunk_log2", C.c_int32),
        ("max_ctas", C.c_int32),
        ("reserved", C.c_int32 * 8),
    ]


# name -> (restype, argtypes); every symbol include/edge_loops.h declares
SIGNATURES = {
    "el_version": (C.c_int, []),
    "el_status_string": (C.c_char_p, [C.c_int]),
    "el_last_error_string": (C.c_char_p, []),
    "el_spmv_opts_default": (None, [C.POINTER(ElSpmvOpts)]),
    "el_workspace_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "el_workspace_destroy": (C.c_int, [C.c_void_p]),
    "el_workspace_errors": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_uint32), C.c_int]),
    "el_spmv": (C.c_int, [C.c_void_p, C.POINTER(ElCsr), C.c_int32, C.POINTER(ElSpmvOpts),
                          C.c_void_p, C.c_void_p, C.c_void_p]),
    "el_spmm": (C.c_int, [C.c_void_p, C.POINTER(ElCsr), C.c_int32, C.POINTER(ElSpmvOpts),
                          C.c_void_p, C.c_int32, C.c_int64, C.c_int64, C.c_void_p, C.c_int64,
                          C.c_void_p]),
    "el_csr_validate": (C.c_int, [C.POINTER(ElCsr), C.c_void_p, C.POINTER(C.c_uint32)]),
    "el_merge_path_num_tiles": (C.c_int64, [C.c_int64, C.c_int64, C.c_int32, C.c_int32]),
    "el_merge_path_partition": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int32,
                                          C.c_int32, C.c_void_p, C.c_void_p]),
    "el_merge_path_thread_coords": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int32,
                                              C.c_int32, C.c_void_p, C.c_void_p]),
    "el_work_oriented_partition": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int64,
                                             C.c_void_p, C.c_void_p]),
    "el_quantize_values": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_int32,
                                     C.c_void_p, C.c_void_p, C.c_void_p]),
    "el_batch_opts_default": (None, [C.POINTER(ElBatchOpts)]),
    "el_batch_plan_create": (C.c_int, [C.POINTER(ElBatchItem), C.c_int32,
                                       C.POINTER(ElBatchOpts), C.c_void_p,
                                       C.POINTER(C.c_void_p)]),
    "el_batch_plan_execute": (C.c_int, [C.c_void_p, C.c_void_p]),
    "el_batch_plan_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                     C.POINTER(C.c_int32)]),
    "el_batch_plan_errors": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_uint32), C.c_int]),
    "el_batch_plan_destroy": (C.c_int, [C.c_void_p]),
    "el_spmv_static_scratch": (C.c_int, [C.POINTER(ElCsr), C.c_void_p, C.c_void_p, C.c_int32,
                                         C.POINTER(C.c_uint32), C.c_void_p]),
    "el_spmv_static_scratch_errors": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32), C.c_int]),
    "el_spmv_host": (C.c_int, [C.c_void_p, C.POINTER(ElCsr), C.c_int32, C.POINTER(ElSpmvOpts),
                               C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "el_read_matrix_market": (C.c_int, [C.c_char_p, C.POINTER(ElCoo)]),
    "el_coo_free": (None, [C.POINTER(ElCoo)]),
    "el_csr_from_coo": (C.c_int, [C.c_void_p, C.POINTER(ElCoo), C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p]),
    "el_coo_sort": (C.c_int, [C.c_void_p, C.POINTER(ElCoo), C.c_int32, C.c_void_p]),
    "el_csr_row_indices": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p,
                                     C.c_void_p]),
    "el_edge_partition_coordinate_plan": (C.c_int, [C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                                    C.c_int64, C.c_int64, C.c_int64,
                                                    C.POINTER(ElEdgePartition)]),
    "el_edge_partition_position_plan": (C.c_int, [C.c_int64, C.c_int64, C.c_int64,
                                                  C.POINTER(ElEdgePartition)]),
    "el_edge_partition_coordinate": (C.c_int, [C.c_void_p, C.POINTER(ElCoo), C.c_int64,
                                               C.c_int64, C.c_int64, C.c_int64,
                                               C.POINTER(ElEdgePartition), C.c_void_p]),
    "el_edge_partition_position": (C.c_int, [C.c_int64, C.c_int64, C.POINTER(ElEdgePartition),
                                             C.c_void_p]),
    "el_csr_row_stats": (C.c_int, [C.c_void_p, C.POINTER(ElCsr), C.POINTER(ElRowStats),
                                   C.c_void_p]),
    "el_select_schedule": (C.c_int, [C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                     C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                     C.POINTER(C.c_double)]),
    "el_select_schedule_stats": (C.c_int, [C.c_int64, C.c_int64, C.c_int64,
                                           C.POINTER(ElRowStats), C.POINTER(C.c_int32),
                                           C.POINTER(ElSpmvOpts), C.POINTER(C.c_double)]),
    "el_spmv_select": (C.c_int, [C.c_void_p, C.POINTER(ElCsr), C.POINTER(C.c_int32),
                                 C.POINTER(ElSpmvOpts), C.c_void_p]),
    "el_debug_range_trace": (C.c_int, [C.c_void_p, C.c_int64]),
    "el_spmv_edge": (C.c_int, [C.c_void_p, C.POINTER(ElCoo), C.POINTER(ElEdgePartition),
                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
}

EL_STATIC_MAX_RANGES = 4096

_lib = None


def lib():
    """Loads libedgeloops.so once (raises OSError if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(
                "libedgeloops.so is not built (run `python -m edge_loops_gb300.build`); "
                "there is no fallback implementation")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class ElError(RuntimeError):
    """A non-EL_OK status from the C ABI."""

    def __init__(self, status, where):
        L = lib()
        self.status = status
        name = L.el_status_string(status).decode()
        msg = L.el_last_error_string().decode()
        super().__init__(f"{where}: {name}: {msg}")


def check(status, where):
    if status != EL_OK:
        raise ElError(status, where)
