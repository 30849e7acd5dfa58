"""The reference's own SpMV kernels on a GPU (TEST INFRASTRUCTURE ONLY).

Loads oracle/_ref/ref_kernels.cubin -- the reference's kernels compiled by
oracle/ref/build_ref.sh from its own headers, for int offsets and indices
and float values -- through the CUDA driver API (ctypes over libcuda, in the
context torch made current) and launches each kernel the way the
reference's launcher does:

  merge_path_flat  block 128, 5 items per thread, one block per merge tile
                   of 640 rows + nonzeros (algorithms/spmv/merge_path_flat.cuh:
                   112-136); the preprocess object is passed with no tile
                   coordinates, which is what the kernel receives from the
                   reference's launcher too (its copy constructor drops them,
                   schedule/merge_path_flat.hxx:214-221), so each block
                   searches its own;
  thread_mapped    block 128, one thread per row (thread_mapped.cuh:74-88);
  group_mapped     block 128, ceil(rows / 128) blocks (group_mapped.cuh:79-90);
  work_oriented    block 128, 2 x SMs blocks (work_oriented.cuh:97-108);
  original         block 128, one thread per row (original.cuh:65-72);
  spmm thread_mapped  block 128, one thread per row of C, all columns
                   (algorithms/spmm/thread_mapped.cuh:67-86).

y is zeroed first (the atomic schedules add into it).  The arrays handed to
the kernels come from pad(): copies with zeroed room after the end, because
the merge_path_flat kernel loads values[nz] and indices[nz] of each item
before it tests whether the item is a nonzero (algorithms/spmv/
merge_path_flat.cuh:70-75), so the last thread of the last tile reads one
element past both arrays (and then x at that index).  Nothing here is part of
the library; tests and oracle/ref/time_ref_gpu.py use it to compare the
library with the reference's kernels on the same inputs.
"""
import ctypes as C
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(os.path.dirname(HERE), "_ref")
CUBIN = os.path.join(REF, "ref_kernels.cubin")
LAYOUT = os.path.join(REF, "ref_kernels.json")

SCHEDULES = ("merge_path_flat", "thread_mapped", "group_mapped", "work_oriented", "original")


def available():
    return os.path.exists(CUBIN) and os.path.exists(LAYOUT)


def pad(t, extra=256):
    """A copy of the 1-D tensor t followed by `extra` zeros, viewed at t's
    length (the kernels get t's sizes; the zeros only absorb the reads past
    the end described above)."""
    import torch
    out = torch.zeros(t.numel() + extra, dtype=t.dtype, device=t.device)
    out[:t.numel()].copy_(t)
    return out[:t.numel()]


class RefKernels:
    def __init__(self):
        import torch
        if not available():
            raise FileNotFoundError("oracle/_ref/ref_kernels.cubin is not built "
                                    "(oracle/ref/build_ref.sh needs the reference sources)")
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current
        self.cu = C.CDLL("libcuda.so.1")
        self.info = json.load(open(LAYOUT))
        mod = C.c_void_p()
        self._check(self.cu.cuModuleLoad(C.byref(mod), CUBIN.encode()), "cuModuleLoad")
        self.mod = mod
        self.fn = {}
        for key, name in self.info["kernels"].items():
            f = C.c_void_p()
            self._check(self.cu.cuModuleGetFunction(C.byref(f), mod, name.encode()),
                        "cuModuleGetFunction " + key)
            self.fn[key] = f
        self.sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        self.cu.cuLaunchKernel.argtypes = [C.c_void_p] + [C.c_uint] * 7 + [
            C.c_void_p, C.POINTER(C.c_void_p), C.c_void_p]

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: CUDA driver error {rc}")

    def _setup_bytes(self, offsets_ptr, rows, nnz):
        b = bytearray.fromhex(self.info["thread_mapped_setup"])
        s = self.info["sentinels"]
        for key, val in (("offsets", offsets_ptr), ("rows", rows), ("nnz", nnz)):
            pat = bytes.fromhex(s[key])
            i = b.find(pat)
            assert i >= 0 and b.find(pat, i + 1) < 0, key
            b[i:i + 8] = int(val).to_bytes(8, "little")
        return (C.c_ubyte * len(b)).from_buffer_copy(bytes(b))

    def _matrix_bytes(self, rows, cols, ptr):
        """A dense matrix_t passed by value: the sentinels replaced, the
        vector member (neither copied nor read on the GPU) zeroed."""
        t = bytes.fromhex(self.info["matrix"])
        s = self.info["sentinels"]
        out = bytearray(len(t))
        for key, val in (("rows", rows), ("nnz", cols), ("offsets", ptr)):
            pat = bytes.fromhex(s[key])
            i = t.find(pat)
            assert i >= 0 and t.find(pat, i + 1) < 0, key
            out[i:i + 8] = int(val).to_bytes(8, "little")
        return (C.c_ubyte * len(out)).from_buffer_copy(bytes(out))

    def spmm(self, rows, cols, nnz, offsets, indices, values, B, Cm):
        """C = A B by the reference's SpMM kernel on the current stream; B is
        row-major cols x n and C row-major rows x n (contiguous float32)."""
        import torch
        s = torch.cuda.current_stream()
        n = B.shape[1]
        u64 = C.c_uint64
        args = [self._setup_bytes(offsets.data_ptr(), rows, nnz), u64(rows), u64(cols), u64(nnz),
                C.c_void_p(offsets.data_ptr()), C.c_void_p(indices.data_ptr()),
                C.c_void_p(values.data_ptr()), self._matrix_bytes(cols, n, B.data_ptr()),
                self._matrix_bytes(rows, n, Cm.data_ptr())]
        params = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        grid = max(-(-rows // 128), 1)
        self._check(self.cu.cuLaunchKernel(self.fn["spmm_thread_mapped"], grid, 1, 1, 128, 1, 1,
                                           0, C.c_void_p(s.cuda_stream), params, None),
                    "cuLaunchKernel spmm_thread_mapped")
        return Cm

    def launch(self, schedule, rows, cols, nnz, offsets, indices, values, x, y, zero=True):
        """One SpMV y = A x by the reference kernel of `schedule` on the
        current stream (torch tensors on the current device); y is zeroed
        first unless zero=False (the caller zeroed it)."""
        import torch
        s = torch.cuda.current_stream()
        if zero:
            y.zero_()
        u64 = C.c_uint64
        ptrs = [C.c_void_p(t.data_ptr()) for t in (offsets, indices, values, x, y)]
        tail = [u64(rows), u64(cols), u64(nnz)] + ptrs
        if schedule == "merge_path_flat":
            tiles = -(-(rows + nnz) // 640)
            grid, args = (max(tiles, 1), 1, 1), [(C.c_ubyte * self.info["merge_path_meta_size"])()] + tail
        elif schedule == "thread_mapped":
            grid = (max(-(-rows // 128), 1), 1, 1)
            args = [self._setup_bytes(offsets.data_ptr(), rows, nnz)] + tail
        elif schedule in ("group_mapped", "original"):
            grid, args = (max(-(-rows // 128), 1), 1, 1), tail
        elif schedule == "work_oriented":
            grid, args = (2 * self.sms, 1, 1), tail
        else:
            raise ValueError(schedule)
        params = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        self._check(self.cu.cuLaunchKernel(self.fn[schedule], grid[0], grid[1], grid[2], 128, 1, 1,
                                           0, C.c_void_p(s.cuda_stream), params, None),
                    "cuLaunchKernel " + schedule)
        return y
