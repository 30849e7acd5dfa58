// el_internal.h -- host-side declarations shared by the translation units of
// libedgeloops.so (not installed; the public interface is edge_loops.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/edge_loops.h"
#include "el_device.cuh"

namespace el {

// Largest rows + nnz (merge-path length) accepted: int32 merge coordinates as
// in the reference's search, less 2^16 of headroom so that a coordinate plus
// a tile's extent (at most a few thousand items) never leaves int32.
constexpr long long kMergeLimit = (1LL << 31) - (1LL << 16);

// Records a failure for el_last_error_string() and returns `s`.
el_status fail(el_status s, const char* fmt, ...);
// EL_OK on cudaSuccess, else EL_ERR_CUDA with the CUDA error text.
el_status cuda_status(cudaError_t e, const char* what);

struct DeviceInfo {
  int sm_count;
  int max_smem_optin;  // bytes of dynamic shared memory a CTA may opt into
};
const DeviceInfo& device_info(int device);

// Resident CTAs per SM for a kernel at a block size and dynamic smem size
// (cached per kernel and configuration).
int resident_ctas_per_sm(const void* kernel, int threads, size_t smem);

// Everything a SpMV launcher needs; pointers already validated.
struct SpmvCall {
  el_csr A;
  const float* x;
  float* y;
  el_spmv_opts o;
  WsView ws;
  cudaStream_t stream;
  uint64_t wait_ns;
  int device;
  long long* trace = nullptr;  // el_debug_range_trace buffer (testing only)
  long long trace_cap = 0;     // ranges it holds
};

struct SpmmCall {
  el_csr A;
  const void* B;
  int b_dtype;
  int64_t n, ldb, ldc;
  float* C;
  el_spmv_opts o;
  WsView ws;
  void* scratch;        // workspace scratch (row-vector carries)
  size_t scratch_bytes;
  cudaStream_t stream;
  uint64_t wait_ns;
  int device;
};

// Per value type (VT = float, __nv_bfloat16, __half), defined in
// spmv_impl.cuh and instantiated in spmv_f32.cu / spmv_bf16.cu / spmv_f16.cu.
template <typename VT> el_status spmv_merge_path(const SpmvCall& c);
template <typename VT> long long spmv_merge_path_slots(const SpmvCall& c);
template <typename VT> el_status spmv_thread_mapped(const SpmvCall& c);
template <typename VT> el_status spmv_group_mapped(const SpmvCall& c);
template <typename VT> el_status spmv_work_oriented(const SpmvCall& c);
template <typename VT> long long spmv_work_oriented_slots(const SpmvCall& c);

// Number of carry slots a call may need (the caller sizes the workspace).
long long merge_path_slots_needed(const SpmvCall& c);
long long work_oriented_slots_needed(const SpmvCall& c);

el_status launch_merge_path(const SpmvCall& c);
el_status launch_thread_mapped(const SpmvCall& c);
el_status launch_group_mapped(const SpmvCall& c);
el_status launch_work_oriented(const SpmvCall& c);

el_status launch_spmm(const SpmmCall& c, int schedule);
size_t spmm_scratch_bytes(const SpmmCall& c, int schedule);
long long spmm_slots_needed(const SpmmCall& c, int schedule);

// The range-trace buffer that el_debug_range_trace set on this host thread
// (nullptr and 0 when none).
void range_trace(long long** buf, long long* cap);

// Workspace internals for other translation units of the library.
WsView workspace_view(el_workspace* ws);
// Sizes `ws` for an SpMV of A with `schedule` (default options).
el_status workspace_prepare(el_workspace* ws, const el_csr& A, int schedule);
// The caller's workspace or the library's one for (device, stream).
el_status workspace_resolve(el_workspace* ws, cudaStream_t stream, int device,
                            el_workspace** out);
// At least `bytes` of device staging memory in `ws` (reallocated, which
// waits for the device, when it grows), plus its copy stream and 4 events.
el_status workspace_stage(el_workspace* ws, size_t bytes, void** stage,
                          cudaStream_t* copy_stream, cudaEvent_t* events);

el_status launch_partition_tiles(const int32_t* offsets, int64_t rows,
                                 int64_t nnz, int64_t items,
                                 uint32_t* coords, cudaStream_t s);
el_status launch_partition_threads(const int32_t* offsets, int64_t rows,
                                   int64_t nnz, int tpb, int ipt,
                                   uint32_t* coords, cudaStream_t s);
el_status launch_partition_work_oriented(const int32_t* offsets, int64_t rows,
                                         int64_t nnz, int64_t num_threads,
                                         int64_t* coords, cudaStream_t s);
el_status launch_validate(const el_csr& A, unsigned* d_flags, cudaStream_t s);
el_status launch_quantize(const int32_t* offsets, int64_t rows, int64_t nnz,
                          const float* values, int dtype, void* out,
                          float* row_scale, cudaStream_t s);

}  // namespace el
