// spmv_static.cu -- el_spmv_static_scratch: the merge-path SpMV (the
// default nonzero-tiled warp kernel) with its scratch in a fixed device
// array instead of a workspace, for callers that must not allocate device
// memory (see the declaration in include/edge_loops.h).
//
// The scratch is g_static_scratch: a WsHeader (range ticket, finished-warp
// counter, error flags, launch epoch) followed by EL_STATIC_MAX_RANGES
// carry slots.  It is a module-scope __device__ array, so every GPU that
// loads this library holds it (64 KiB + 64 B) until the process exits, and
// every call on a device shares it.  Host code may not use the array's name
// as a device address: every call looks the address up with
// cudaGetSymbolAddress while the device is current.
#include "el_internal.h"
#include "spmv_merge_path_nz.cuh"

namespace el {
namespace {

constexpr int kStaticRanges = EL_STATIC_MAX_RANGES;
constexpr size_t kStaticBytes = sizeof(WsHeader) + (size_t)kStaticRanges * sizeof(CarrySlot);

static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

// Device address of g_static_scratch on the current device.  Looked up on
// every call rather than cached: after a cudaDeviceReset the library's
// device image is loaded again (on the next call), possibly at another
// address, and a cached pointer would be stale.  Only the first lookup on a
// device (or the first after a reset) loads anything.
el_status static_scratch(void** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(static scratch)");
  *out = p;
  return EL_OK;
}

template <typename VT>
el_status launch_static(const el_csr& A, const float* x, float* y, int ranges, void* scratch,
                        int device, cudaStream_t stream) {
  using namespace mpn;
  const long long total = A.rows + A.nnz;  // the reference's equal split (row weight 1)
  const long long units = (total + kTileNz - 1) / kTileNz;
  long long W = ranges > 0 ? ranges : resident_warps<VT, false>(device);
  if (W > kStaticRanges) W = kStaticRanges;
  if (W > units) W = units;
  if (W < 1) W = 1;
  const long long upr = (units + W - 1) / W;
  Args a;
  a.rows = A.rows;
  a.cols = A.cols;
  a.nnz = A.nnz;
  a.offsets = A.offsets;
  a.indices = A.indices;
  a.values = A.values;
  a.row_scale = A.row_scale;
  a.x = x;
  a.y = y;
  a.range_items = upr * kTileNz;
  a.num_ranges = (units + upr - 1) / upr;
  tile_phase(A.indices, A.values, (int)sizeof(VT), &a.vec_ok, &a.ph);
  a.rw = 1;
  a.test_hooks = 0;
  a.wait_ns = 2000000000ull;
  a.ws.hdr = reinterpret_cast<WsHeader*>(scratch);
  a.ws.slots = reinterpret_cast<CarrySlot*>(reinterpret_cast<char*>(scratch) + sizeof(WsHeader));
  a.ws.nslots = kStaticRanges;
  range_trace(&a.trace, &a.trace_cap);
  const long long grid = (a.num_ranges + kWarps - 1) / kWarps;
  merge_path_nz_kernel<VT, false><<<(unsigned)grid, kTPB, 0, stream>>>(a);
  return cuda_status(cudaGetLastError(), "static-scratch merge_path launch");
}

}  // namespace
}  // namespace el

using namespace el;

extern "C" el_status el_spmv_static_scratch(const el_csr* A, const float* x, float* y,
                                            int32_t num_ranges, uint32_t* flags,
                                            el_stream_t stream) {
  if (!A) return fail(EL_ERR_NULL_POINTER, "A is NULL");
  if (A->rows < 0 || A->cols < 0 || A->nnz < 0)
    return fail(EL_ERR_INVALID_ARGUMENT, "negative size");
  if (A->rows + A->nnz >= kMergeLimit || A->cols >= (1LL << 31))
    return fail(EL_ERR_OVERFLOW, "rows+nnz = %lld: the merge path is int32 (limit 2^31 - 2^16)",
                (long long)(A->rows + A->nnz));
  if (A->value_dtype < EL_F32 || A->value_dtype > EL_F16)
    return fail(EL_ERR_INVALID_ARGUMENT, "unknown value dtype %d", A->value_dtype);
  if (num_ranges < 0 || num_ranges > EL_STATIC_MAX_RANGES)
    return fail(EL_ERR_INVALID_ARGUMENT,
                "num_ranges = %d: the static scratch holds carries for at most %d ranges",
                num_ranges, EL_STATIC_MAX_RANGES);
  if (A->rows > 0 && (!A->offsets || !y)) return fail(EL_ERR_NULL_POINTER, "offsets or y is NULL");
  if (A->nnz > 0 && (!A->indices || !A->values || !x))
    return fail(EL_ERR_NULL_POINTER, "indices, values or x is NULL");
  if (flags) *flags = 0;
  if (A->rows == 0) return EL_OK;
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  void* scratch = nullptr;
  el_status s = static_scratch(&scratch);
  if (s != EL_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  // ticket, finished counter, error flags and their info start at zero each
  // call (the epoch is kept: carries of earlier calls never match it)
  e = cudaMemsetAsync(scratch, 0, 4 * sizeof(unsigned), st);
  if (e != cudaSuccess) return cuda_status(e, "clearing the static scratch header");
  switch (A->value_dtype) {
    case EL_F32: s = launch_static<float>(*A, x, y, num_ranges, scratch, device, st); break;
    case EL_BF16: s = launch_static<__nv_bfloat16>(*A, x, y, num_ranges, scratch, device, st); break;
    default: s = launch_static<__half>(*A, x, y, num_ranges, scratch, device, st); break;
  }
  if (s != EL_OK || !flags) return s;
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_status(e, "cudaStreamSynchronize");
  unsigned h = 0;
  e = cudaMemcpy(&h, reinterpret_cast<char*>(scratch) + offsetof(WsHeader, errors), sizeof(h),
                 cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(e, "reading the static scratch flags");
  *flags = h;
  return h ? fail(EL_ERR_DEVICE, "device flags 0x%x", h) : EL_OK;
}

extern "C" el_status el_spmv_static_scratch_errors(el_stream_t stream, uint32_t* flags,
                                                   int clear) {
  if (!flags) return fail(EL_ERR_NULL_POINTER, "flags is NULL");
  void* scratch = nullptr;
  el_status s = static_scratch(&scratch);
  if (s != EL_OK) return s;
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_status(e, "cudaStreamSynchronize");
  unsigned h = 0;
  char* errs = reinterpret_cast<char*>(scratch) + offsetof(WsHeader, errors);
  e = cudaMemcpy(&h, errs, sizeof(h), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(e, "reading the static scratch flags");
  *flags = h;
  if (clear && h) {
    e = cudaMemset(errs, 0, 2 * sizeof(unsigned));
    if (e != cudaSuccess) return cuda_status(e, "clearing the static scratch flags");
  }
  return EL_OK;
}
