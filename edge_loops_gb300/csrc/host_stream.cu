// host_stream.cu -- el_spmv_host: y = A x for a CSR matrix whose arrays, x
// and y live in host memory (pinned for full link speed).  The rows are cut
// into blocks of about block_nnz nonzeros; block k's offsets, indices,
// values (and row scales) are copied into one of two device staging slots on
// the workspace's copy stream while block k-1 is multiplied on the caller's
// stream, so the transfer over the host link overlaps the SpMV and the
// device holds only two blocks, x and y at a time.
#include <algorithm>
#include <vector>

#include "el_internal.h"

namespace el {
namespace {

__global__ void rebase_kernel(int* __restrict__ off, long long n, int base) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    off[i] -= base;
}

size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace
}  // namespace el

using namespace el;

extern "C" el_status el_spmv_host(el_workspace* ws, const el_csr* A, int32_t schedule,
                                  const el_spmv_opts* opts, const float* x, float* y,
                                  int64_t block_nnz, el_stream_t stream) {
  if (!A) return fail(EL_ERR_NULL_POINTER, "A is NULL");
  if (A->rows < 0 || A->cols < 0 || A->nnz < 0)
    return fail(EL_ERR_INVALID_ARGUMENT, "negative size");
  if (A->rows + A->nnz >= kMergeLimit || A->cols >= (1LL << 31))
    return fail(EL_ERR_OVERFLOW, "rows+nnz = %lld: the merge path is int32 (limit 2^31 - 2^16)",
                (long long)(A->rows + A->nnz));
  if (A->value_dtype < EL_F32 || A->value_dtype > EL_F16)
    return fail(EL_ERR_INVALID_ARGUMENT, "unknown value dtype %d", A->value_dtype);
  if (block_nnz < 0) return fail(EL_ERR_INVALID_ARGUMENT, "block_nnz < 0");
  if (A->rows > 0 && (!A->offsets || !y)) return fail(EL_ERR_NULL_POINTER, "offsets or y is NULL");
  if (A->nnz > 0 && (!A->indices || !A->values || !x))
    return fail(EL_ERR_NULL_POINTER, "indices, values or x is NULL");
  if (A->rows == 0) return EL_OK;
  const int* off = A->offsets;  // read on the host to cut the blocks
  if (off[0] != 0 || (long long)off[A->rows] != A->nnz)
    return fail(EL_ERR_MALFORMED_CSR, "offsets[0] = %d, offsets[rows] = %d, nnz = %lld", off[0],
                off[A->rows], (long long)A->nnz);

  // blocks of whole rows, about `target` nonzeros each (at least one row);
  // by default two blocks of 2^22 .. 2^27 nonzeros: every block costs a few
  // copies, a launch and two stream hand-offs, and the host link, not the
  // SpMV, bounds the whole
  long long target = block_nnz > 0 ? block_nnz : (A->nnz + 1) / 2;
  if (block_nnz == 0) target = std::min(std::max(target, 1LL << 22), 1LL << 27);
  std::vector<long long> cut{0};
  long long max_rows = 0, max_nnz = 0;
  while (cut.back() < A->rows) {
    const long long r0 = cut.back();
    const long long goal = (long long)off[r0] + target;
    long long r = std::lower_bound(off + r0 + 1, off + A->rows + 1, goal,
                                   [](int a, long long b) { return (long long)a < b; }) -
                  off;
    if (r > A->rows) r = A->rows;
    if (r <= r0) r = r0 + 1;
    if (off[r] < off[r0] || off[r] > A->nnz)
      return fail(EL_ERR_MALFORMED_CSR, "offsets decrease between rows %lld and %lld", r0, r);
    max_rows = std::max(max_rows, r - r0);
    max_nnz = std::max(max_nnz, (long long)(off[r] - off[r0]));
    cut.push_back(r);
  }

  // staging: x | y | two slots of (offsets, indices, values, row scales)
  const size_t vb = A->value_dtype == EL_F32 ? 4 : 2;
  const bool scaled = A->row_scale != nullptr;
  const size_t x_bytes = round256((size_t)std::max<long long>(A->cols, 1) * 4);
  const size_t y_bytes = round256((size_t)A->rows * 4);
  const size_t o_bytes = round256((size_t)(max_rows + 1) * 4);
  const size_t i_bytes = round256((size_t)std::max<long long>(max_nnz, 1) * 4);
  const size_t v_bytes = round256((size_t)std::max<long long>(max_nnz, 1) * vb);
  const size_t s_bytes = scaled ? round256((size_t)max_rows * 4) : 0;
  const size_t slot_bytes = o_bytes + i_bytes + v_bytes + s_bytes;
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  cudaStream_t s0 = (cudaStream_t)stream;
  el_workspace* w = nullptr;
  el_status st = workspace_resolve(ws, s0, device, &w);
  if (st != EL_OK) return st;
  void* stage = nullptr;
  cudaStream_t cs = nullptr;
  cudaEvent_t ev[4];  // 0, 1: slot multiplied; 2, 3: slot copied
  st = workspace_stage(w, x_bytes + y_bytes + 2 * slot_bytes, &stage, &cs, ev);
  if (st != EL_OK) return st;
  char* base = static_cast<char*>(stage);
  float* dx = reinterpret_cast<float*>(base);
  float* dy = reinterpret_cast<float*>(base + x_bytes);
  char* slot[2] = {base + x_bytes + y_bytes, base + x_bytes + y_bytes + slot_bytes};

  // the copies start after earlier work on the caller's stream (which may
  // still read the staging memory)
  e = cudaEventRecord(ev[2], s0);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, ev[2], 0);
  if (e == cudaSuccess && A->nnz > 0)
    e = cudaMemcpyAsync(dx, x, (size_t)A->cols * 4, cudaMemcpyHostToDevice, cs);
  if (e != cudaSuccess) return cuda_status(e, "el_spmv_host: x");
  const char* hv = static_cast<const char*>(A->values);
  for (size_t k = 0; k + 1 < cut.size(); ++k) {
    const int sl = (int)(k & 1);
    const long long r0 = cut[k], r1 = cut[k + 1];
    const long long o0 = off[r0], o1 = off[r1];
    int* doff = reinterpret_cast<int*>(slot[sl]);
    int* didx = reinterpret_cast<int*>(slot[sl] + o_bytes);
    void* dval = slot[sl] + o_bytes + i_bytes;
    float* dsc = scaled ? reinterpret_cast<float*>(slot[sl] + o_bytes + i_bytes + v_bytes) : nullptr;
    // block k reuses the slot of block k-2: wait until that one is done
    if (k >= 2) e = cudaStreamWaitEvent(cs, ev[sl], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(doff, off + r0, (size_t)(r1 - r0 + 1) * 4, cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess && o1 > o0)
      e = cudaMemcpyAsync(didx, A->indices + o0, (size_t)(o1 - o0) * 4, cudaMemcpyHostToDevice,
                          cs);
    if (e == cudaSuccess && o1 > o0)
      e = cudaMemcpyAsync(dval, hv + (size_t)o0 * vb, (size_t)(o1 - o0) * vb,
                          cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess && scaled)
      e = cudaMemcpyAsync(dsc, A->row_scale + r0, (size_t)(r1 - r0) * 4, cudaMemcpyHostToDevice,
                          cs);
    if (e == cudaSuccess) e = cudaEventRecord(ev[2 + sl], cs);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s0, ev[2 + sl], 0);
    if (e != cudaSuccess) return cuda_status(e, "el_spmv_host: block copy");
    // offsets of the block start at 0 on the device
    const long long n_off = r1 - r0 + 1;
    rebase_kernel<<<(unsigned)std::min<long long>((n_off + 255) / 256, 1024), 256, 0, s0>>>(
        doff, n_off, (int)o0);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e, "el_spmv_host: rebase");
    el_csr B = *A;
    B.rows = r1 - r0;
    B.nnz = o1 - o0;
    B.offsets = doff;
    B.indices = didx;
    B.values = dval;
    B.row_scale = dsc;
    st = el_spmv(w, &B, schedule, opts, dx, dy + r0, (el_stream_t)s0);
    if (st != EL_OK) return st;
    e = cudaMemcpyAsync(y + r0, dy + r0, (size_t)(r1 - r0) * 4, cudaMemcpyDeviceToHost, s0);
    if (e == cudaSuccess) e = cudaEventRecord(ev[sl], s0);
    if (e != cudaSuccess) return cuda_status(e, "el_spmv_host: y");
  }
  return EL_OK;
}
