// csr_build.cu -- el_csr_from_coo: COO (device) -> CSR (device), the
// reference's CSR construction [include/loops/container/csr.hxx:86-94]:
// sort the entries by (row, column) [coo.hxx:104-113, :145-148], take the
// column indices and values in that order, and offsets[r] = the first
// sorted position whose row is >= r [detail/convert.hxx:75-77].
//
// The sort is a stable LSD radix sort of the 62-bit key row << 31 | column
// (cub::DeviceRadixSort over only the bits the sizes need), so entries with
// equal (row, column) keep their input order -- the reference's thrust sort
// leaves their order unspecified and keeps them all, and so does this.  The
// offsets are found by one binary search per row.  Entries whose row or
// column is outside the matrix are an error (EL_ERR_MALFORMED_CSR), checked
// before anything is written.
#include <cub/device/device_radix_sort.cuh>

#include "el_internal.h"

namespace el {
namespace {

__global__ void keys_kernel(const int32_t* __restrict__ ri, const int32_t* __restrict__ ci,
                            long long nnz, long long rows, long long cols,
                            unsigned long long* __restrict__ keys, int32_t* __restrict__ pos,
                            unsigned* __restrict__ bad) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (long long)gridDim.x * blockDim.x) {
    const int r = ri[k], c = ci[k];
    if ((unsigned long long)(unsigned)r >= (unsigned long long)rows ||
        (unsigned long long)(unsigned)c >= (unsigned long long)cols)
      atomicOr(bad, 1u);
    keys[k] = ((unsigned long long)(unsigned)r << 31) | (unsigned)c;
    pos[k] = (int32_t)k;
  }
}

__global__ void gather_kernel(const unsigned long long* __restrict__ keys,
                              const int32_t* __restrict__ pos, const float* __restrict__ vin,
                              long long nnz, int32_t* __restrict__ indices,
                              float* __restrict__ values) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (long long)gridDim.x * blockDim.x) {
    indices[k] = (int32_t)(keys[k] & 0x7fffffffull);
    values[k] = vin[pos[k]];
  }
}

// offsets[r] = number of sorted entries with row < r
__global__ void offsets_kernel(const unsigned long long* __restrict__ keys, long long nnz,
                               long long rows, int32_t* __restrict__ offsets) {
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r <= rows;
       r += (long long)gridDim.x * blockDim.x) {
    const unsigned long long key = (unsigned long long)r << 31;
    long long lo = 0, hi = nnz;
    while (lo < hi) {
      const long long mid = (lo + hi) >> 1;
      if (keys[mid] < key) lo = mid + 1; else hi = mid;
    }
    offsets[r] = (int32_t)lo;
  }
}

int bits_for(long long n) {  // bits to hold values 0 .. n-1
  int b = 1;
  while (b < 62 && (1LL << b) < n) ++b;
  return b;
}

size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace
}  // namespace el

using namespace el;

extern "C" el_status el_csr_from_coo(el_workspace* ws, const el_coo* coo, int32_t* offsets,
                                     int32_t* indices, float* values, el_stream_t stream) {
  if (!coo) return fail(EL_ERR_NULL_POINTER, "coo is NULL");
  if (coo->rows < 0 || coo->cols < 0 || coo->nnz < 0)
    return fail(EL_ERR_INVALID_ARGUMENT, "negative size");
  if (coo->rows >= (1LL << 31) - 1 || coo->cols >= (1LL << 31) || coo->nnz >= (1LL << 31))
    return fail(EL_ERR_OVERFLOW, "sizes exceed int32");
  if (!offsets) return fail(EL_ERR_NULL_POINTER, "offsets is NULL");
  if (coo->nnz > 0 && (!coo->row_indices || !coo->col_indices || !coo->values || !indices ||
                       !values))
    return fail(EL_ERR_NULL_POINTER, "an array is NULL");
  cudaStream_t s = (cudaStream_t)stream;
  const long long nnz = coo->nnz;
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  const int sms = device_info(device).sm_count;
  if (nnz == 0) {
    e = cudaMemsetAsync(offsets, 0, (size_t)(coo->rows + 1) * sizeof(int32_t), s);
    return cuda_status(e, "el_csr_from_coo: offsets");
  }
  // temporaries in the workspace's staging memory:
  // keys in/out, positions in/out, the bad flag, CUB's temporary storage
  const int end_bit = 31 + bits_for(coo->rows > 0 ? coo->rows : 1);
  size_t cub_bytes = 0;
  cub::DoubleBuffer<unsigned long long> kb(nullptr, nullptr);
  cub::DoubleBuffer<int32_t> pb(nullptr, nullptr);
  e = cub::DeviceRadixSort::SortPairs(nullptr, cub_bytes, kb, pb, (int)nnz, 0, end_bit, s);
  if (e != cudaSuccess) return cuda_status(e, "el_csr_from_coo: sort size");
  const size_t kbytes = round256((size_t)nnz * 8), pbytes = round256((size_t)nnz * 4);
  const size_t total = 2 * kbytes + 2 * pbytes + 256 + round256(cub_bytes);
  el_workspace* w = nullptr;
  el_status st = workspace_resolve(ws, s, device, &w);
  if (st != EL_OK) return st;
  void* stage = nullptr;
  cudaStream_t cs = nullptr;
  cudaEvent_t ev[4];
  st = workspace_stage(w, total, &stage, &cs, ev);
  if (st != EL_OK) return st;
  char* p = static_cast<char*>(stage);
  unsigned long long* k0 = reinterpret_cast<unsigned long long*>(p);
  unsigned long long* k1 = reinterpret_cast<unsigned long long*>(p + kbytes);
  int32_t* p0 = reinterpret_cast<int32_t*>(p + 2 * kbytes);
  int32_t* p1 = reinterpret_cast<int32_t*>(p + 2 * kbytes + pbytes);
  unsigned* bad = reinterpret_cast<unsigned*>(p + 2 * kbytes + 2 * pbytes);
  void* tmp = p + 2 * kbytes + 2 * pbytes + 256;

  const unsigned grid = (unsigned)std::min<long long>((nnz + 255) / 256, (long long)sms * 8);
  e = cudaMemsetAsync(bad, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return cuda_status(e, "el_csr_from_coo");
  keys_kernel<<<grid, 256, 0, s>>>(coo->row_indices, coo->col_indices, nnz, coo->rows, coo->cols,
                                   k0, p0, bad);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e, "el_csr_from_coo: keys");
  unsigned h_bad = 0;
  e = cudaMemcpyAsync(&h_bad, bad, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(e, "el_csr_from_coo: check");
  if (h_bad) return fail(EL_ERR_MALFORMED_CSR, "COO entry outside %lld x %lld",
                         (long long)coo->rows, (long long)coo->cols);
  cub::DoubleBuffer<unsigned long long> keys(k0, k1);
  cub::DoubleBuffer<int32_t> pos(p0, p1);
  size_t tb = round256(cub_bytes);
  e = cub::DeviceRadixSort::SortPairs(tmp, tb, keys, pos, (int)nnz, 0, end_bit, s);
  if (e != cudaSuccess) return cuda_status(e, "el_csr_from_coo: sort");
  gather_kernel<<<grid, 256, 0, s>>>(keys.Current(), pos.Current(), coo->values, nnz, indices,
                                     values);
  const unsigned ogrid =
      (unsigned)std::min<long long>((coo->rows + 1 + 255) / 256, (long long)sms * 8);
  offsets_kernel<<<ogrid, 256, 0, s>>>(keys.Current(), nnz, coo->rows, offsets);
  return cuda_status(cudaGetLastError(), "el_csr_from_coo: gather");
}
