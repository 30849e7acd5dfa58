// util_kernels.cu -- partition kernels (split points exposed for bit-exact
// checks), CSR validation and value quantisation.
#include "el_internal.h"

namespace el {

// ------------------------------------------------------------- partitions
// One warp per tile boundary: the reference's generate_search_coordinates
// [include/loops/schedule/merge_path_flat.hxx:108-138] writes the start of
// every merge tile (plus the end of the last) at diagonal k * items.
__global__ void partition_tiles_kernel(const int* __restrict__ offsets,
                                       long long rows, long long nnz,
                                       long long items, long long ncoords,
                                       unsigned* __restrict__ out) {
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= ncoords) return;  // warp-uniform
  const long long diag = w * items;
  // warp_merge_search assumes diag <= rows+nnz; past the end the reference's
  // inverted search range returns {rows, nnz}
  if (diag >= rows + nnz) {
    if ((threadIdx.x & 31) == 0) {
      out[2 * w] = (unsigned)rows;
      out[2 * w + 1] = (unsigned)(diag - (diag - nnz));
    }
    return;
  }
  const long long x = warp_merge_search(offsets + 1, rows, nnz, diag);
  if ((threadIdx.x & 31) == 0) {
    out[2 * w] = (unsigned)(x < rows ? x : rows);
    out[2 * w + 1] = (unsigned)(diag - x);
  }
}

// One CTA of tpb threads per tile, exactly the reference's
// setup<merge_path_flat>::init [merge_path_flat.hxx:321-385]: threads 0/1
// search the tile's diagonals, the block gathers the tile's row-end offsets
// (item < tile rows + ipt, index clamped to rows-1), and every thread
// searches its local diagonal tid*ipt in that gathered array.
__global__ void partition_threads_kernel(const int* __restrict__ offsets,
                                         long long rows, long long nnz,
                                         int ipt, long long tiles,
                                         unsigned* __restrict__ out) {
  extern __shared__ int s_end[];  // tpb*ipt + ipt + 1
  __shared__ long long s_c[4];
  const long long t = blockIdx.x;
  const int tpb = blockDim.x;
  const long long items = (long long)tpb * ipt;
  auto row_end = [&](long long k) { return __ldg(offsets + 1 + k); };
  if (threadIdx.x < 2) {
    const long long diag = (t + threadIdx.x) * items;
    const long long f = seq_merge_search(row_end, rows, 0, nnz, diag);
    s_c[2 * threadIdx.x] = f < rows ? f : rows;
    s_c[2 * threadIdx.x + 1] = diag - f;
  }
  __syncthreads();
  const long long sx = s_c[0], sy = s_c[1];
  const long long ntiles = s_c[2] - sx, natoms = s_c[3] - sy;
  for (long long item = threadIdx.x; item < ntiles + ipt; item += tpb) {
    long long o = sx + item;
    if (o > rows - 1) o = rows - 1;
    s_end[item] = __ldg(offsets + 1 + o);
  }
  __syncthreads();
  auto tile_a = [&](long long k) { return s_end[k]; };
  const long long diag = (long long)threadIdx.x * ipt;
  const long long f = seq_merge_search(tile_a, ntiles, sy, natoms, diag);
  out[2 * (t * tpb + threadIdx.x)] = (unsigned)(f < ntiles ? f : ntiles);
  out[2 * (t * tpb + threadIdx.x) + 1] = (unsigned)(diag - f);
  (void)tiles;
}

// The reference's work_oriented even share
// [include/loops/schedule/work_oriented.hxx:141-167].
__global__ void partition_wo_kernel(const int* __restrict__ offsets,
                                    long long rows, long long nnz,
                                    long long num_threads,
                                    long long* __restrict__ out) {
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= num_threads) return;
  const long long total = rows + nnz;
  const long long wpt = (total + num_threads - 1) / num_threads;
  long long upper = wpt * tid;
  if (upper > total) upper = total;
  long long lower = upper + wpt;
  if (lower > total) lower = total;
  auto row_end = [&](long long k) { return __ldg(offsets + 1 + k); };
  const long long s = seq_merge_search(row_end, rows, 0, nnz, upper);
  const long long e = seq_merge_search(row_end, rows, 0, nnz, lower);
  out[4 * tid] = s < rows ? s : rows;
  out[4 * tid + 1] = upper - s;
  out[4 * tid + 2] = e < rows ? e : rows;
  out[4 * tid + 3] = lower - e;
}

el_status launch_partition_tiles(const int32_t* offsets, int64_t rows,
                                 int64_t nnz, int64_t items, uint32_t* coords,
                                 cudaStream_t s) {
  const long long tiles = (rows + nnz + items - 1) / items;
  const long long ncoords = tiles + 1;
  const long long threads = ncoords * 32;
  const int tpb = 256;
  const long long grid = (threads + tpb - 1) / tpb;
  partition_tiles_kernel<<<(unsigned)grid, tpb, 0, s>>>(offsets, rows, nnz, items,
                                                       ncoords, coords);
  return cuda_status(cudaGetLastError(), "partition_tiles launch");
}

el_status launch_partition_threads(const int32_t* offsets, int64_t rows,
                                   int64_t nnz, int tpb, int ipt,
                                   uint32_t* coords, cudaStream_t s) {
  const long long items = (long long)tpb * ipt;
  const long long tiles = (rows + nnz + items - 1) / items;
  if (tiles == 0) return EL_OK;
  const size_t smem = (size_t)(items + ipt + 1) * sizeof(int);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(
        partition_threads_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
        (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "partition_threads smem");
  }
  partition_threads_kernel<<<(unsigned)tiles, tpb, smem, s>>>(offsets, rows, nnz,
                                                             ipt, tiles, coords);
  return cuda_status(cudaGetLastError(), "partition_threads launch");
}

el_status launch_partition_work_oriented(const int32_t* offsets, int64_t rows,
                                         int64_t nnz, int64_t num_threads,
                                         int64_t* coords, cudaStream_t s) {
  const int tpb = 256;
  const long long grid = (num_threads + tpb - 1) / tpb;
  partition_wo_kernel<<<(unsigned)grid, tpb, 0, s>>>(
      offsets, rows, nnz, num_threads, reinterpret_cast<long long*>(coords));
  return cuda_status(cudaGetLastError(), "partition_work_oriented launch");
}

// ------------------------------------------------------------- validation
__global__ void validate_kernel(const el_csr A, unsigned* __restrict__ flags) {
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  unsigned f = 0;
  if (tid == 0) {
    if (__ldg(A.offsets) != 0 || __ldg(A.offsets + A.rows) != A.nnz)
      f |= EL_FLAG_NNZ_MISMATCH;
  }
  for (long long r = tid; r < A.rows; r += stride) {
    const int lo = __ldg(A.offsets + r), hi = __ldg(A.offsets + r + 1);
    if (lo < 0 || hi < lo || hi > A.nnz) f |= EL_FLAG_OFFSETS;
  }
  for (long long k = tid; k < A.nnz; k += stride) {
    const int c = __ldg(A.indices + k);
    if (c < 0 || c >= A.cols) f |= EL_FLAG_INDEX_RANGE;
  }
  f = __reduce_or_sync(kFullMask, f);
  if (f && (threadIdx.x & 31) == 0) atomicOr(flags, f);
}

el_status launch_validate(const el_csr& A, unsigned* d_flags, cudaStream_t s) {
  const int tpb = 256;
  long long work = A.rows > A.nnz ? A.rows : A.nnz;
  long long grid = (work + tpb - 1) / tpb;
  if (grid < 1) grid = 1;
  if (grid > 4096) grid = 4096;
  validate_kernel<<<(unsigned)grid, tpb, 0, s>>>(A, d_flags);
  return cuda_status(cudaGetLastError(), "validate launch");
}

// ----------------------------------------------------------- quantisation
// One warp per row: with scales, the row's largest magnitude m picks a power
// of two s so that m / s lands in [2^top, 2^(top+1)) and the stored value is
// round-to-nearest-even(v / s) (the division by s is exact).  BF16 has
// FP32's exponent range, so top = 0; FP16 tops out at 65504 and goes
// subnormal below 2^-14, so top = 14 keeps the most of each row normal.
template <typename OT>
__device__ __forceinline__ OT from_f32(float v);
template <>
__device__ __forceinline__ __nv_bfloat16 from_f32<__nv_bfloat16>(float v) {
  return __float2bfloat16_rn(v);
}
template <>
__device__ __forceinline__ __half from_f32<__half>(float v) {
  return __float2half_rn(v);
}

template <typename OT> struct QTop;
template <> struct QTop<__nv_bfloat16> { static constexpr int value = 0; };
template <> struct QTop<__half> { static constexpr int value = 14; };

template <typename OT>
__global__ void quantize_kernel(const int* __restrict__ offsets, long long rows,
                                const float* __restrict__ vals,
                                OT* __restrict__ out, float* __restrict__ scale) {
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long r = w; r < rows; r += nw) {
    const long long b = __ldg(offsets + r), e = __ldg(offsets + r + 1);
    int ex = 0;
    if (scale) {
      float m = 0.f;
      for (long long k = b + lane; k < e; k += 32) m = fmaxf(m, fabsf(__ldg(vals + k)));
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) m = fmaxf(m, __shfl_xor_sync(kFullMask, m, d));
      if (m > 0.f && isfinite(m)) {
        const unsigned bits = __float_as_uint(m);
        const int be = (int)((bits >> 23) & 0xff);
        ex = (be == 0 ? -126 : be - 127) - QTop<OT>::value;  // floor(log2 m) - top
      }
      if (lane == 0) scale[r] = ldexpf(1.f, ex);
    }
    for (long long k = b + lane; k < e; k += 32)
      out[k] = from_f32<OT>(ldexpf(__ldg(vals + k), -ex));
  }
}

el_status launch_quantize(const int32_t* offsets, int64_t rows, int64_t nnz,
                          const float* values, int dtype, void* out,
                          float* row_scale, cudaStream_t s) {
  (void)nnz;
  const int tpb = 256;
  long long grid = (rows * 32 + tpb - 1) / tpb;
  if (grid > 65535) grid = 65535;
  if (grid < 1) grid = 1;
  if (dtype == EL_BF16)
    quantize_kernel<__nv_bfloat16><<<(unsigned)grid, tpb, 0, s>>>(
        offsets, rows, values, reinterpret_cast<__nv_bfloat16*>(out), row_scale);
  else
    quantize_kernel<__half><<<(unsigned)grid, tpb, 0, s>>>(
        offsets, rows, values, reinterpret_cast<__half*>(out), row_scale);
  return cuda_status(cudaGetLastError(), "quantize launch");
}

}  // namespace el
