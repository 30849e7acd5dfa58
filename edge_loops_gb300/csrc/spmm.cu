// spmm.cu -- CSR SpMM C = A B for sm_103a (B, C dense row-major).
//
//  thread_mapped: the reference's algorithms/spmm/thread_mapped.cuh:28-53
//    (one thread per row, every column re-walks the row, sums in nonzero
//    order without fused multiply-add: bit-identical to the CPU loop).
//  group_mapped:  a warp per row; each nonzero's B row is read once,
//    coalesced, by the 32 lanes, each lane owning up to VEC columns.
//  merge_path:    the merge path of row ends and nonzeros split into equal
//    ranges, one per warp (ids from an atomic ticket); a warp walks its
//    range with a row-vector accumulator, and a row that crosses ranges is
//    finished by the range where it ends from the row vectors the earlier
//    ranges publish (bounded spins, fixed order, deterministic).
// At most 128 columns per pass; wider B is processed in column blocks.
#include "el_internal.h"

namespace el {
namespace spmm {

struct Args {
  long long rows, cols, nnz;
  const int* offsets;
  const int* indices;
  const void* values;
  const float* row_scale;
  const void* B;
  long long ldb;
  float* C;
  long long ldc;
  int n;  // columns in this pass
  WsHeader* hdr;
};

struct MpArgs {
  Args a;
  long long range_items;
  long long num_ranges;
  CarrySlot* flags;
  float* vec;  // num_ranges x 128 row-vector carries
  unsigned long long wait_ns;
};

template <typename T>
__device__ __forceinline__ float ld_f32(const T* p) {
  return to_f32(*p);
}
template <>
__device__ __forceinline__ float ld_f32<float>(const float* p) {
  return __ldg(p);
}

__device__ __forceinline__ bool col_ok(const Args& a, int col, long long nz) {
  if ((unsigned)col < (unsigned long long)a.cols) return true;
  raise_flag(a.hdr, EL_FLAG_INDEX_RANGE, (unsigned)nz);
  return false;
}

__device__ __forceinline__ void bounds(const Args& a, long long row, long long* b,
                                       long long* e) {
  long long lo = __ldg(a.offsets + row), hi = __ldg(a.offsets + row + 1);
  if (lo < 0 || hi > a.nnz || hi < lo) {
    raise_flag(a.hdr, EL_FLAG_OFFSETS, (unsigned)row);
    lo = lo < 0 ? 0 : (lo > a.nnz ? a.nnz : lo);
    hi = hi < lo ? lo : (hi > a.nnz ? a.nnz : hi);
  }
  *b = lo;
  *e = hi;
}

// sum += A[row, b..e) . B[.., col] in nonzero order (each product rounded,
// then added), W nonzeros' value and B loads issued together and the next
// W's index loads in flight with them; a column index outside [0, cols)
// contributes 0 and sets `bad`.
template <typename VT, typename BT, int W>
__device__ __forceinline__ float column_sum(const Args& a, const VT* vals, const BT* B,
                                            long long b, long long e, int col, bool& bad) {
  float sum = 0.f;
  if (b >= e) return sum;
  const unsigned long long cols = (unsigned long long)a.cols;
  int c[W];
#pragma unroll
  for (int k = 0; k < W; ++k) c[k] = b + k < e ? __ldg(a.indices + b + k) : -1;
  for (long long nz = b;;) {
    float bv[W], v[W];
#pragma unroll
    for (int k = 0; k < W; ++k) {
      const bool t = nz + k < e;
      const bool ok = (unsigned)c[k] < cols;
      bad |= t && !ok;
      bv[k] = t && ok ? ld_f32(B + (long long)c[k] * a.ldb + col) : 0.f;
      v[k] = t && ok ? to_f32(vals[nz + k]) : 0.f;
    }
    const long long nn = nz + W;
#pragma unroll
    for (int k = 0; k < W; ++k) c[k] = nn + k < e ? __ldg(a.indices + nn + k) : -1;
#pragma unroll
    for (int k = 0; k < W; ++k)
      if (nz + k < e) sum = __fadd_rn(sum, __fmul_rn(v[k], bv[k]));
    if (nn >= e) break;
    nz = nn;
  }
  return sum;
}

// sum[j] += A[row, b..e) . B[.., col + j] for NC adjacent columns in one walk
// of the row: each column's sum still runs in nonzero order (the same
// roundings as a walk per column), while each index and value is loaded
// once for the NC columns; W nonzeros per step, the next W indices in flight.
template <typename VT, typename BT, int W, int NC>
__device__ __forceinline__ void column_sums(const Args& a, const VT* vals, const BT* B,
                                            long long b, long long e, int col,
                                            float (&sum)[NC], bool& bad) {
#pragma unroll
  for (int j = 0; j < NC; ++j) sum[j] = 0.f;
  if (b >= e) return;
  const unsigned long long cols = (unsigned long long)a.cols;
  int c[W];
#pragma unroll
  for (int k = 0; k < W; ++k) c[k] = b + k < e ? __ldg(a.indices + b + k) : -1;
  for (long long nz = b;;) {
    float bv[W][NC], v[W];
#pragma unroll
    for (int k = 0; k < W; ++k) {
      const bool t = nz + k < e;
      const bool ok = (unsigned)c[k] < cols;
      bad |= t && !ok;
      v[k] = t && ok ? to_f32(vals[nz + k]) : 0.f;
      const BT* brow = B + (long long)(t && ok ? c[k] : 0) * a.ldb + col;
#pragma unroll
      for (int j = 0; j < NC; ++j) bv[k][j] = t && ok ? ld_f32(brow + j) : 0.f;
    }
    const long long nn = nz + W;
#pragma unroll
    for (int k = 0; k < W; ++k) c[k] = nn + k < e ? __ldg(a.indices + nn + k) : -1;
#pragma unroll
    for (int k = 0; k < W; ++k)
      if (nz + k < e) {
#pragma unroll
        for (int j = 0; j < NC; ++j) sum[j] = __fadd_rn(sum[j], __fmul_rn(v[k], bv[k][j]));
      }
    if (nn >= e) break;
    nz = nn;
  }
}

// A thread's time is its row's length times the number of columns, so the
// longest row sets the kernel's: sixteen B loads in flight per step, at
// three CTAs per SM.
template <typename VT, typename BT>
__global__ void __launch_bounds__(256, 3) thread_mapped_kernel(const Args a) {
  const VT* vals = reinterpret_cast<const VT*>(a.values);
  const BT* B = reinterpret_cast<const BT*>(a.B);
  for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < a.rows;
       row += (long long)gridDim.x * blockDim.x) {
    long long b, e;
    bounds(a, row, &b, &e);
    const float s = a.row_scale ? __ldg(a.row_scale + row) : 1.f;
    bool bad = false;
    int col = 0;
    for (; col + 4 <= a.n; col += 4) {  // four columns per walk of the row
      float sum[4];
      column_sums<VT, BT, 8, 4>(a, vals, B, b, e, col, sum, bad);
#pragma unroll
      for (int j = 0; j < 4; ++j) a.C[row * a.ldc + col + j] = a.row_scale ? sum[j] * s : sum[j];
    }
    for (; col < a.n; ++col) {
      const float sum = column_sum<VT, BT, 16>(a, vals, B, b, e, col, bad);
      a.C[row * a.ldc + col] = a.row_scale ? sum * s : sum;
    }
    if (bad) raise_flag(a.hdr, EL_FLAG_INDEX_RANGE, (unsigned)row);
  }
}

template <typename VT, typename BT, int VEC>
__device__ __forceinline__ void axpy_row(const Args& a, const BT* B, int col, float v,
                                         float (&acc)[VEC]) {
  const int lane = threadIdx.x & 31;
  const BT* brow = B + (long long)col * a.ldb;
#pragma unroll
  for (int k = 0; k < VEC; ++k) {
    const int c = lane + 32 * k;
    if (c < a.n) acc[k] = __fadd_rn(acc[k], __fmul_rn(v, ld_f32(brow + c)));
  }
}

template <int VEC>
__device__ __forceinline__ void store_row(const Args& a, long long row,
                                          const float (&acc)[VEC]) {
  const int lane = threadIdx.x & 31;
  const float s = a.row_scale ? __ldg(a.row_scale + row) : 1.f;
#pragma unroll
  for (int k = 0; k < VEC; ++k) {
    const int c = lane + 32 * k;
    if (c < a.n) a.C[row * a.ldc + c] = a.row_scale ? acc[k] * s : acc[k];
  }
}

template <typename VT, typename BT, int VEC>
__global__ void __launch_bounds__(256) group_mapped_kernel(const Args a) {
  const VT* vals = reinterpret_cast<const VT*>(a.values);
  const BT* B = reinterpret_cast<const BT*>(a.B);
  const int lane = threadIdx.x & 31;
  const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long row = w0; row < a.rows; row += nw) {  // warp-uniform
    long long b, e;
    bounds(a, row, &b, &e);
    float acc[VEC];
#pragma unroll
    for (int k = 0; k < VEC; ++k) acc[k] = 0.f;
    for (long long base = b; base < e; base += 32) {
      int mc = -1;
      float mv = 0.f;
      if (base + lane < e) {
        mc = __ldg(a.indices + base + lane);
        mv = to_f32(vals[base + lane]);
        if (!col_ok(a, mc, base + lane)) mc = -1;
      }
      const int cnt = (int)(e - base < 32 ? e - base : 32);
      // eight nonzeros at a time: their B rows are loaded together, then
      // added in nonzero order
      for (int j0 = 0; j0 < cnt; j0 += 8) {  // warp-uniform
        float bv[8][VEC], vv[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int col = __shfl_sync(kFullMask, mc, (j0 + j) & 31);
          vv[j] = __shfl_sync(kFullMask, mv, (j0 + j) & 31);
          const bool use = j0 + j < cnt && col >= 0;
          const BT* brow = B + (long long)(use ? col : 0) * a.ldb;
#pragma unroll
          for (int k = 0; k < VEC; ++k) {
            const int cc = lane + 32 * k;
            bv[j][k] = use && cc < a.n ? ld_f32(brow + cc) : 0.f;
          }
          if (!use) vv[j] = 0.f;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          if (j0 + j < cnt) {
#pragma unroll
            for (int k = 0; k < VEC; ++k) acc[k] = __fadd_rn(acc[k], __fmul_rn(vv[j], bv[j][k]));
          }
        }
      }
    }
    store_row<VEC>(a, row, acc);
  }
}

template <typename VT, typename BT, int VEC>
__global__ void __launch_bounds__(256) merge_path_kernel(const MpArgs m) {
  const Args& a = m.a;
  const VT* vals = reinterpret_cast<const VT*>(a.values);
  const BT* B = reinterpret_cast<const BT*>(a.B);
  const int lane = threadIdx.x & 31;
  unsigned wt = 0, ep = 0;
  if (lane == 0) {
    wt = atomicAdd(&a.hdr->ticket, 1u);
    ep = read_epoch(a.hdr);
  }
  const long long w = __shfl_sync(kFullMask, wt, 0);
  const unsigned epoch = __shfl_sync(kFullMask, ep, 0);
  const unsigned tag = epoch_tag(epoch);
  const long long total = a.rows + a.nnz;
  if (w < m.num_ranges) {
    long long d0 = w * m.range_items, d1 = d0 + m.range_items;
    if (d0 > total) d0 = total;
    if (d1 > total) d1 = total;
    const long long rs = warp_merge_search(a.offsets + 1, a.rows, a.nnz, d0);
    const long long ns = d0 - rs;
    const long long re = warp_merge_search(a.offsets + 1, a.rows, a.nnz, d1);
    const long long ne = d1 - re;
    const long long off_rs = __ldg(a.offsets + rs);
    const bool need_lb = ns > off_rs;
    float acc[VEC], pend[VEC];
#pragma unroll
    for (int k = 0; k < VEC; ++k) acc[k] = pend[k] = 0.f;
    bool has_pend = false;
    long long x = rs, y = ns;
    const long long kNoEnd = 1LL << 40;
    long long cur_end = x < re ? __ldg(a.offsets + x + 1) : kNoEnd;
    long long bb = y;
    int mc = -1;
    float mv = 0.f;
    auto load_batch = [&](long long at) {
      bb = at;
      mc = -1;
      mv = 0.f;
      if (at + lane < ne) {
        mc = __ldg(a.indices + at + lane);
        mv = to_f32(vals[at + lane]);
        if (!col_ok(a, mc, at + lane)) mc = -1;
      }
    };
    load_batch(y);
    for (;;) {
      while (x < re && y >= cur_end) {  // row end(s)
        if (x == rs && need_lb) {
#pragma unroll
          for (int k = 0; k < VEC; ++k) pend[k] = acc[k];
          has_pend = true;
        } else {
          store_row<VEC>(a, x, acc);
        }
#pragma unroll
        for (int k = 0; k < VEC; ++k) acc[k] = 0.f;
        ++x;
        cur_end = x < re ? __ldg(a.offsets + x + 1) : kNoEnd;
      }
      if (y >= ne) break;
      if (y - bb >= 32) load_batch(y);
      const int j = (int)(y - bb);
      const int col = __shfl_sync(kFullMask, mc, j);
      const float v = __shfl_sync(kFullMask, mv, j);
      if (col >= 0) axpy_row<VT, BT, VEC>(a, B, col, v, acc);
      ++y;
    }
    if (x < re) raise_flag(a.hdr, EL_FLAG_OFFSETS, (unsigned)x);  // malformed
    // publish the open row's partial vector if this range holds any of it
    if (re < a.rows) {
      const long long off_re = __ldg(a.offsets + re);
      const long long lo = off_re > ns ? off_re : ns;
      if (ne > lo && w < m.num_ranges) {
        float* dst = m.vec + w * 128;
#pragma unroll
        for (int k = 0; k < VEC; ++k) {
          const int c = lane + 32 * k;
          if (c < a.n) __stcg(dst + c, acc[k]);
        }
        __threadfence();
        __syncwarp();
        if (lane == 0) st_release_u32(&m.flags[w].flag, tag);
      }
    }
    if (has_pend) {
      const long long wfirst = (rs + off_rs) / m.range_items;
      float chain[VEC];
#pragma unroll
      for (int k = 0; k < VEC; ++k) chain[k] = 0.f;
      bool ok = true;
      for (long long k2 = wfirst; k2 < w && ok; ++k2) {
        unsigned f = ld_acquire_u32(&m.flags[k2].flag);
        if (f != tag) {
          const uint64_t t0 = global_timer_ns();
          while ((f = ld_acquire_u32(&m.flags[k2].flag)) != tag) {
            if (global_timer_ns() - t0 > m.wait_ns) break;
            __nanosleep(100);
          }
        }
        ok = __all_sync(kFullMask, f == tag);
        if (!ok) break;
        const float* src = m.vec + k2 * 128;
#pragma unroll
        for (int k = 0; k < VEC; ++k) {
          const int c = lane + 32 * k;
          if (c < a.n) chain[k] = __fadd_rn(chain[k], __ldcg(src + c));
        }
        __syncwarp();
      }
      if (!ok && lane == 0) raise_flag(a.hdr, EL_FLAG_TIMEOUT, 6);
#pragma unroll
      for (int k = 0; k < VEC; ++k) chain[k] = __fadd_rn(chain[k], pend[k]);
      store_row<VEC>(a, rs, chain);
    }
  }
  // the last warp to finish resets the ticket for the next launch
  if (lane == 0) {
    __threadfence();
    const unsigned total_warps = gridDim.x * (blockDim.x >> 5);
    const unsigned prev = atomicAdd(&a.hdr->done, 1u);
    if (prev == total_warps - 1) finish_launch(a.hdr, epoch);
  }
}

template <typename VT, typename BT>
el_status launch_typed(const SpmmCall& c, int schedule) {
  Args a;
  a.rows = c.A.rows;
  a.cols = c.A.cols;
  a.nnz = c.A.nnz;
  a.offsets = c.A.offsets;
  a.indices = c.A.indices;
  a.values = c.A.values;
  a.row_scale = c.A.row_scale;
  a.ldb = c.ldb;
  a.ldc = c.ldc;
  a.hdr = c.ws.hdr;
  const int sms = device_info(c.device).sm_count;
  for (long long cb = 0; cb < c.n; cb += 128) {
    a.n = (int)(c.n - cb < 128 ? c.n - cb : 128);
    a.B = reinterpret_cast<const BT*>(c.B) + cb;
    a.C = c.C + cb;
    if (schedule == EL_SCHED_THREAD_MAPPED) {
      long long grid = (a.rows + 255) / 256;
      if (grid > (long long)sms * 32) grid = (long long)sms * 32;
      thread_mapped_kernel<VT, BT><<<(unsigned)grid, 256, 0, c.stream>>>(a);
    } else if (schedule == EL_SCHED_GROUP_MAPPED) {
      long long grid = (a.rows * 32 + 255) / 256;
      if (grid > (long long)sms * 32) grid = (long long)sms * 32;
      if (a.n <= 32)
        group_mapped_kernel<VT, BT, 1><<<(unsigned)grid, 256, 0, c.stream>>>(a);
      else
        group_mapped_kernel<VT, BT, 4><<<(unsigned)grid, 256, 0, c.stream>>>(a);
    } else {
      MpArgs m;
      m.a = a;
      const int per_sm = resident_ctas_per_sm(
          a.n <= 32 ? (const void*)merge_path_kernel<VT, BT, 1>
                    : (const void*)merge_path_kernel<VT, BT, 4>,
          256, 0);
      long long warps = (long long)(per_sm > 0 ? per_sm : 1) * sms * 8;
      const long long total = a.rows + a.nnz;
      long long ri = (total + warps - 1) / warps;
      if (ri < 64) ri = 64;
      m.range_items = ri;
      m.num_ranges = (total + ri - 1) / ri;
      if (m.num_ranges > c.ws.nslots ||
          (size_t)m.num_ranges * 128 * sizeof(float) > c.scratch_bytes)
        return fail(EL_ERR_INVALID_ARGUMENT, "spmm merge_path: workspace too small");
      m.flags = c.ws.slots;
      m.vec = reinterpret_cast<float*>(c.scratch);
      m.wait_ns = c.wait_ns;
      const long long grid = (m.num_ranges + 7) / 8;
      if (a.n <= 32)
        merge_path_kernel<VT, BT, 1><<<(unsigned)grid, 256, 0, c.stream>>>(m);
      else
        merge_path_kernel<VT, BT, 4><<<(unsigned)grid, 256, 0, c.stream>>>(m);
    }
    el_status s = cuda_status(cudaGetLastError(), "spmm launch");
    if (s != EL_OK) return s;
  }
  return EL_OK;
}

}  // namespace spmm

// Ranges the merge-path SpMM may use: one per resident warp of the kernel
// (of either column width) that fits most CTAs on an SM.
static long long spmm_mp_ranges(const SpmmCall& c) {
  int per_sm = 1;
  const void* kerns[] = {(const void*)spmm::merge_path_kernel<float, float, 4>,
                         (const void*)spmm::merge_path_kernel<float, float, 1>,
                         (const void*)spmm::merge_path_kernel<float, __nv_bfloat16, 4>,
                         (const void*)spmm::merge_path_kernel<float, __nv_bfloat16, 1>,
                         (const void*)spmm::merge_path_kernel<__nv_bfloat16, float, 1>,
                         (const void*)spmm::merge_path_kernel<__half, __half, 1>};
  for (const void* k : kerns) {
    const int p = resident_ctas_per_sm(k, 256, 0);
    if (p > per_sm) per_sm = p;
  }
  return (long long)per_sm * device_info(c.device).sm_count * 8;
}

size_t spmm_scratch_bytes(const SpmmCall& c, int schedule) {
  if (schedule != EL_SCHED_MERGE_PATH_FLAT) return 0;
  return (size_t)spmm_mp_ranges(c) * 128 * sizeof(float);
}

long long spmm_slots_needed(const SpmmCall& c, int schedule) {
  return schedule == EL_SCHED_MERGE_PATH_FLAT ? spmm_mp_ranges(c) : 0;
}

el_status launch_spmm(const SpmmCall& c, int schedule) {
  const int vt = c.A.value_dtype, bt = c.b_dtype;
  if (vt == EL_F32 && bt == EL_F32) return spmm::launch_typed<float, float>(c, schedule);
  if (vt == EL_F32 && bt == EL_BF16) return spmm::launch_typed<float, __nv_bfloat16>(c, schedule);
  if (vt == EL_BF16 && bt == EL_BF16)
    return spmm::launch_typed<__nv_bfloat16, __nv_bfloat16>(c, schedule);
  if (vt == EL_BF16 && bt == EL_F32) return spmm::launch_typed<__nv_bfloat16, float>(c, schedule);
  if (vt == EL_F16 && bt == EL_F16) return spmm::launch_typed<__half, __half>(c, schedule);
  if (vt == EL_F16 && bt == EL_F32) return spmm::launch_typed<__half, float>(c, schedule);
  if (vt == EL_F32 && bt == EL_F16) return spmm::launch_typed<float, __half>(c, schedule);
  return fail(EL_ERR_UNSUPPORTED, "SpMM value/B dtype pair (%d, %d) not built", vt, bt);
}

}  // namespace el
