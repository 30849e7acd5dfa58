// batched.cu -- batched SpMV: many independent CSR matrices in one
// persistent launch captured in a CUDA graph (el_batch_plan_*).
//
// Plan creation: one statistics kernel reads every matrix's row offsets
// (rows, nonzeros, max row length, sum of squared lengths); the host maps
// each matrix to a (kernel mode, work-item size) pair -- from the tuning
// table bucket of (rows, mean row length, coefficient of variation) or the
// built-in rule -- and a split kernel cuts every matrix into work items of
// whole rows at merge-path diagonals k * 2^chunk (so every item holds about
// 2^chunk rows + nonzeros).  Execution: a persistent grid whose warps stride
// over the work list; a warp runs its item either with the nonzero-tiled
// walk of the merge-path kernel (tiles of 256 nonzeros, 8 per lane, row
// ends from the offsets window) or with TPR lanes per row (the
// thread_mapped schedule generalised to TPR lanes with a fixed xor-tree
// reduction).  Items hold whole rows, so no partial sums cross warps; no
// atomics: deterministic.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "el_internal.h"
#include "spmv_merge_path_nz.cuh"

namespace el {
namespace batch {

struct Desc {  // one matrix, device side
  const int* offsets;
  const int* indices;
  const void* values;
  const float* row_scale;
  const float* x;
  float* y;
  int rows;
  int cols;
  int nnz;
  int ph;  // tile phase of the nonzero-tiled walk, -1: no 128-bit loads
};

struct Item {  // rows [r0, r1) of matrix m, run in `mode`
  int m;
  int r0;
  int r1;
  int mode;  // 0..5: 1 << mode lanes per row; kNzWalk: nonzero-tiled walk
};

constexpr int kNzWalk = 6;

struct Stats {
  double sum_sq;
  int max_len;
  int bad;  // offsets outside [0, nnz] or decreasing
};

__global__ void stats_kernel(const Desc* __restrict__ d, Stats* __restrict__ out) {
  const Desc m = d[blockIdx.x];
  if (m.rows == 0) {  // offsets may be NULL: nothing to read
    if (threadIdx.x == 0) out[blockIdx.x] = Stats{0.0, 0, m.nnz != 0};
    return;
  }
  double sq = 0.0;
  int mx = 0, bad = 0;
  for (int r = threadIdx.x; r < m.rows; r += blockDim.x) {
    const int lo = __ldg(m.offsets + r), hi = __ldg(m.offsets + r + 1);
    const int len = hi - lo;
    if (lo < 0 || hi > m.nnz || len < 0) bad = 1;
    const double l = len > 0 ? (double)len : 0.0;
    sq += l * l;
    mx = max(mx, len);
  }
  __shared__ double s_sq[8];
  __shared__ int s_mx[8], s_bad[8];
  for (int o = 16; o > 0; o >>= 1) {
    sq += __shfl_xor_sync(kFullMask, sq, o);
    mx = max(mx, __shfl_xor_sync(kFullMask, mx, o));
    bad |= __shfl_xor_sync(kFullMask, bad, o);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    s_sq[w] = sq;
    s_mx[w] = mx;
    s_bad[w] = bad;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) {
      sq += s_sq[i];
      mx = max(mx, s_mx[i]);
      bad |= s_bad[i];
    }
    if (__ldg(m.offsets) != 0 || __ldg(m.offsets + m.rows) != m.nnz) bad = 1;
    out[blockIdx.x] = Stats{sq, mx, bad};
  }
}

template <typename VT, int TPR>
__device__ __forceinline__ void rows_tpr(const Desc& d, int r0, int r1, int lane, WsHeader* hdr) {
  const int sub = lane % TPR;
  constexpr int RPW = 32 / TPR;
  const VT* vals = reinterpret_cast<const VT*>(d.values);
  for (int base = r0; base < r1; base += RPW) {  // warp-uniform
    const int row = base + lane / TPR;
    float acc = 0.f;
    if (row < r1) {
      int b = __ldg(d.offsets + row), e = __ldg(d.offsets + row + 1);
      if (b < 0 || e > d.nnz || e < b) {
        raise_flag(hdr, EL_FLAG_OFFSETS, (unsigned)row);
        b = min(max(b, 0), d.nnz);
        e = min(max(e, b), d.nnz);
      }
      // four nonzeros' index, value and x loads issued together, added in
      // nonzero order; a bad column adds 0 and raises the flag once
      bool bad = false;
      int nz = b + sub;
      for (; nz + 3 * TPR < e; nz += 4 * TPR) {
        int c[4];
        float v[4], xv[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          c[k] = __ldg(d.indices + nz + k * TPR);
          v[k] = to_f32(vals[nz + k * TPR]);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const bool ok = (unsigned)c[k] < (unsigned)d.cols;
          bad |= !ok;
          xv[k] = ok ? __ldg(d.x + c[k]) : 0.f;
          if (!ok) v[k] = 0.f;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) acc = __fadd_rn(acc, __fmul_rn(v[k], xv[k]));
      }
      for (; nz < e; nz += TPR) {
        const int col = __ldg(d.indices + nz);
        const bool ok = (unsigned)col < (unsigned)d.cols;
        bad |= !ok;
        acc = __fadd_rn(acc, ok ? __fmul_rn(to_f32(vals[nz]), __ldg(d.x + col)) : 0.f);
      }
      if (bad) raise_flag(hdr, EL_FLAG_INDEX_RANGE, (unsigned)row);
    }
#pragma unroll
    for (int o = TPR / 2; o > 0; o >>= 1) acc = __fadd_rn(acc, __shfl_xor_sync(kFullMask, acc, o));
    if (sub == 0 && row < r1) d.y[row] = d.row_scale ? acc * __ldg(d.row_scale + row) : acc;
  }
}

// Rows [r0, r1) by the nonzero-tiled walk (whole rows: nothing is carried
// out of the item).  Offsets are clamped, so any content stays in bounds.
template <typename VT>
__device__ __forceinline__ void rows_nz(const Desc& d, int r0, int r1, int lane,
                                        mpn::WarpSmem<false>& S, bool& bad, bool& bad_col) {
  const int ns = min(max(__ldg(d.offsets + r0), 0), d.nnz);
  const int ne = min(max(__ldg(d.offsets + r1), ns), d.nnz);
  const mpn::Src m{d.offsets, d.indices,        d.values, d.row_scale,       d.x,
                   d.y,       d.rows,           (unsigned)d.cols, d.nnz, d.ph >= 0 ? 1 : 0,
                   d.ph >= 0 ? d.ph : 0};
  int ra = r0;
  (void)mpn::walk_rows<VT, false>(m, S, lane, r0, r1, ns, ne, false, bad, bad_col, ra);
}

template <typename VT>
__global__ void __launch_bounds__(256, mpn::kPer == 16 ? 2 : 3)
    batched_spmv_kernel(const Desc* __restrict__ descs, const Item* __restrict__ items,
                        long long n_items, WsHeader* hdr) {
  __shared__ mpn::WarpSmem<false> smem[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  bool bad = false, bad_col = false;
  const long long stride = (long long)gridDim.x * 8;
  for (long long it = (long long)blockIdx.x * 8 + warp; it < n_items; it += stride) {  // warp-uniform
    const Item w = items[it];
    const Desc d = descs[w.m];
    switch (w.mode) {
      case 0: rows_tpr<VT, 1>(d, w.r0, w.r1, lane, hdr); break;
      case 1: rows_tpr<VT, 2>(d, w.r0, w.r1, lane, hdr); break;
      case 2: rows_tpr<VT, 4>(d, w.r0, w.r1, lane, hdr); break;
      case 3: rows_tpr<VT, 8>(d, w.r0, w.r1, lane, hdr); break;
      case 4: rows_tpr<VT, 16>(d, w.r0, w.r1, lane, hdr); break;
      case 5: rows_tpr<VT, 32>(d, w.r0, w.r1, lane, hdr); break;
      default: rows_nz<VT>(d, w.r0, w.r1, lane, smem[warp], bad, bad_col); break;
    }
  }
  if (__any_sync(kFullMask, bad_col) && lane == 0) raise_flag(hdr, EL_FLAG_INDEX_RANGE, 0);
  if (__any_sync(kFullMask, bad) && lane == 0) raise_flag(hdr, EL_FLAG_OFFSETS, 0);
}

// Work items: item i arrives as {m, k, chunk_log2, mode} and leaves as
// {m, r0, r1, mode} with rows [r0, r1) = the rows whose end falls in merge
// diagonals [k << chunk, (k + 1) << chunk) of matrix m.
__global__ void split_kernel(const Desc* __restrict__ descs, Item* __restrict__ items,
                             long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Item w = items[i];
  const Desc d = descs[w.m];
  const long long total = (long long)d.rows + d.nnz;
  const long long d0 = (long long)w.r0 << w.r1;
  long long d1 = d0 + (1LL << w.r1);
  if (d1 > total) d1 = total;
  const int* row_end = d.offsets + 1;
  auto a = [&](long long k) { return __ldg(row_end + k); };
  const long long x0 = seq_merge_search(a, d.rows, 0, d.nnz, d0 < total ? d0 : total);
  const long long x1 = d1 >= total ? d.rows : seq_merge_search(a, d.rows, 0, d.nnz, d1);
  w.r0 = (int)min(x0, (long long)d.rows);
  w.r1 = (int)min(max(x1, x0), (long long)d.rows);
  items[i] = w;
}

int row_bucket(long long rows) {
  int b = 0;
  while (b < EL_BATCH_ROW_BUCKETS - 1 && (2LL << b) <= rows) ++b;
  return b;
}
int len_bucket(double avg) {
  if (avg < 1.0) return 0;
  int b = 1;
  while (b < EL_BATCH_LEN_BUCKETS - 1 && avg >= (double)(1LL << b)) ++b;
  return b;
}
int cv_bucket(double cv) { return cv < 0.25 ? 0 : cv < 0.75 ? 1 : cv < 1.5 ? 2 : 3; }

// Kernel mode of a threads-per-row value: 1..32 lanes per row (rounded up
// to a power of two), EL_BATCH_NZ_WALK: the nonzero-tiled walk.
int mode_of(int tpr) {
  if (tpr >= EL_BATCH_NZ_WALK) return kNzWalk;
  int l2 = 0;
  while ((1 << l2) < tpr && l2 < 5) ++l2;
  return l2;
}

// Built-in rule (used where the table has no entry): the nonzero-tiled
// walk with work items of 2^12 rows + nonzeros.
void builtin_rule(double, double, int* mode, int* chunk_log2) {
  *mode = kNzWalk;
  *chunk_log2 = 12;
}

}  // namespace batch

}  // namespace el

struct el_batch_plan {
  int device;
  int dtype;
  void* d_descs;
  void* d_items;
  long long n_items;
  int grid;
  int tpr_counts[7];
  std::vector<int> heavy;  // matrices run as separate merge-path launches
  std::vector<el_batch_item> items;
  el_workspace* ws;
  cudaGraph_t graph;
  cudaGraphExec_t exec;
  bool use_graph;
};

using namespace el;

static el_status enqueue_plan(el_batch_plan* p, cudaStream_t s, void* hdr) {
  if (p->n_items > 0) {
    const batch::Desc* d = reinterpret_cast<const batch::Desc*>(p->d_descs);
    const batch::Item* it = reinterpret_cast<const batch::Item*>(p->d_items);
    WsHeader* h = reinterpret_cast<WsHeader*>(hdr);
    switch (p->dtype) {
      case EL_F32:
        batch::batched_spmv_kernel<float><<<p->grid, 256, 0, s>>>(d, it, p->n_items, h);
        break;
      case EL_BF16:
        batch::batched_spmv_kernel<__nv_bfloat16><<<p->grid, 256, 0, s>>>(d, it, p->n_items, h);
        break;
      default:
        batch::batched_spmv_kernel<__half><<<p->grid, 256, 0, s>>>(d, it, p->n_items, h);
        break;
    }
    el_status st = cuda_status(cudaGetLastError(), "batched launch");
    if (st != EL_OK) return st;
  }
  for (int m : p->heavy) {
    const el_batch_item& b = p->items[m];
    el_status st = el_spmv(p->ws, &b.A, EL_SCHED_MERGE_PATH_FLAT, nullptr, b.x, b.y,
                           (el_stream_t)s);
    if (st != EL_OK) return st;
  }
  return EL_OK;
}

// The plan's own workspace header (for the error flags of its kernels).
static void* plan_hdr(el_batch_plan* p) { return workspace_view(p->ws).hdr; }

extern "C" {

void el_batch_opts_default(el_batch_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->use_graph = 1;
}

el_status el_batch_plan_create(const el_batch_item* items, int32_t count,
                               const el_batch_opts* opts, el_stream_t stream,
                               el_batch_plan** out) {
  if (!out) return fail(EL_ERR_NULL_POINTER, "out is NULL");
  *out = nullptr;
  if (count < 0) return fail(EL_ERR_INVALID_ARGUMENT, "count < 0");
  if (count > 0 && !items) return fail(EL_ERR_NULL_POINTER, "items is NULL");
  el_batch_opts o;
  el_batch_opts_default(&o);
  if (opts) o = *opts;
  if (o.force_threads_per_row < 0 ||
      (o.force_threads_per_row > 32 && o.force_threads_per_row != EL_BATCH_NZ_WALK) ||
      (o.force_threads_per_row & (o.force_threads_per_row - 1)) != 0)
    return fail(EL_ERR_INVALID_ARGUMENT,
                "force_threads_per_row must be a power of two <= 32 or EL_BATCH_NZ_WALK");
  int dtype = count > 0 ? items[0].A.value_dtype : EL_F32;
  for (int i = 0; i < count; ++i) {
    const el_csr& A = items[i].A;
    if (A.rows < 0 || A.cols < 0 || A.nnz < 0)
      return fail(EL_ERR_INVALID_ARGUMENT, "matrix %d: negative size", i);
    if (A.rows + A.nnz >= kMergeLimit || A.cols >= (1LL << 31))
      return fail(EL_ERR_OVERFLOW, "matrix %d: rows+nnz >= 2^31 - 2^16", i);
    if (A.value_dtype != dtype)
      return fail(EL_ERR_UNSUPPORTED, "matrix %d: all matrices of a plan share one dtype", i);
    if (A.value_dtype < EL_F32 || A.value_dtype > EL_F16)
      return fail(EL_ERR_INVALID_ARGUMENT, "matrix %d: unknown dtype", i);
    if (A.rows > 0 && (!A.offsets || !items[i].y))
      return fail(EL_ERR_NULL_POINTER, "matrix %d: offsets or y is NULL", i);
    if (A.nnz > 0 && (!A.indices || !A.values || !items[i].x))
      return fail(EL_ERR_NULL_POINTER, "matrix %d: indices, values or x is NULL", i);
  }
  el_batch_plan* p = new el_batch_plan();
  p->dtype = dtype;
  p->d_descs = p->d_items = nullptr;
  p->n_items = 0;
  p->grid = 1;
  std::memset(p->tpr_counts, 0, sizeof(p->tpr_counts));
  p->items.assign(items, items + count);
  p->ws = nullptr;
  p->graph = nullptr;
  p->exec = nullptr;
  p->use_graph = o.use_graph != 0;
  cudaStream_t s = (cudaStream_t)stream;
  auto bail = [&](el_status st) {
    el_batch_plan_destroy(p);
    return st;
  };
  cudaError_t e = cudaGetDevice(&p->device);
  if (e != cudaSuccess) return bail(cuda_status(e, "cudaGetDevice"));
  el_status st = el_workspace_create(p->device, &p->ws);
  if (st != EL_OK) return bail(st);

  // descriptors and statistics
  std::vector<batch::Desc> descs(count);
  for (int i = 0; i < count; ++i) {
    const el_batch_item& b = items[i];
    int vec_ok = 0, ph = 0;
    mpn::tile_phase(b.A.indices, b.A.values, b.A.value_dtype == EL_F32 ? 4 : 2, &vec_ok, &ph);
    descs[i] = batch::Desc{b.A.offsets, b.A.indices, b.A.values, b.A.row_scale, b.x, b.y,
                           (int)b.A.rows, (int)b.A.cols, (int)b.A.nnz, vec_ok ? ph : -1};
  }
  std::vector<batch::Stats> stats(count);
  if (count > 0) {
    e = cudaMalloc(&p->d_descs, sizeof(batch::Desc) * count);
    if (e != cudaSuccess) return bail(cuda_status(e, "batch descriptors"));
    e = cudaMemcpyAsync(p->d_descs, descs.data(), sizeof(batch::Desc) * count,
                        cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return bail(cuda_status(e, "batch descriptors upload"));
    batch::Stats* d_stats = nullptr;
    e = cudaMalloc(&d_stats, sizeof(batch::Stats) * count);
    if (e != cudaSuccess) return bail(cuda_status(e, "batch statistics"));
    batch::stats_kernel<<<count, 256, 0, s>>>(
        reinterpret_cast<const batch::Desc*>(p->d_descs), d_stats);
    e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(stats.data(), d_stats, sizeof(batch::Stats) * count,
                          cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d_stats);
    if (e != cudaSuccess) return bail(cuda_status(e, "batch statistics"));
  }

  // per-matrix configuration and the work list
  std::vector<batch::Item> work;
  for (int i = 0; i < count; ++i) {
    const el_csr& A = items[i].A;
    if (A.rows == 0) continue;
    if (stats[i].bad)
      return bail(fail(EL_ERR_MALFORMED_CSR, "matrix %d: malformed offsets", i));
    if (stats[i].max_len > EL_BATCH_MAX_ROW_NNZ) {
      p->heavy.push_back(i);
      continue;
    }
    const double rows = (double)A.rows;
    const double avg = (double)A.nnz / rows;
    const double var = std::max(0.0, stats[i].sum_sq / rows - avg * avg);
    const double cv = avg > 0 ? std::sqrt(var) / avg : 0.0;
    int mode = batch::kNzWalk, cl = 12;
    batch::builtin_rule(avg, cv, &mode, &cl);
    if (o.table) {
      const int idx = (batch::row_bucket(A.rows) * EL_BATCH_LEN_BUCKETS + batch::len_bucket(avg)) *
                          EL_BATCH_CV_BUCKETS + batch::cv_bucket(cv);
      const int ent = o.table[idx];
      if (ent > 0) {
        mode = batch::mode_of(ent & 0xff);
        cl = (ent >> 8) & 0xff;
      }
    }
    if (o.force_threads_per_row > 0) mode = batch::mode_of(o.force_threads_per_row);
    if (o.force_chunk_log2 > 0) cl = o.force_chunk_log2;
    cl = std::min(std::max(cl, 6), 24);
    p->tpr_counts[mode]++;
    const long long total = (long long)A.rows + A.nnz;
    const long long nk = (total + (1LL << cl) - 1) >> cl;
    for (long long k = 0; k < nk; ++k) work.push_back(batch::Item{i, (int)k, cl, mode});
  }
  p->n_items = (long long)work.size();
  if (p->n_items > 0) {
    e = cudaMalloc(&p->d_items, sizeof(batch::Item) * work.size());
    if (e != cudaSuccess) return bail(cuda_status(e, "batch work list"));
    e = cudaMemcpyAsync(p->d_items, work.data(), sizeof(batch::Item) * work.size(),
                        cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
      batch::split_kernel<<<(unsigned)((p->n_items + 255) / 256), 256, 0, s>>>(
          reinterpret_cast<const batch::Desc*>(p->d_descs),
          reinterpret_cast<batch::Item*>(p->d_items), p->n_items);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return bail(cuda_status(e, "batch work list"));
  }
  const int per_sm = resident_ctas_per_sm(
      dtype == EL_F32 ? (const void*)batch::batched_spmv_kernel<float>
                      : dtype == EL_BF16 ? (const void*)batch::batched_spmv_kernel<__nv_bfloat16>
                                         : (const void*)batch::batched_spmv_kernel<__half>,
      256, 0);
  long long grid = (long long)std::max(per_sm, 1) * device_info(p->device).sm_count;
  if (o.max_ctas > 0) grid = std::min<long long>(grid, o.max_ctas);
  grid = std::min<long long>(grid, std::max(p->n_items, 1LL));
  p->grid = (int)grid;

  // heavy matrices: size the plan workspace now (no allocation may happen
  // while the graph is being captured)
  for (int m : p->heavy) {
    st = workspace_prepare(p->ws, p->items[m].A, EL_SCHED_MERGE_PATH_FLAT);
    if (st != EL_OK) return bail(st);
  }

  if (p->use_graph) {
    cudaStream_t cs;
    e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(cuda_status(e, "capture stream"));
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
      cudaStreamDestroy(cs);
      return bail(cuda_status(e, "begin capture"));
    }
    st = enqueue_plan(p, cs, plan_hdr(p));
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(cs, &g);
    cudaStreamDestroy(cs);
    if (st != EL_OK) {
      if (g) cudaGraphDestroy(g);
      return bail(st);
    }
    if (e2 != cudaSuccess) return bail(cuda_status(e2, "end capture"));
    p->graph = g;
    e = cudaGraphInstantiate(&p->exec, g, 0);
    if (e != cudaSuccess) return bail(cuda_status(e, "graph instantiate"));
  }
  *out = p;
  return EL_OK;
}

el_status el_batch_plan_execute(el_batch_plan* p, el_stream_t stream) {
  if (!p) return fail(EL_ERR_NULL_POINTER, "plan is NULL");
  if (p->use_graph)
    return cuda_status(cudaGraphLaunch(p->exec, (cudaStream_t)stream), "graph launch");
  return enqueue_plan(p, (cudaStream_t)stream, plan_hdr(p));
}

el_status el_batch_plan_info(const el_batch_plan* p, int64_t* work_items,
                             int32_t* tpr_counts, int32_t* heavy) {
  if (!p) return fail(EL_ERR_NULL_POINTER, "plan is NULL");
  if (work_items) *work_items = p->n_items;
  if (tpr_counts)
    for (int i = 0; i < 7; ++i) tpr_counts[i] = p->tpr_counts[i];
  if (heavy) *heavy = (int32_t)p->heavy.size();
  return EL_OK;
}

el_status el_batch_plan_errors(el_batch_plan* p, el_stream_t stream, uint32_t* flags,
                               int clear) {
  if (!p) return fail(EL_ERR_NULL_POINTER, "plan is NULL");
  return el_workspace_errors(p->ws, stream, flags, clear);
}

el_status el_batch_plan_destroy(el_batch_plan* p) {
  if (!p) return EL_OK;
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  if (p->d_descs) cudaFree(p->d_descs);
  if (p->d_items) cudaFree(p->d_items);
  if (p->ws) el_workspace_destroy(p->ws);
  delete p;
  return EL_OK;
}

}  // extern "C"
