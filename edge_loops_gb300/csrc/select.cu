// select.cu -- schedule selection from row statistics: the predictor the
// reference's paper fits to its per-matrix timings (plots/data/heuristics.csv:
// a schedule chosen per matrix from its sizes), here a cost model of this
// library's kernels on GB300.
//
// One pass over the offsets gives the row statistics (el_csr_row_stats; the
// caller's one synchronisation), and el_select_schedule turns them into a
// schedule with a closed-form time estimate per candidate (microseconds,
// L2 cold):
//   merge_path          a + e (nnz + rows)
//   thread_mapped, T    a + c max_row + d rows + e nnz      T = 1, 4, 32 lanes
//   staged (T = 1)      the same form, where rows hold at most 27 nonzeros
//                       and consecutive rows are coherent (el_row_stats)
// The constants were fitted (non-negative least squares, relative error) to
// times of every schedule on 133 synthetic shapes -- uniform, log-normal
// (sigma 0.5, 1, 1.5) and Zipf row lengths, 64 to 4M rows, 1 to 256
// nonzeros per row, and 27-point stencils on 16^3 to 128^3 grids, the
// staged kernel's on the stencils, the shapes it applies to -- measured with
// edge_loops_gb300/tune_select.py, which refits them on other hardware.  merge_path wins on any skewed matrix and
// on every large one; thread_mapped wins on small or short regular rows,
// where the persistent merge-path launch's fixed cost (ticket, split
// search, completion counter: about 15 us with a cold L2) dominates.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "el_internal.h"

namespace el {
namespace {

// per-block max / sum / sum of squares / empty rows, combined by atomics;
// and, on every `stride`-th row r, how many of the first (up to 32) column
// pairs (col(r, j), col(r + 1, j)) step by 0, 1 or 2: the row-to-row
// coherence of a banded or stencil matrix, whose consecutive rows hold the
// same pattern shifted by one column
__global__ void row_stats_kernel(const int32_t* __restrict__ offsets,
                                 const int32_t* __restrict__ indices, long long rows,
                                 long long nnz, long long stride,
                                 unsigned long long* __restrict__ acc) {
  long long mx = 0, empty = 0;
  double sum = 0.0, sq = 0.0;
  unsigned long long pairs = 0, steps = 0;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (long long)gridDim.x * blockDim.x) {
    const long long lo = offsets[r], hi = offsets[r + 1];
    const long long len = hi - lo;
    mx = max(mx, len);
    empty += len == 0;
    sum += (double)len;
    sq += (double)len * (double)len;
    if (indices && r % stride == 0 && r + 1 < rows) {
      const long long hi2 = offsets[r + 2];
      long long m = min(len, hi2 - hi);
      m = min(m, 32LL);
      if (lo >= 0 && hi >= lo && hi2 >= hi && hi2 <= nnz) {
        for (long long j = 0; j < m; ++j) {
          const long long d = (long long)indices[hi + j] - indices[lo + j];
          steps += d >= 0 && d <= 2;
        }
        pairs += m > 0 ? (unsigned long long)m : 0ull;
      }
    }
  }
  for (int d = 16; d > 0; d >>= 1) {
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, d));
    empty += __shfl_xor_sync(0xffffffffu, empty, d);
    sum += __shfl_xor_sync(0xffffffffu, sum, d);
    sq += __shfl_xor_sync(0xffffffffu, sq, d);
    pairs += __shfl_xor_sync(0xffffffffu, pairs, d);
    steps += __shfl_xor_sync(0xffffffffu, steps, d);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(acc + 0, (unsigned long long)max(mx, 0LL));
    atomicAdd(acc + 1, (unsigned long long)empty);
    atomicAdd(reinterpret_cast<double*>(acc + 2), sum);
    atomicAdd(reinterpret_cast<double*>(acc + 3), sq);
    atomicAdd(acc + 4, pairs);
    atomicAdd(acc + 5, steps);
  }
}

struct Cost {
  double a, c, d, e;  // a + c max_row + d rows/1e3 + e nnz/1e6 (us)
};
// merge_path: a + e (nnz + rows)/1e6 (c = d = 0)
constexpr Cost kMergePath = {14.71, 0.0, 0.0, 3.541};
constexpr int kTprs[3] = {1, 4, 32};
constexpr Cost kThreadMapped[3] = {
    {7.099, 0.06098, 0.008628, 3.794},  // one lane per row (the reference's thread_mapped)
    {6.931, 0.04388, 0.0257, 2.481},
    {6.782, 0.00683, 0.1977, 1.707},    // a warp per row
};
// one lane per row, rows staged through shared memory (thread_mapped
// variant 1): a candidate where every 32-row chunk fits its buffer (rows of
// at most kStagedRows nonzeros) and consecutive rows are coherent (at least
// kStagedCoherence of the sampled column pairs step by 0..2), so that the
// row-aligned x gathers hit L1; on scattered columns the unstaged walk, with
// more warps resident, hides the gathers' latency better
constexpr Cost kStaged = {0.0, 0.305, 0.03758, 0.0};
constexpr int64_t kStagedRows = 27;
constexpr double kStagedCoherence = 0.5;

// The model: the schedule, lanes per row and kernel variant for
// thread_mapped, and the estimate.
void select_impl(int64_t rows, int64_t nnz, int64_t max_row, double coherence,
                 int32_t* schedule, int32_t* tpr_out, int32_t* variant, double* est) {
  const double R = (double)rows, N = (double)nnz, M = (double)max_row;
  double best = kMergePath.a + kMergePath.e * (N + R) / 1e6;
  int sched = EL_SCHED_MERGE_PATH_FLAT, tpr = 0, var = 0;
  for (int i = 0; i < 3; ++i) {
    const Cost& k = kThreadMapped[i];
    const double t = k.a + k.c * M + k.d * R / 1e3 + k.e * N / 1e6;
    if (t < best) {
      best = t;
      sched = EL_SCHED_THREAD_MAPPED;
      tpr = kTprs[i];
    }
  }
  if (max_row <= kStagedRows && coherence >= kStagedCoherence) {
    const double t = kStaged.a + kStaged.c * M + kStaged.d * R / 1e3 + kStaged.e * N / 1e6;
    if (t < best) {
      best = t;
      sched = EL_SCHED_THREAD_MAPPED;
      tpr = 1;
      var = 1;
    }
  }
  *schedule = sched;
  *tpr_out = tpr;
  *variant = var;
  if (est) *est = best;
}

}  // namespace
}  // namespace el

using namespace el;

extern "C" el_status el_select_schedule(int64_t rows, int64_t cols, int64_t nnz,
                                        int64_t max_row_nnz, int32_t* schedule,
                                        int32_t* threads_per_row, double* est_us) {
  if (!schedule || !threads_per_row) return fail(EL_ERR_NULL_POINTER, "output is NULL");
  if (rows < 0 || cols < 0 || nnz < 0 || max_row_nnz < 0 || max_row_nnz > nnz)
    return fail(EL_ERR_INVALID_ARGUMENT, "bad row statistics");
  int32_t variant = 0;
  select_impl(rows, nnz, max_row_nnz, 0.0, schedule, threads_per_row, &variant, est_us);
  return EL_OK;
}

extern "C" el_status el_select_schedule_stats(int64_t rows, int64_t cols, int64_t nnz,
                                              const el_row_stats* stats, int32_t* schedule,
                                              el_spmv_opts* opts, double* est_us) {
  if (!stats || !schedule || !opts) return fail(EL_ERR_NULL_POINTER, "argument is NULL");
  const int64_t mx = std::min<int64_t>(stats->max_row_nnz, nnz);
  if (rows < 0 || cols < 0 || nnz < 0 || mx < 0)
    return fail(EL_ERR_INVALID_ARGUMENT, "bad row statistics");
  int32_t tpr = 0, variant = 0;
  select_impl(rows, nnz, mx, stats->coherence, schedule, &tpr, &variant, est_us);
  if (*schedule == EL_SCHED_THREAD_MAPPED) {
    opts->threads_per_row = tpr;
    opts->variant = variant;
  }
  return EL_OK;
}

extern "C" el_status el_csr_row_stats(el_workspace* ws, const el_csr* A, el_row_stats* out,
                                      el_stream_t stream) {
  if (!A || !out) return fail(EL_ERR_NULL_POINTER, "matrix or output is NULL");
  if (A->rows < 0 || A->nnz < 0) return fail(EL_ERR_INVALID_ARGUMENT, "negative size");
  if (A->rows >= (1LL << 31)) return fail(EL_ERR_OVERFLOW, "rows exceed int32");
  *out = el_row_stats{};
  if (A->rows == 0) return EL_OK;
  if (!A->offsets) return fail(EL_ERR_NULL_POINTER, "offsets is NULL");
  cudaStream_t s = (cudaStream_t)stream;
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  el_workspace* w = nullptr;
  el_status st = workspace_resolve(ws, s, device, &w);
  if (st != EL_OK) return st;
  void* stage = nullptr;
  cudaStream_t cs = nullptr;
  cudaEvent_t ev[4];
  st = workspace_stage(w, 256, &stage, &cs, ev);
  if (st != EL_OK) return st;
  unsigned long long* acc = static_cast<unsigned long long*>(stage);
  e = cudaMemsetAsync(acc, 0, 6 * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return cuda_status(e, "el_csr_row_stats");
  const int sms = device_info(device).sm_count;
  const unsigned grid =
      (unsigned)std::max<long long>(1, std::min<long long>((A->rows + 255) / 256, sms * 4LL));
  // coherence from about 2^16 sampled rows
  const long long stride = std::max<long long>(1, A->rows >> 16);
  row_stats_kernel<<<grid, 256, 0, s>>>(A->offsets, A->nnz > 0 ? A->indices : nullptr,
                                        A->rows, A->nnz, stride, acc);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e, "el_csr_row_stats: launch");
  unsigned long long h[6];
  e = cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(e, "el_csr_row_stats: read");
  double sum, sq;
  std::memcpy(&sum, &h[2], sizeof(double));
  std::memcpy(&sq, &h[3], sizeof(double));
  out->max_row_nnz = (int64_t)h[0];
  out->empty_rows = (int64_t)h[1];
  out->mean_row_nnz = sum / (double)A->rows;
  const double var = sq / (double)A->rows - out->mean_row_nnz * out->mean_row_nnz;
  out->cv = out->mean_row_nnz > 0 ? std::sqrt(var > 0 ? var : 0.0) / out->mean_row_nnz : 0.0;
  out->coherence = h[4] > 0 ? (double)h[5] / (double)h[4] : 0.0;
  return EL_OK;
}

extern "C" el_status el_spmv_select(el_workspace* ws, const el_csr* A, int32_t* schedule,
                                    el_spmv_opts* opts, el_stream_t stream) {
  if (!A || !schedule || !opts) return fail(EL_ERR_NULL_POINTER, "argument is NULL");
  el_row_stats rs;
  el_status st = el_csr_row_stats(ws, A, &rs, stream);
  if (st != EL_OK) return st;
  return el_select_schedule_stats(A->rows, A->cols, A->nnz, &rs, schedule, opts, nullptr);
}
