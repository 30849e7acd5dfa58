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
// The constants were fitted (non-negative least squares, relative error) to
// times of every schedule on 119 synthetic shapes -- uniform, log-normal
// (sigma 0.5, 1, 1.5) and Zipf row lengths, 64 to 4M rows, 1 to 256
// nonzeros per row -- measured with edge_loops_gb300/tune_select.py, which
// refits them on other hardware.  merge_path wins on any skewed matrix and
// on every large one; thread_mapped wins on small or short regular rows,
// where the persistent merge-path launch's fixed cost (ticket, split
// search, completion counter: about 15 us with a cold L2) dominates.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "el_internal.h"

namespace el {
namespace {

// per-block max / sum / sum of squares / empty rows, combined by atomics
__global__ void row_stats_kernel(const int32_t* __restrict__ offsets, long long rows,
                                 unsigned long long* __restrict__ acc) {
  long long mx = 0, empty = 0;
  double sum = 0.0, sq = 0.0;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (long long)gridDim.x * blockDim.x) {
    const long long len = (long long)offsets[r + 1] - offsets[r];
    mx = max(mx, len);
    empty += len == 0;
    sum += (double)len;
    sq += (double)len * (double)len;
  }
  for (int d = 16; d > 0; d >>= 1) {
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, d));
    empty += __shfl_xor_sync(0xffffffffu, empty, d);
    sum += __shfl_xor_sync(0xffffffffu, sum, d);
    sq += __shfl_xor_sync(0xffffffffu, sq, d);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(acc + 0, (unsigned long long)max(mx, 0LL));
    atomicAdd(acc + 1, (unsigned long long)empty);
    atomicAdd(reinterpret_cast<double*>(acc + 2), sum);
    atomicAdd(reinterpret_cast<double*>(acc + 3), sq);
  }
}

struct Cost {
  double a, c, d, e;  // a + c max_row + d rows/1e3 + e nnz/1e6 (us)
};
// merge_path: a + e (nnz + rows)/1e6 (c = d = 0)
constexpr Cost kMergePath = {14.66, 0.0, 0.0, 3.901};
constexpr int kTprs[3] = {1, 4, 32};
constexpr Cost kThreadMapped[3] = {
    {7.034, 0.06009, 0.00394, 5.571},  // one lane per row (the reference's thread_mapped)
    {6.698, 0.04393, 0.02568, 3.156},
    {6.71, 0.007042, 0.2044, 1.804},   // a warp per row
};

}  // namespace
}  // namespace el

using namespace el;

extern "C" el_status el_select_schedule(int64_t rows, int64_t cols, int64_t nnz,
                                        int64_t max_row_nnz, int32_t* schedule,
                                        int32_t* threads_per_row, double* est_us) {
  if (!schedule || !threads_per_row) return fail(EL_ERR_NULL_POINTER, "output is NULL");
  if (rows < 0 || cols < 0 || nnz < 0 || max_row_nnz < 0 || max_row_nnz > nnz)
    return fail(EL_ERR_INVALID_ARGUMENT, "bad row statistics");
  (void)cols;
  const double R = (double)rows, N = (double)nnz, M = (double)max_row_nnz;
  double best = kMergePath.a + kMergePath.e * (N + R) / 1e6;
  int sched = EL_SCHED_MERGE_PATH_FLAT, tpr = 0;
  for (int i = 0; i < 3; ++i) {
    const Cost& k = kThreadMapped[i];
    const double t = k.a + k.c * M + k.d * R / 1e3 + k.e * N / 1e6;
    if (t < best) {
      best = t;
      sched = EL_SCHED_THREAD_MAPPED;
      tpr = kTprs[i];
    }
  }
  *schedule = sched;
  *threads_per_row = tpr;
  if (est_us) *est_us = best;
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
  e = cudaMemsetAsync(acc, 0, 4 * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return cuda_status(e, "el_csr_row_stats");
  const int sms = device_info(device).sm_count;
  const unsigned grid =
      (unsigned)std::max<long long>(1, std::min<long long>((A->rows + 255) / 256, sms * 4LL));
  row_stats_kernel<<<grid, 256, 0, s>>>(A->offsets, A->rows, acc);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e, "el_csr_row_stats: launch");
  unsigned long long h[4];
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
  return EL_OK;
}

extern "C" el_status el_spmv_select(el_workspace* ws, const el_csr* A, int32_t* schedule,
                                    el_spmv_opts* opts, el_stream_t stream) {
  if (!A || !schedule || !opts) return fail(EL_ERR_NULL_POINTER, "argument is NULL");
  el_row_stats rs;
  el_status st = el_csr_row_stats(ws, A, &rs, stream);
  if (st != EL_OK) return st;
  int32_t tpr = 0;
  st = el_select_schedule(A->rows, A->cols, A->nnz, std::min<int64_t>(rs.max_row_nnz, A->nnz),
                          schedule, &tpr, nullptr);
  if (st != EL_OK) return st;
  if (*schedule == EL_SCHED_THREAD_MAPPED) opts->threads_per_row = tpr;
  return EL_OK;
}
